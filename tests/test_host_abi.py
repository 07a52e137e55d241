"""CPU tests of the C-ABI library: it loads, exports every symbol the header
declares, its host-side discretisation helpers match the oracle, and its
compute entry points fail cleanly (no CPU fallback) where no GPU is usable."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLD = ROOT / "tests" / "golden" / "golden.npz"


def _declared_symbols():
    text = (ROOT / "include" / "helmgpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hz_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(hz):
    lib = hz._lib.load()
    syms = _declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(hz._lib.SIGNATURES), set(syms) ^ set(hz._lib.SIGNATURES)
    assert lib.hz_version() == 1


def test_struct_layouts_match_header(hz):
    L = hz._lib
    # sizes implied by the header (LP64: int32 4, int64/double/pointer 8, natural alignment)
    assert C.sizeof(L.hz_problem) == 4 + 4 + 24 + 24 + 8 + 8 + 8 + 8 + 4 + 4 + 4 + 4
    assert C.sizeof(L.hz_stats) == 4 * 4 + 8 * 3 + 8 * 3
    o = L.hz_options()
    L.load().hz_default_options(C.byref(o))
    assert (o.levels, o.inner, o.relax_pre, o.relax_post, chr(o.cycle)) == (3, 10, 1, 1, "V")
    assert o.relax_param == 0.8 and o.shift == 0.5 and o.rel_tol == 1e-8


def test_abl_matches_oracle(hz, O):
    g = np.load(GOLD)
    w = float(g["w2"])
    for neu in (0, 1):
        a = hz.getABL([17, 9], bool(neu), [3, 2], 0.9 * w).ravel(order="F")
        np.testing.assert_allclose(a, g[f"abl2_neu{neu}"], rtol=1e-15, atol=1e-15 * w)
        a3 = hz.getABL([7, 5, 9], bool(neu), [2, 2, 3], 0.9 * float(g["w3"])).ravel(order="F")
        np.testing.assert_allclose(a3, g[f"abl3_neu{neu}"], rtol=1e-14, atol=1e-14 * float(g["w3"]))
    # larger cases straight from the oracle
    for n, pad in (([129, 129], [16, 16]), ([33, 20, 17], [4, 3, 5])):
        for neu in (False, True):
            np.testing.assert_allclose(hz.getABL(n, neu, pad, 2.5), O.getABL(n, neu, pad, 2.5), rtol=1e-14,
                                       atol=1e-14)


def test_sommerfeld_mass_and_source_match_oracle(hz, O):
    g = np.load(GOLD)
    M = hz.getRegularMesh([0.0, 2.0, 0.0, 1.0], [16, 8])
    Mo = O.getRegularMesh([0.0, 2.0, 0.0, 1.0], [16, 8])
    m, w = g["m2"], float(g["w2"])
    for neu in (0, 1):
        s = hz.getSommerfeldBC(M, m, w, bool(neu)).ravel(order="F")
        np.testing.assert_allclose(s, g[f"somm2_neu{neu}"], rtol=1e-15, atol=0)
    p = hz.HelmholtzParam(M, g["gamma2"], m, w, True, True)
    mass = hz.helmholtz_mass(p)
    np.testing.assert_allclose(mass, O.helmholtz_mass(Mo, m, w, g["gamma2"], True, True), rtol=1e-14, atol=0)
    q, src = hz.getAcousticPointSource(M)
    np.testing.assert_array_equal(q.ravel(order="F"), g["q2"])
    assert src == [8, 1]
    M3 = hz.getRegularMesh([0.0, 1.5, 0.0, 1.0, 0.0, 2.0], [6, 4, 8])
    q3, src3 = hz.getAcousticPointSource(M3)
    np.testing.assert_array_equal(q3.ravel(order="F"), g["q3"])
    assert hz.loc2cs([7, 5, 9], src3) == O.loc2cs([7, 5, 9], src3)
    assert hz.getMaximalFrequency(g["m3"], M3) == pytest.approx(float(g["maxfreq_case"][0]), rel=1e-15)


def test_complex_omega_mass(hz, O):
    """GetHelmholtzOperator accepts complex omega (test/AttenuationTest.jl:46)."""
    M = hz.getRegularMesh([0.0, 1.0, 0.0, 1.0], [8, 8])
    Mo = O.getRegularMesh([0.0, 1.0, 0.0, 1.0], [8, 8])
    m = np.linspace(0.2, 0.4, 81)
    gam = np.linspace(0.0, 1.0, 81)
    w = 3.0 - 0.7j
    p = hz.HelmholtzParam(M, gam, m, w, False, True)
    np.testing.assert_allclose(hz.helmholtz_mass(p), O.helmholtz_mass(Mo, m, w, gam, False, True), rtol=1e-14)


def test_argument_errors_without_gpu_work(hz):
    L = hz._lib
    lib = L.load()
    g = np.zeros(10)
    with pytest.raises(L.HelmgpuError):
        hz.getABL([10], False, [2], 1.0)  # dim 1
    p = L.hz_problem()
    p.dim = 4
    o = L.hz_options()
    lib.hz_default_options(C.byref(o))
    h = C.c_void_p()
    assert lib.hz_create(C.byref(p), C.byref(o), C.byref(h)) == L.HZ_ERR_ARG
    assert b"dim" in lib.hz_last_error(None)
    assert not h.value
    assert lib.hz_solve(None, None, None, 0, 0, 0, 0, None) == L.HZ_ERR_ARG
    assert lib.hz_destroy(None) == 0


def test_create_reports_missing_device(hz):
    """On a machine without a GPU, hz_create refuses (there is no CPU path)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = hz._lib
    M = hz.getRegularMesh([0.0, 1.0, 0.0, 1.0], [8, 8])
    p = hz.HelmholtzParam(M, np.zeros(81), np.ones(81), 2.0, True, True)
    with pytest.raises(L.HelmgpuError) as ei:
        hz.GetHelmholtzOperator(p) @ np.ones(81)
    assert ei.value.code in (L.HZ_ERR_NO_DEVICE, L.HZ_ERR_CUDA)


def test_api_validation(hz):
    MG = hz.getMGparam(complex, int, 3, 1, 50, 1e-8, "Jac-GMRES", 0.8, 1, 1, "K", "Julia")
    assert MG.levels == 3 and MG.relaxType == "Jac-GMRES" and MG.cycleType == "K"
    M = hz.getRegularMesh([0.0, 1.0, 0.0, 1.0], [8, 8])
    p = hz.HelmholtzParam(M, np.zeros(81), np.ones(81), 2.0, True, True)
    S = hz.getShiftedLaplacianMultigridSolver(p, MG, 0.5, "GMRES", 10)
    assert np.all(S.shift == 0.5) and S.shift.size == 3
    # an option outside the built subset is refused before any device work
    MGs = hz.getMGparam(complex, int, 3, 1, 50, 1e-8, "SPAI", 0.8, 1, 1, "V", "Julia")
    Ss = hz.getShiftedLaplacianMultigridSolver(p, MGs, 0.5, "GMRES", 10)
    with pytest.raises(NotImplementedError):
        hz.solveLinearSystem(None, np.ones(81), Ss)
    # zero right-hand side: zeros, without touching the device (src/ShiftedLaplacianMultigridSolver.jl:40-43)
    MG2 = hz.getMGparam(complex, int, 3, 1, 50, 1e-8, "Jac", 0.8, 1, 1, "V", "Julia")
    S2 = hz.getShiftedLaplacianMultigridSolver(p, MG2, 0.5, "GMRES", 10)
    X, _ = hz.solveLinearSystem(None, np.zeros((81, 1), dtype=complex), S2)
    assert X.shape == (81,) and not np.any(X)
    S3 = hz.copySolver(S2)
    assert S3.MG is not S2.MG and S3.inner == 10


def _ctypes_kind(t):
    if t is None:
        return "void"
    if t is C.c_char_p:
        return "charp"
    if t is C.c_void_p or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    if t is C.c_double:
        return "double"
    return ("int", C.sizeof(t))


def _c_kind(t):
    if t in ("char*", "const char*"):
        return "charp"
    if t.endswith("*"):
        return "ptr"
    if t == "double":
        return "double"
    if t == "void":
        return "void"
    return ("int", {"int": 4, "int32_t": 4, "int64_t": 8}[t])


def test_ctypes_signatures_match_prototypes(hz):
    """Every ctypes binding has the C prototype's arity, integer widths, floating
    and pointer kinds, and return type (no silent truncation of an int64 size)."""
    import cheader
    protos = cheader.prototypes()
    for name, (res, args) in hz._lib.SIGNATURES.items():
        cres, cargs = protos[name]
        assert _ctypes_kind(res) == _c_kind(cres), (name, res, cres)
        assert [_ctypes_kind(a) for a in args] == [_c_kind(c) for c in cargs], (name, args, cargs)


def test_handles_follow_the_selected_device(hz, monkeypatch):
    """New handles (solver, operator products, networks) are built on the device the
    process selected with torch.cuda.set_device, device 0 without torch or a GPU."""
    import sys
    import types
    from helmholtz_jl_gb300 import api
    fake = types.SimpleNamespace(cuda=types.SimpleNamespace(is_available=lambda: True, current_device=lambda: 3))
    monkeypatch.setitem(sys.modules, "torch", fake)
    assert api.current_device() == 3
    assert api._default_options().device == 3
    fake.cuda.is_available = lambda: False
    assert api.current_device() == 0
    monkeypatch.delitem(sys.modules, "torch")
    assert api.current_device() == 0 and api._default_options().device == 0


def test_jac_gmres_option_checks(hz):
    """relax_type HZ_RELAX_JAC_GMRES: its argument checks run before any device
    work; valid options proceed to the device check."""
    L = hz._lib
    lib = L.load()
    m = np.ones(81)
    g = np.zeros(81)
    p = L.hz_problem()
    p.dim, p.n[0], p.n[1], p.h[0], p.h[1], p.omega_re = 2, 8, 8, 0.125, 0.125, 2.0
    p.m = m.ctypes.data_as(C.POINTER(C.c_double))
    p.gamma = g.ctypes.data_as(C.POINTER(C.c_double))
    p.order_neumann_bc = 2

    def create(**kw):
        o = L.hz_options()
        lib.hz_default_options(C.byref(o))
        o.relax_type, o.cycle = L.HZ_RELAX_JAC_GMRES, ord("K")
        for k, v in kw.items():
            setattr(o, k, v)
        h = C.c_void_p()
        st = lib.hz_create(C.byref(p), C.byref(o), C.byref(h))
        if st == L.HZ_OK:
            lib.hz_destroy(h)
        return st, (lib.hz_last_error(None) or b"").decode()

    assert create()[0] in (L.HZ_OK, L.HZ_ERR_NO_DEVICE)
    assert create(relax_from=1)[0] in (L.HZ_OK, L.HZ_ERR_NO_DEVICE)
    for bad in (dict(krylov=L.HZ_KRYLOV_BICGSTAB, cycle=ord("V")), dict(relax_pre=3), dict(relax_post=-1),
                dict(relax_from=3), dict(relax_from=-1), dict(relax_type=2)):
        assert create(**bad)[0] == L.HZ_ERR_ARG, bad
    # the Python layer maps the option
    MG = hz.getMGparam(complex, int, 3, 1, 50, 1e-8, "Jac-GMRES", 0.8, 2, 2, "K", "Julia", relaxFrom=1)
    S = hz.getShiftedLaplacianMultigridSolver(hz.HelmholtzParam(hz.getRegularMesh([0.0, 1.0, 0.0, 1.0], [8, 8]),
                                                                g, m, 2.0, True, True), MG, 0.5, "GMRES", 10)
    o = hz.api._options(S)
    assert (o.relax_type, o.relax_from, o.relax_pre) == (L.HZ_RELAX_JAC_GMRES, 1, 2)
    assert hz.copySolver(S).MG.relaxFrom == 1


@pytest.mark.parametrize("nc", [(24, 16), (8, 6, 10)])
def test_mass_with_first_order_laplacian_keeps_order_two_sommerfeld(hz, O, nc):
    """hz_helmholtz_mass for orderNeumannBC = 1: the Sommerfeld term is the BC = 2
    one of src/GetHelmholtz.jl:45, the same as for orderNeumannBC = 2."""
    import problems as PB
    P = PB.layered(nc, seed=2, pad=2, neumann=False, ellipsoid=len(nc) == 3)
    p = PB.hz_param(hz, P)
    m1 = hz.helmholtz_mass(p, 1)
    np.testing.assert_array_equal(m1, hz.helmholtz_mass(p, 2))
    ref = PB.operator_from_parts(P, 1).diagonal() - O.getNodalLaplacianMatrix(P["M"], 1).diagonal()
    np.testing.assert_allclose(m1, ref, rtol=1e-13, atol=0)


def test_3d_sommerfeld_and_mass_match_oracle(hz, O):
    """3D: the library's Sommerfeld rows (both top-face rules) against the golden
    vectors, and its mass term with the absorbing layer against the oracle."""
    g = np.load(GOLD)
    M3 = hz.getRegularMesh([0.0, 1.5, 0.0, 1.0, 0.0, 2.0], [6, 4, 8])
    Mo = O.getRegularMesh([0.0, 1.5, 0.0, 1.0, 0.0, 2.0], [6, 4, 8])
    m3, w3 = g["m3"], float(g["w3"])
    for neu in (0, 1):
        s = hz.getSommerfeldBC(M3, m3, w3, bool(neu)).ravel(order="F")
        np.testing.assert_allclose(s, g[f"somm3_neu{neu}"], rtol=1e-15, atol=0)
        np.testing.assert_array_equal(O.getSommerfeldBC(Mo, m3, w3, bool(neu)).ravel(order="F"), g[f"somm3_neu{neu}"])
    for neu, somm in ((False, True), (True, True), (True, False)):
        p = hz.HelmholtzParam(M3, g["gamma3"], m3, w3, neu, somm)
        np.testing.assert_allclose(hz.helmholtz_mass(p), O.helmholtz_mass(Mo, m3, w3, g["gamma3"], neu, somm),
                                   rtol=1e-14, atol=0)


def _header_constants():
    text = (ROOT / "include" / "helmgpu.h").read_text()
    return {k: int(v) for k, v in re.findall(r"^#define (HZ_[A-Z0-9_]+)\s+\(?(-?\d+)\)?", text, flags=re.M)}


def test_binding_constants_match_header(hz):
    """Every HZ_* value the Python and Julia bindings define is the header's."""
    consts = _header_constants()
    assert {"HZ_NET_CONV_WARP_MMA", "HZ_NET_CONV_TCGEN05", "HZ_NET_CONV_AUTO", "HZ_ERR_NO_DEVICE"} <= set(consts)
    lib = hz._lib
    py = {k: getattr(lib, k) for k in dir(lib) if re.fullmatch(r"HZ_[A-Z0-9_]+", k)}
    assert py, "the Python binding defines no HZ_* constants"
    for k, v in py.items():
        assert k in consts and consts[k] == v, (k, v, consts.get(k))
    shim = (ROOT / "helmholtz.jl_gb300" / "julia" / "HelmholtzGB300.jl").read_text()
    jl = dict(re.findall(r"^const (HZ_[A-Z0-9_]+) = Int32\((-?\d+)\)", shim, flags=re.M))
    assert jl, "the Julia shim defines no HZ_* constants"
    for k, v in jl.items():
        assert k in consts and consts[k] == int(v), (k, v, consts.get(k))
