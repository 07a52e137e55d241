"""CPU tests of the host-side operator algebra (api.HelmholtzOperator,
GetHelmholtzShiftOP, getHelmholtzFun, src/GetHelmholtz.jl:81-95).  The device
handle is replaced by a fake that applies the oracle's sparse H or
SH(s) = H + i s w^2 diag(m) (or their adjoints), so every composition is held to
the matrix it stands for: which handle shift, which operator and which adjoint
flag a product selects."""
import numpy as np
import pytest


@pytest.fixture()
def fake_devices(hz, O, monkeypatch):
    from helmholtz_jl_gb300 import api
    made = []

    class FakeDevice:
        def __init__(self, param, shift, orderNeumannBC=2, opts=None):
            Mo = O.getRegularMesh(param.Mesh.domain, param.Mesh.n)
            self.H = O.GetHelmholtzOperator(Mo, param.m, param.omega, param.gamma, param.NeumannOnTop,
                                            param.Sommerfeld).tocsr()
            self.S = O.GetHelmholtzShiftOP(param.m, float(np.real(param.omega)), shift)
            self.shift = shift
            made.append(shift)

        def apply(self, op, adj, X):
            A = self.H if op == hz._lib.HZ_OP_H else (self.H + self.S)
            A = A.conj().T if adj else A
            return A @ X

    monkeypatch.setattr(api, "_Device", FakeDevice)
    return made


def _problem(hz, O):
    M = hz.getRegularMesh([0.0, 1.0, 0.0, 0.5], [8, 4])
    rng = np.random.default_rng(1)
    m = rng.uniform(0.2, 0.5, size=45)
    gamma = rng.uniform(0.0, 1.0, size=45)
    w = 7.0
    p = hz.HelmholtzParam(M, gamma, m, w, True, True)
    Ho = O.GetHelmholtzOperator(O.getRegularMesh([0.0, 1.0, 0.0, 0.5], [8, 4]), m, w, gamma, True, True).tocsr()
    return p, Ho, m, w


def test_products_match_the_matrices_they_stand_for(hz, O, fake_devices):
    p, Ho, m, w = _problem(hz, O)
    H = hz.GetHelmholtzOperator(p)
    Sh = hz.GetHelmholtzShiftOP(m, w, 0.5)
    D = lambda s: 1j * s * w**2 * np.diag(m)  # noqa: E731
    Hd = Ho.toarray()
    x = np.random.default_rng(2).standard_normal((45, 3)) + 0j
    cases = {
        "H": (H, Hd),
        "H^H": (H.H, Hd.conj().T),
        "SH": (H + Sh, Hd + D(0.5)),
        "SH^H": ((H + Sh).H, (Hd + D(0.5)).conj().T),
        "Sh + H": (Sh + H, Hd + D(0.5)),
        "H^H + Sh": (H.H + Sh, Hd.conj().T + D(0.5)),
        "SH - Sh": ((H + Sh) + (-Sh), Hd),
        "H + 0.2 + 0.3": (H + hz.GetHelmholtzShiftOP(m, w, 0.2) + hz.GetHelmholtzShiftOP(m, w, 0.3), Hd + D(0.5)),
    }
    for name, (op, A) in cases.items():
        np.testing.assert_allclose(op @ x, A @ x, rtol=1e-13, atol=0, err_msg=name)
        np.testing.assert_allclose(op @ x[:, 0], A @ x[:, 0], rtol=1e-13, atol=0, err_msg=name)
    # one handle per distinct shift: H products reuse whichever exists
    assert sorted(set(fake_devices)) == [-0.5, 0.5]


def test_helmholtz_fun_evaluates_h_and_its_adjoint(hz, O, fake_devices):
    """getHelmholtzFun(SH', Shift) is H (src/GetHelmholtz.jl:85-95); with (SH, -Shift) it is H^H."""
    p, Ho, m, w = _problem(hz, O)
    SH = hz.GetHelmholtzOperator(p) + hz.GetHelmholtzShiftOP(m, w, 0.5)
    Sh = hz.GetHelmholtzShiftOP(m, w, 0.5)
    x = np.random.default_rng(3).standard_normal(45) + 1j * np.random.default_rng(4).standard_normal(45)
    np.testing.assert_allclose(hz.getHelmholtzFun(SH.H, Sh)(x), Ho @ x, rtol=1e-13)
    np.testing.assert_allclose(hz.getHelmholtzFun(SH, -Sh)(x), Ho.conj().T @ x, rtol=1e-13)


def test_algebra_rejections(hz, O, fake_devices):
    p, Ho, m, w = _problem(hz, O)
    H = hz.GetHelmholtzOperator(p)
    Sh = hz.GetHelmholtzShiftOP(m, w, 0.5)
    with pytest.raises(ValueError):
        H + H                                    # noqa: B018 - the sum of two operators is not built
    with pytest.raises(ValueError):
        -H                                       # noqa: B018
    with pytest.raises(ValueError):
        H + hz.GetHelmholtzShiftOP(m * 2, w, 0.5)  # another m
    with pytest.raises(TypeError):
        Sh @ np.ones(45)
    with pytest.raises(ValueError):
        hz.getHelmholtzFun(H, H)
    np.testing.assert_allclose(Sh.diagonal_shift(), 1j * 0.5 * w**2 * m)
    assert fake_devices == []                    # nothing above reached a device
