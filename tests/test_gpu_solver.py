"""GPU parity of the full shifted-Laplacian multigrid FGMRES solve
(src/ShiftedLaplacianMultigridSolver.jl:33-102) against the oracle:
the plain FP64 form to relative error <= 1e-6 at residual 1e-8, the mixed
form to <= 1e-4 at residual 1e-6 (bounds of the solver's specification);
iteration counts of the FP64 form equal the C oracle's."""
import numpy as np
import pytest

import problems as PB

pytestmark = pytest.mark.gpu


def _solver(hz, P, levels, tol, precision="fp64", cycle="V", inner=10, max_outer=60, pre=1, post=1):
    MG = hz.getMGparam(complex, int, levels, 1, max_outer, tol, "Jac", 0.8, pre, post, cycle, "Julia", 0.5, 0.0,
                       precision=precision)
    return hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "GMRES", inner)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_config1_point_source_fp64(hz, O):
    """129x129 gradient+ellipse model, source at (0.5, 2h), 3 levels V(1,1), FGMRES(10), tol 1e-8."""
    P = PB.gradient_2d((128, 128), pad=16)
    M = PB.hz_param(hz, P).Mesh
    q, src = hz.getAcousticPointSource(M, np.complex128, [65, 3])
    q = q.ravel(order="F")
    S = _solver(hz, P, 3, 1e-8)
    X, S = hz.solveLinearSystem(None, q, S)
    assert X.shape == q.shape
    Xref = O.direct_solve(P["H"], q)
    assert _rel(X, Xref) <= 1e-6
    assert np.linalg.norm(P["H"] @ X - q) / np.linalg.norm(q) <= 1e-8
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, q, levels=3, tol=1e-8, max_outer=60)
    assert int(S.last_iters[0]) == int(sol.result.iters[0])
    assert S.setupTime > 0 and S.solveTime > 0 and S.nPrec >= 1


@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-8, 1e-6), ("mixed", 1e-6, 1e-4)])
def test_multi_rhs_2d(hz, O, cpu_slmg, precision, tol, bound):
    P = PB.layered((128, 64), seed=3, pad=8, lengths=[2.0, 1.0])
    n = P["m"].size
    B = PB.rhs(n, 6, seed=2)
    B[:, 4] = 0.0  # zero column -> zero solution
    S = _solver(hz, P, 4, tol, precision)
    X, S = hz.solveLinearSystem(None, B, S)
    Xref = O.direct_solve(P["H"], B)
    for c in range(6):
        if c == 4:
            assert not np.any(X[:, 4])
            continue
        assert _rel(X[:, c], Xref[:, c]) <= bound, c
        assert np.linalg.norm(P["H"] @ X[:, c] - B[:, c]) / np.linalg.norm(B[:, c]) <= tol * 1.0001
    if precision == "fp64":
        SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
        r = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 4).solve(B, tol=tol, max_outer=60)
        np.testing.assert_array_equal(S.last_iters, r.iters)


@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-8, 1e-6), ("mixed", 1e-6, 1e-4)])
def test_3d_layered_ellipsoid(hz, O, precision, tol, bound):
    P = PB.layered((32, 32, 32), seed=6, pad=4, ellipsoid=True)
    n = P["m"].size
    B = PB.rhs(n, 3, seed=4)
    S = _solver(hz, P, 3, tol, precision)
    X, S = hz.solveLinearSystem(None, B, S)
    Xref = O.direct_solve(P["H"], B)
    assert _rel(X, Xref) <= bound
    assert np.max(S.last_relres) <= tol


def test_transpose_solve(hz, O):
    P = PB.gradient_2d((64, 64), pad=8)
    n = P["m"].size
    B = PB.rhs(n, 2, seed=8)
    S = _solver(hz, P, 3, 1e-8)
    X, S = hz.solveLinearSystem(None, B, S, 1)
    Xref = O.direct_solve(P["H"].conj().T.tocsr(), B)
    assert _rel(X, Xref) <= 1e-6
    X0, S = hz.solveLinearSystem(None, B, S, 0)  # and back: both hierarchies kept
    assert _rel(X0, O.direct_solve(P["H"], B)) <= 1e-6


def test_w_cycle_and_more_sweeps(hz, O, cpu_slmg):
    P = PB.gradient_2d((64, 64), pad=8)
    n = P["m"].size
    B = PB.rhs(n, 2, seed=12)
    S = _solver(hz, P, 3, 1e-8, cycle="W", pre=2, post=2)
    X, S = hz.solveLinearSystem(None, B, S)
    assert _rel(X, O.direct_solve(P["H"], B)) <= 1e-6
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    r = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 3).solve(B, tol=1e-8, max_outer=60, cycle="W", pre=2, post=2)
    np.testing.assert_array_equal(S.last_iters, r.iters)


def test_device_arrays_and_inplace(hz, O):
    import torch
    P = PB.gradient_2d((64, 32), pad=6)
    n = P["m"].size
    B = PB.rhs(n, 3, seed=21)
    S = _solver(hz, P, 3, 1e-8)
    Xh, S = hz.solveLinearSystem(None, B, S)
    Xd, S = hz.solveLinearSystem(None, torch.from_numpy(B).to("cuda"), S)
    np.testing.assert_allclose(Xd.cpu().numpy(), Xh, rtol=0, atol=1e-14 * np.abs(Xh).max())
    Xi = np.zeros_like(B)
    hz.solveLinearSystemInPlace(None, B, Xi, S)
    np.testing.assert_array_equal(Xi, Xh)


def test_single_level_and_restart_lengths(hz, O):
    P = PB.gradient_2d((32, 32), pad=4)
    n = P["m"].size
    B = PB.rhs(n, 2, seed=5)
    Xref = O.direct_solve(P["H"], B)
    for levels, inner in ((1, 5), (2, 20), (3, 17)):
        S = _solver(hz, P, levels, 1e-9, inner=inner)
        X, S = hz.solveLinearSystem(None, B, S)
        assert _rel(X, Xref) <= 1e-6, (levels, inner)


def test_not_converged_is_a_warning(hz, O, capsys):
    P = PB.gradient_2d((64, 64), pad=8)
    n = P["m"].size
    B = PB.rhs(n, 1, seed=3)
    S = _solver(hz, P, 3, 1e-12, max_outer=1, inner=3)
    X, S = hz.solveLinearSystem(None, B, S)
    assert "WARNING" in capsys.readouterr().out
    assert np.all(np.isfinite(X))
    assert S.last_relres[0] > 1e-12


def test_nan_rhs_is_an_error(hz):
    P = PB.gradient_2d((32, 32), pad=4)
    n = P["m"].size
    B = PB.rhs(n, 2, seed=5)
    B[3, 1] = np.nan
    S = _solver(hz, P, 2, 1e-8)
    with pytest.raises(hz._lib.HelmgpuError) as ei:
        hz.solveLinearSystem(None, B, S)
    assert ei.value.code == hz._lib.HZ_ERR_NUMERIC
    # the handle stays usable
    B[3, 1] = 0.0
    X, S = hz.solveLinearSystem(None, B, S)
    assert np.all(np.isfinite(X))


def test_clear_and_copy(hz, O):
    P = PB.gradient_2d((32, 32), pad=4)
    n = P["m"].size
    B = PB.rhs(n, 1, seed=5)[:, 0]
    S = _solver(hz, P, 3, 1e-8)
    X1, S = hz.solveLinearSystem(None, B, S)
    hz.clear_(S)
    X2, S = hz.solveLinearSystem(None, B, S)
    np.testing.assert_array_equal(X1, X2)
    S2 = hz.copySolver(S)
    X3, S2 = hz.solveLinearSystem(None, B, S2)
    np.testing.assert_array_equal(X1, X3)


def _bicg_solver(hz, P, levels, tol, precision="fp64", max_iter=400):
    MG = hz.getMGparam(complex, int, levels, 1, max_iter, tol, "Jac", 0.8, 1, 1, "V", "Julia", 0.5, 0.0,
                       precision=precision)
    return hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "BiCGSTAB", 0)


@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-8, 1e-6), ("mixed", 1e-6, 1e-4)])
def test_bicgstab_2d(hz, O, precision, tol, bound):
    """solveBiCGSTAB_MG path (src/ShiftedLaplacianMultigridSolver.jl:91-93, the reference's default Krylov)."""
    P = PB.gradient_2d((64, 64), pad=8)
    n = P["m"].size
    B = PB.rhs(n, 4, seed=3)
    B[:, 2] = 0.0
    S = _bicg_solver(hz, P, 3, tol, precision)
    X, S = hz.solveLinearSystem(None, B, S)
    Xref = O.direct_solve(P["H"], B)
    assert not np.any(X[:, 2])
    for c in (0, 1, 3):
        assert _rel(X[:, c], Xref[:, c]) <= bound
    assert np.max(S.last_relres) <= tol
    if precision == "fp64":
        sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=3, tol=tol, max_outer=400,
                           krylov="BiCGSTAB")
        # same algorithm in FP64: iteration counts agree up to rounding of the stopping test
        assert np.all(np.abs(S.last_iters.astype(int) - sol.result.iters.astype(int)) <= 1)


def test_bicgstab_3d_transpose(hz, O):
    P = PB.layered((24, 24, 24), seed=9, pad=3, ellipsoid=True)
    n = P["m"].size
    B = PB.rhs(n, 2, seed=4)
    S = _bicg_solver(hz, P, 3, 1e-8)
    X, S = hz.solveLinearSystem(None, B, S, 1)
    Xref = O.direct_solve(P["H"].conj().T.tocsr(), B)
    assert _rel(X, Xref) <= 1e-6


@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-8, 1e-6), ("mixed", 1e-6, 1e-4)])
def test_rediscretized_coarse_levels(hz, O, precision, tol, bound):
    """The re-discretised hierarchy (src/ShiftedLaplacianMultigridSolver.jl:51-62)."""
    P = PB.gradient_2d((64, 64), pad=8)
    n = P["m"].size
    B = PB.rhs(n, 3, seed=13)
    MG = hz.getMGparam(complex, int, 3, 1, 100, tol, "Jac", 0.8, 1, 1, "V", "Julia", 0.5, 0.0, precision=precision,
                       coarseOperator="Rediscretize")
    S = hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "GMRES", 10)
    X, S = hz.solveLinearSystem(None, B, S)
    assert _rel(X, O.direct_solve(P["H"], B)) <= bound
    if precision == "fp64":
        sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=3, tol=tol, max_outer=100,
                           coarse="rediscretize")
        assert np.all(np.abs(S.last_iters.astype(int) - sol.result.iters.astype(int)) <= 1)
        Xt, S = hz.solveLinearSystem(None, B, S, 1)
        assert _rel(Xt, O.direct_solve(P["H"].conj().T.tocsr(), B)) <= bound


def test_rediscretized_3d(hz, O):
    P = PB.layered((32, 32, 32), seed=6, pad=4, ellipsoid=True)
    B = PB.rhs(P["m"].size, 2, seed=4)
    MG = hz.getMGparam(complex, int, 3, 1, 100, 1e-8, "Jac", 0.8, 1, 1, "V", "Julia", coarseOperator="Rediscretize")
    S = hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "GMRES", 10)
    X, S = hz.solveLinearSystem(None, B, S)
    assert _rel(X, O.direct_solve(P["H"], B)) <= 1e-6


def test_multi_frequency_farming(hz, O):
    """Several frequencies x shots in batches: one hierarchy per frequency, reused across batches."""
    from helmholtz_jl_gb300.farm import solve_frequencies
    P = PB.gradient_2d((64, 32), pad=6)
    Mo = P["M"]
    M = hz.getRegularMesh(Mo.domain, Mo.n)
    n = P["m"].size
    B = PB.rhs(n, 5, seed=17)
    params, refs = [], []
    for scale in (0.6, 1.0):
        w = P["w"] * scale
        gam = hz.getABL(Mo.n + 1, True, [6, 6], 0.95 * w).ravel(order="F") + 0.01 * w
        params.append(hz.HelmholtzParam(M, gam, P["m"], w, True, True))
        refs.append(O.GetHelmholtzOperator(Mo, P["m"], w, gam, True, True))
    MG = hz.getMGparam(complex, int, 3, 1, 100, 1e-8, "Jac", 0.8, 1, 1, "V", "Julia")
    res = solve_frequencies(params, B, MG, batch=2)
    for k in range(2):
        Xref = O.direct_solve(refs[k], B)
        assert _rel(res.X[k], Xref) <= 1e-6
        assert np.all(res.relres[k] <= 1e-8) and np.all(res.iters[k] > 0)


@pytest.mark.parametrize("case", ["2d", "3d", "2d_transpose"])
def test_emulated_fp64_outer_matches_native(hz, O, case):
    """Mixed form with the outer FGMRES in FP64 emulated by FP32 pairs: same
    accuracy bound as the native-FP64 mixed form and about the same iterations."""
    if case == "3d":
        P = PB.layered((32, 32, 32), seed=6, pad=4, ellipsoid=True)
    else:
        P = PB.layered((128, 64), seed=3, pad=8, lengths=[2.0, 1.0])
    tr = 1 if case == "2d_transpose" else 0
    B = PB.rhs(P["m"].size, 4, seed=23)
    B[:, 1] = 0.0
    its = {}
    for arith in ("fp64", "emulated"):
        MG = hz.getMGparam(complex, int, 3, 1, 60, 1e-6, "Jac", 0.8, 1, 1, "V", "Julia", precision="mixed",
                           outerArithmetic=arith)
        S = hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "GMRES", 10)
        X, S = hz.solveLinearSystem(None, B, S, tr)
        Href = P["H"].conj().T.tocsr() if tr else P["H"]
        Xref = O.direct_solve(Href, B)
        assert not np.any(X[:, 1])
        for c in (0, 2, 3):
            assert _rel(X[:, c], Xref[:, c]) <= 1e-4
            assert np.linalg.norm(Href @ X[:, c] - B[:, c]) / np.linalg.norm(B[:, c]) <= 1e-6 * 1.0001
        its[arith] = S.last_iters.astype(int)
    assert np.all(np.abs(its["emulated"] - its["fp64"]) <= 2), its


@pytest.fixture(scope="module")
def full_2d(O):
    """configs[1] at its full size: 1025 x 513 nodes (cells of 10 m), a seeded layered
    model with an absorbing layer of 32 cells; four random right-hand sides and their
    direct solution (SciPy SuperLU of the oracle's operator)."""
    P = PB.layered((1024, 512), seed=7, pad=32, lengths=[10.24, 5.12])
    B = PB.rhs(P["m"].size, 4, seed=5)
    return P, B, O.direct_solve(P["H"], B)


@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-8, 1e-6), ("mixed", 1e-6, 1e-4)])
def test_full_size_2d_against_direct_solve(hz, full_2d, precision, tol, bound):
    """Five Galerkin levels, the K-cycle with damped Jacobi, FGMRES(10): every column to
    the tolerance and within the specification's error bound of the direct solve."""
    P, B, Xref = full_2d
    S = _solver(hz, P, 5, tol, precision, cycle="K")
    X, S = hz.solveLinearSystem(None, B, S)
    assert S.last_relres.max() <= tol
    for c in range(B.shape[1]):
        assert _rel(X[:, c], Xref[:, c]) <= bound, (c, _rel(X[:, c], Xref[:, c]))
        assert np.linalg.norm(P["H"] @ X[:, c] - B[:, c]) / np.linalg.norm(B[:, c]) <= tol * 1.0001


@pytest.fixture(scope="module")
def full_3d(O, cpu_slmg):
    """configs[2] at its full size: 129^3 nodes (cells of 10 m), a seeded layered model
    with an ellipsoidal body, an absorbing layer of 12 cells and 16 point sources on a
    4 x 4 grid of the surface (depth index 1).  The FP64 reference for column 0 is the C
    oracle's plain FP64 solve (the same 4-level V(1,1) cycle) continued to relative
    residual 1e-9; its iteration count to 1e-6 is kept for the FP64 form."""
    P = PB.layered((128, 128, 128), seed=11, pad=12, ellipsoid=True, lengths=[1.28] * 3)
    nn = P["M"].n + 1
    B = np.zeros((P["m"].size, 16), dtype=np.complex128, order="F")
    grid = np.linspace(0.2 * nn[0], 0.8 * nn[0], 4).astype(np.int64)
    amp = 1.0 / float(np.linalg.norm(P["M"].h)) ** 2
    for c in range(16):
        B[int(grid[c % 4]) + nn[0] * (int(grid[c // 4]) + nn[1] * 1), c] = amp
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    cpu = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 4)
    r6 = cpu.solve(B[:, :1], tol=1e-6, max_outer=80)
    r9 = cpu.solve(B[:, :1], tol=1e-9, max_outer=80, X0=r6.X)
    assert r9.relres[0] <= 1e-9
    return P, B, int(r6.iters[0]), r9.X[:, 0]


def test_full_size_3d_against_oracle(hz, full_3d):
    """The mixed form on all 16 columns and the plain FP64 form on two, four Galerkin
    levels, V(1,1) damped Jacobi, FGMRES(10) to 1e-6: every column to the tolerance, the
    error of column 0 within the specification's bound of the oracle's solution, and the
    FP64 form's iterations within 2 % (at least 2) of the oracle's."""
    P, B, it_ref, xref = full_3d
    H = P["H"]
    for precision, cols in (("mixed", 16), ("fp64", 2)):
        S = _solver(hz, P, 4, 1e-6, precision, max_outer=80)
        X, S = hz.solveLinearSystem(None, np.asfortranarray(B[:, :cols]), S)
        assert S.last_relres.max() <= 1e-6, precision
        for c in range(cols):
            assert np.linalg.norm(H @ X[:, c] - B[:, c]) / np.linalg.norm(B[:, c]) <= 1e-6 * 1.0001, (precision, c)
        assert _rel(X[:, 0], xref) <= 1e-4, (precision, _rel(X[:, 0], xref))
        if precision == "fp64":
            assert abs(int(S.last_iters[0]) - it_ref) <= max(2, 0.02 * it_ref), (S.last_iters, it_ref)
