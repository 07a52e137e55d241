"""The reference's own shifted-Laplacian example, test/ShiftedLaplacianTest.jl,
replayed through the library's API call by call: the same model, mesh, source,
multigrid parameters and solver calls (copySolver, clear!, W-cycle GMRES(20),
W-cycle BiCGSTAB, two random right-hand sides, K-cycle "Jac-GMRES" GMRES(5)).
The reference only prints each solve's relative residual; here every solve must
reach the example's tolerance, agree with the direct solve within 1e-4 (the
residual is 1e-6) and take the NumPy oracle's iteration count to within one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def example(hz, O):
    """test/ShiftedLaplacianTest.jl:14-60: v = 1.5 on 257 x 129 nodes of
    [0, 13.5] x [0, 4.2], f = 2.5, gamma = 0.01 w plus the absorbing layer (pad 16,
    amplitude getMaximalFrequency), Neumann top, Sommerfeld, shift 0.2 / 10 on every
    level; the point source 1/h1^2 at (div(n1, 2), 1); two random right-hand sides."""
    Minv = hz.getRegularMesh([0.0, 13.5, 0.0, 4.2], [256, 128])
    m = (1.0 / 1.5**2) * np.ones(257 * 129)
    w = 2 * np.pi * 2.5
    amp = hz.getMaximalFrequency(m, Minv)
    _, gamma = hz.GetHelmholtzOperator(Minv, m, w, w * np.ones(m.size) * 0.01, True, [16, 16], amp, True)
    Hparam = hz.HelmholtzParam(Minv, np.ravel(gamma, order="F"), m, w, True, True)
    Mo = O.getRegularMesh([0.0, 13.5, 0.0, 4.2], [256, 128])
    H, _ = O.GetHelmholtzOperatorABL(Mo, m, w, w * 0.01 * np.ones(m.size), True, [16, 16],
                                     O.getMaximalFrequency(m, Mo), True)
    n = Mo.n + 1
    q = np.zeros(int(np.prod(n)), dtype=complex)
    q[O.loc2cs(n, [n[0] // 2, 1]) - 1] = 1.0 / Mo.h[0] ** 2
    B2 = np.random.default_rng(0).random((q.size, 2)) + 1j * np.random.default_rng(1).random((q.size, 2))
    return dict(Hparam=Hparam, Mo=Mo, m=m, w=w, gamma=np.ravel(gamma, order="F"), H=H, q=q, B2=B2,
                shift=np.array([0.2, 0.2, 0.2]) / 10.0)


def _check(O, ex, X, B, S, krylov, cycle, restart, relax):
    """Tolerance reached, direct-solve error and the oracle's iterations."""
    H = ex["H"]
    X = X.reshape(H.shape[0], -1)
    B = B.reshape(H.shape[0], -1)
    assert np.max(S.last_relres) <= 1e-6
    for c in range(B.shape[1]):
        assert np.linalg.norm(H @ X[:, c] - B[:, c]) <= 1e-6 * 1.0001 * np.linalg.norm(B[:, c])
    Xd = O.direct_solve(H, B)
    assert np.linalg.norm(X - Xd) / np.linalg.norm(Xd) <= 1e-4
    sol = O.slmg_solve(ex["Mo"], ex["m"], ex["gamma"], ex["w"], True, True, B, levels=2, shift=0.02, relax_w=0.75,
                       pre=2, post=2, restart=max(restart, 1), tol=1e-6, max_outer=30, cycle=cycle, krylov=krylov,
                       relax_type=relax)
    assert np.all(np.abs(np.asarray(S.last_iters) - sol.result.iters) <= 1), (S.last_iters, sol.result.iters)


def test_shifted_laplacian_example_sequence(hz, O, example):
    ex = example
    Hparam, shift, q = ex["Hparam"], ex["shift"], ex["q"]
    # :49-84  levels 2, maxIter 30, tol 1e-6, "Jac" 0.75 with 2/2 sweeps, 'W', "NoMUMPS"; GMRES(20), copySolver
    MG = hz.getMGparam(complex, int, 2, 2, 30, 1e-6, "Jac", 0.75, 2, 2, "W", "NoMUMPS", 0.5, 0.0)
    Ainv = hz.getShiftedLaplacianMultigridSolver(Hparam, MG, shift, "GMRES", 20, True)
    Ainv = hz.copySolver(Ainv)
    b = q.copy()
    x, Ainv = hz.solveLinearSystem(None, b, Ainv)
    assert x.shape == b.shape
    _check(O, ex, x, b, Ainv, "GMRES", "W", 20, "Jac")
    # :86-89  the same parameters with BiCGSTAB
    MG.relaxType = "Jac"
    MG.cycleType = "W"
    Ainv = hz.getShiftedLaplacianMultigridSolver(Hparam, MG, shift, "BiCGSTAB", 0, True)
    x, Ainv = hz.solveLinearSystem(None, b, Ainv)
    _check(O, ex, x, b, Ainv, "BiCGSTAB", "W", 0, "Jac")
    # :121-132  coarse solve "Julia", two random right-hand sides, clear! before the solve
    MG = hz.getMGparam(complex, int, 2, 2, 30, 1e-6, "Jac", 0.75, 2, 2, "W", "Julia", 0.5, 0.0)
    Ainv = hz.getShiftedLaplacianMultigridSolver(Hparam, MG, shift, "BiCGSTAB", 0, True)
    B = ex["B2"]
    hz.clear_(Ainv)
    Ainv.helmParam = Hparam
    x, Ainv = hz.solveLinearSystem(None, B, Ainv)
    assert x.shape == B.shape
    _check(O, ex, x, B, Ainv, "BiCGSTAB", "W", 0, "Jac")
    # :134-139  relaxType "Jac-GMRES", the K-cycle, GMRES(5)
    MG = hz.getMGparam(complex, int, 2, 2, 30, 1e-6, "Jac", 0.75, 2, 2, "W", "Julia")
    MG.relaxType = "Jac-GMRES"
    MG.cycleType = "K"
    Ainv = hz.getShiftedLaplacianMultigridSolver(Hparam, MG, shift, "GMRES", 5, True)
    x, Ainv = hz.solveLinearSystem(None, B, Ainv)
    _check(O, ex, x, B, Ainv, "GMRES", "K", 5, "Jac-GMRES")
