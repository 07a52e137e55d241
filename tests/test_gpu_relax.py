"""GPU parity of the "Jac-GMRES" smoother (Multigrid.jl relaxType of
test/ShiftedLaplacianTest.jl:138): one or two GMRES steps per smoothing,
right-preconditioned by a damped-Jacobi sweep, on every level or from a coarse
level down.  Plain FP64: solution within 1e-6 of the direct solve at residual
1e-8 and iteration counts within one of the NumPy oracle's; mixed form within
1e-4 at residual 1e-6; CUDA-graph replays identical to eager launches."""
import numpy as np
import pytest

import problems as PB

pytestmark = pytest.mark.gpu


def _solver(hz, P, levels, tol, cycle="K", pre=1, post=1, relax_from=0, precision="fp64", outer="fp64",
            graph=True):
    MG = hz.getMGparam(complex, int, levels, 1, 60, tol, "Jac-GMRES", 0.8, pre, post, cycle, "Julia", 0.5, 0.0,
                       precision=precision, outerArithmetic=outer, relaxFrom=relax_from)
    MG.cudaGraph = graph
    return hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "GMRES", 10)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("cycle,pre,post,relax_from", [("V", 1, 1, 0), ("V", 2, 2, 0), ("K", 1, 1, 1),
                                                       ("K", 2, 1, 0), ("W", 2, 2, 1)])
def test_jac_gmres_fp64_matches_oracle(hz, O, cycle, pre, post, relax_from):
    P = PB.layered((64, 64), seed=3, pad=8)
    B = PB.rhs(P["m"].size, 3, seed=1)
    S = _solver(hz, P, 4, 1e-8, cycle=cycle, pre=pre, post=post, relax_from=relax_from)
    X, S = hz.solveLinearSystem(None, B, S)
    Xref = O.direct_solve(P["H"], B)
    for c in range(3):
        assert _rel(X[:, c], Xref[:, c]) <= 1e-6
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=4, tol=1e-8, max_outer=60,
                       cycle=cycle, pre=pre, post=post, relax_type="Jac-GMRES", gmres_from=relax_from)
    assert np.all(np.abs(S.last_iters - sol.result.iters) <= 1), (S.last_iters, sol.result.iters)


@pytest.mark.parametrize("outer", ["fp64", "emulated"])
def test_jac_gmres_mixed_deep_3d(hz, O, outer):
    """3D 33^3, four Galerkin levels, K-cycle with GMRES smoothing below the fine
    level: the mixed form to 1e-6, the adjoint solve too."""
    P = PB.layered((32, 32, 32), seed=7, pad=4, ellipsoid=True)
    B = PB.rhs(P["m"].size, 2, seed=2)
    S = _solver(hz, P, 4, 1e-6, relax_from=1, precision="mixed", outer=outer)
    X, S = hz.solveLinearSystem(None, B, S)
    Xref = O.direct_solve(P["H"], B)
    for c in range(2):
        assert _rel(X[:, c], Xref[:, c]) <= 1e-4
    assert S.last_relres.max() <= 1e-6
    Xa, S = hz.solveLinearSystem(None, B, S, 1)
    HH = P["H"].conj().T.tocsr()
    for c in range(2):
        assert np.linalg.norm(HH @ Xa[:, c] - B[:, c]) / np.linalg.norm(B[:, c]) <= 1e-6 * 1.0001


def test_jac_gmres_graph_replay_matches_eager(hz):
    P = PB.layered((64, 64), seed=4, pad=8)
    B = PB.rhs(P["m"].size, 3, seed=3)
    Xs = []
    for graph in (False, True):
        S = _solver(hz, P, 4, 1e-8, cycle="K", pre=2, post=2, relax_from=1, graph=graph)
        X, S = hz.solveLinearSystem(None, B, S)
        Xs.append((X, S.last_iters.copy()))
    np.testing.assert_array_equal(Xs[0][1], Xs[1][1])
    np.testing.assert_array_equal(Xs[0][0], Xs[1][0])
