"""CPU tests of the multi-frequency farming scheduler (farm.py): batching of the
shots, assembly of each frequency's solution, per-column statistics, release of
every frequency's solver, and argument errors.  The per-batch GPU solve is
replaced by a fake that records what it was given; the all-zero right-hand
side goes through the real solveLinearSystem path, which touches no device."""
import numpy as np
import pytest


def _param(hz, omega, n=(8, 8)):
    M = hz.getRegularMesh([0.0, 1.0, 0.0, 1.0], list(n))
    N = (n[0] + 1) * (n[1] + 1)
    return hz.HelmholtzParam(M, np.zeros(N), np.ones(N), omega, True, True)


def _mg(hz):
    return hz.getMGparam(complex, int, 2, 1, 50, 1e-8, "Jac", 0.8, 1, 1, "V", "Julia")


def test_farm_batches_and_assembles(hz, monkeypatch):
    from helmholtz_jl_gb300 import api, farm
    calls, cleared = [], []

    def fake_solve(_, B, S, doTranspose=0):
        calls.append((S.helmParam.omega, B.shape[1], doTranspose))
        S.last_relres = np.full(B.shape[1], 1e-9 * S.helmParam.omega)
        S.last_iters = np.full(B.shape[1], 7, dtype=np.int32)
        S.setupTime, S.solveTime = 0.5, S.solveTime + 1.0
        X = (S.helmParam.omega + 1j) * B
        return (X[:, 0] if X.shape[1] == 1 else X), S

    monkeypatch.setattr(api, "solveLinearSystem", fake_solve)
    monkeypatch.setattr(api, "clear_", lambda S: cleared.append(S.helmParam.omega))
    params = [_param(hz, w) for w in (2.0, 3.0)]
    rng = np.random.default_rng(0)
    B = rng.standard_normal((81, 7)) + 1j * rng.standard_normal((81, 7))
    res = farm.solve_frequencies(params, B, _mg(hz), batch=3, doTranspose=1)
    # 7 shots in batches of 3, 3, 1 per frequency, in order, transpose passed through
    assert calls == [(w, k, 1) for w in (2.0, 3.0) for k in (3, 3, 1)]
    for w, X, rr, it in zip((2.0, 3.0), res.X, res.relres, res.iters):
        np.testing.assert_array_equal(X, (w + 1j) * B)
        np.testing.assert_array_equal(rr, np.full(7, 1e-9 * w))
        np.testing.assert_array_equal(it, np.full(7, 7))
    assert res.solve_time == [3.0, 3.0] and res.setup_time == [0.5, 0.5]
    assert cleared == [2.0, 3.0]
    # keep=True leaves the solvers alone
    cleared.clear()
    farm.solve_frequencies(params, [B[:, :2], B[:, 2:4]], _mg(hz), batch=8, keep=True)
    assert cleared == [] and calls[-2:] == [(2.0, 2, 0), (3.0, 2, 0)]


def test_farm_zero_shots_report_zero_residuals(hz):
    """All-zero shots come back as zeros with zero residual and no iterations,
    through the library's own zero right-hand-side path (no device touched)."""
    from helmholtz_jl_gb300 import farm
    res = farm.solve_frequencies([_param(hz, 2.0)], np.zeros((81, 5), dtype=complex), _mg(hz), batch=2)
    assert not np.any(res.X[0]) and res.X[0].shape == (81, 5)
    np.testing.assert_array_equal(res.relres[0], 0.0)
    np.testing.assert_array_equal(res.iters[0], 0)


def test_zero_rhs_resets_column_stats(hz):
    """A zero right-hand side after a solve does not leave the earlier solve's
    per-column residuals on the solver."""
    S = hz.getShiftedLaplacianMultigridSolver(_param(hz, 2.0), _mg(hz), 0.5, "GMRES", 10)
    S.last_relres, S.last_iters = np.array([0.3, 0.4]), np.array([9, 9], dtype=np.int32)
    X, S = hz.solveLinearSystem(None, np.zeros((81, 3), dtype=complex), S)
    assert X.shape == (81, 3) and not np.any(X)
    np.testing.assert_array_equal(S.last_relres, np.zeros(3))
    np.testing.assert_array_equal(S.last_iters, np.zeros(3))


def test_farm_argument_errors(hz):
    from helmholtz_jl_gb300 import farm
    p = _param(hz, 2.0)
    B = np.zeros((81, 2), dtype=complex)
    with pytest.raises(ValueError):
        farm.solve_frequencies([], B, _mg(hz))
    with pytest.raises(ValueError):
        farm.solve_frequencies([p, p], [B], _mg(hz))
    with pytest.raises(ValueError):
        farm.solve_frequencies([p], B, _mg(hz), batch=0)
