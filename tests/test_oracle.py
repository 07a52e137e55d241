"""CPU tests of the oracle: pinned by the reference's own known-answer test,
checked against the committed golden vectors, and cross-checked between the
NumPy and the C restatements."""
from pathlib import Path

import numpy as np
import pytest

import problems as PB

GOLD = Path(__file__).resolve().parent / "golden" / "golden.npz"


def _fictitious_source(O, u, mfun, w, rhs, refinements=4):
    """test/testFictitiousSource2D.jl:10-70 restated: manufactured solution on
    [-1,1]^2 starting from 32x48 cells, absorbing layer getABL(n+1, true, 5, 0.1),
    no Sommerfeld; energy error |V (u_h - u)^H A (u_h - u)| per refinement."""
    n = np.array([32, 48])
    errs = []
    for _ in range(refinements):
        n = n * 2
        M = O.getRegularMesh([-1.0, 1.0, -1.0, 1.0], n)
        xn = O.getNodalGrid(M)
        gamma = O.getABL(M.n + 1, True, [5, 5], 0.1).ravel(order="F")
        uk = u(xn[:, 0], xn[:, 1])
        mk = mfun(xn[:, 0], xn[:, 1])
        rk = rhs(xn[:, 0], xn[:, 1]) + 1j * w**2 * gamma * mk * uk
        A = O.GetHelmholtzOperator(M, mk, w, gamma, True, False)
        ut = O.direct_solve(A, -rk)
        e = ut - uk
        errs.append(abs(M.h[0] * M.h[1] * np.vdot(e, A @ e)))
    return np.array(errs)


@pytest.mark.parametrize("model", ["constant", "gaussian"])
def test_oracle_manufactured_solution_second_order(O, model):
    w = 2 * np.pi
    u = lambda x, y: np.cos(np.pi * x) * np.cos(np.pi * y)  # noqa: E731
    if model == "constant":
        mfun = lambda x, y: np.ones_like(x)  # noqa: E731
    else:
        mfun = lambda x, y: np.exp(-2.0 * (x**2 + y**2))  # noqa: E731
    rhs = lambda x, y: -2 * np.pi**2 * u(x, y) + mfun(x, y) * u(x, y) * w**2  # noqa: E731
    errs = _fictitious_source(O, u, mfun, w, rhs)
    factors = errs[:-1] / errs[1:]
    assert np.all(factors > 1.5), factors
    # energy error converges at second order: factor -> 4 per halving of h
    assert factors[-1] > 3.4, factors


def test_oracle_matches_golden(O):
    g = np.load(GOLD)
    M = O.getRegularMesh([0.0, 2.0, 0.0, 1.0], [16, 8])
    nn = M.n + 1
    m, w = g["m2"], float(g["w2"])
    for neu in (0, 1):
        np.testing.assert_array_equal(O.getABL(nn, bool(neu), [3, 2], 0.9 * w).ravel(order="F"), g[f"abl2_neu{neu}"])
        np.testing.assert_array_equal(O.getSommerfeldBC(M, m, w, bool(neu)).ravel(order="F"), g[f"somm2_neu{neu}"])
    H, gam = O.GetHelmholtzOperatorABL(M, m, w, 0.01 * w * np.ones(m.size), True, [3, 2], 0.9 * w, True)
    np.testing.assert_array_equal(np.ravel(gam, order="F"), g["gamma2"])
    np.testing.assert_allclose(H @ g["X2"], g["HX2"], rtol=0, atol=1e-12 * np.abs(g["HX2"]).max())
    H1 = O.GetHelmholtzOperator(M, m, w, gam, True, True, 1)
    np.testing.assert_allclose(H1 @ g["X2"], g["HX2_bc1"], rtol=0, atol=1e-12 * np.abs(g["HX2_bc1"]).max())
    M3 = O.getRegularMesh([0.0, 1.5, 0.0, 1.0, 0.0, 2.0], [6, 4, 8])
    for neu in (0, 1):
        np.testing.assert_array_equal(O.getABL(M3.n + 1, bool(neu), [2, 2, 3], 0.9 * float(g["w3"])).ravel(order="F"),
                                      g[f"abl3_neu{neu}"])


def _attenuated_point_source(O, nn, pad, src0, complex_omega):
    """test/AttenuationTest.jl restated: unit slowness on [0,10]^2 with nn x nn nodes,
    f = 2.5 (w = 5 pi), attenuation alpha = pi, absorbing layer getABL(n, false,
    [pad, pad], getMaximalFrequency), no Sommerfeld, q = 1/h^2 at node src0 (0-based).
    Either the attenuation joins gamma at real w (s1 of the test) or the frequency
    becomes w - i alpha/2 (s2).  Returns (u, r, k): the direct solution, the distance
    of every node from the source, and the wavenumber of the free-space problem."""
    n = np.array([nn, nn])
    M = O.getRegularMesh([0.0, 10.0, 0.0, 10.0], n - 1)
    m = np.ones(nn * nn)
    w, alpha = 2 * np.pi * 2.5, 0.5 * 2 * np.pi
    gamma = O.getABL(n, False, [pad, pad], O.getMaximalFrequency(m, M)).ravel(order="F")
    q = np.zeros((nn * nn, 1), dtype=complex)
    q[O.loc2cs(n, [src0 + 1, src0 + 1]) - 1] = 1.0 / M.h[0] ** 2
    if complex_omega:
        H = O.GetHelmholtzOperator(M, m, w - 0.5j * alpha, gamma, False, False)
        k = w - 0.5j * alpha                         # k^2 = w'^2 exactly (gamma = 0 inside)
    else:
        H = O.GetHelmholtzOperator(M, m, w, gamma + alpha, False, False)
        k = np.sqrt(w * w - 1j * alpha * w)          # k^2 = w^2 (1 - i alpha / w)
        k = k if k.imag < 0 else -k
    xn = O.getNodalGrid(M)
    r = np.hypot(xn[:, 0] - src0 * M.h[0], xn[:, 1] - src0 * M.h[1])
    return O.direct_solve(H, q)[:, 0], r, k


def _green_error(u, r, k, r0=0.3, r1=2.5):
    """Relative L2 distance to the decaying free-space Green's function of
    -Laplace - k^2, (-i/4) H0^(2)(k r), over r0 <= r <= r1 (inside the layer)."""
    from scipy.special import hankel2
    sel = (r >= r0) & (r <= r1)
    g = -0.25j * hankel2(0, k * r[sel])
    return float(np.linalg.norm(u[sel] - g) / np.linalg.norm(g))


@pytest.mark.parametrize("complex_omega", [False, True])
def test_attenuation_matches_greens_function(O, complex_omega):
    """The reference's attenuation example (512^2 nodes, source at div(n, 2)) only
    plots its two solutions beside an analytic ray solution; here each is held to
    the exact damped Green's function of its own continuous problem."""
    u, r, k = _attenuated_point_source(O, 512, 35, 255, complex_omega)
    assert _green_error(u, r, k) < 0.05


def test_attenuated_green_error_is_second_order(O):
    """Halving h (257^2 -> 513^2 nodes, same physical layer width, source at the
    centre node) divides the distance to the Green's function by about 4."""
    e = [_green_error(*_attenuated_point_source(O, nn, pad, (nn - 1) // 2, True)) for nn, pad in ((257, 18), (513, 35))]
    assert 3.5 < e[0] / e[1] < 4.6, e


@pytest.mark.parametrize("shifted", [False, True])
def test_surface_source_matches_half_space_greens_function(O, shifted):
    """test/HelmholtzTest.jl restated (it only plots): 257x129 nodes on
    [0,13.5]x[0,4.2], unit slowness, f = 1, gamma = 0.01, Neumann top with the
    absorbing layer (pad 25, getMaximalFrequency) and Sommerfeld rows elsewhere,
    the top point source q = 1/||h||^2, solved with H and with SH = H + shift 0.1.
    The Neumann rows mirror the half-space, so away from the layer the solution is
    the full-space damped Green's function with strength q hx hy.  This holds the
    source scaling, the mirror rows of the Neumann top and the sign of the shift
    (the Sommerfeld rows matter little here: the layer already absorbs)."""
    from scipy.special import hankel2
    M = O.getRegularMesh([0.0, 13.5, 0.0, 4.2], [256, 128])
    m = np.ones(257 * 129)
    w = 2 * np.pi
    H, _ = O.GetHelmholtzOperatorABL(M, m, w, 0.01 * np.ones(m.size), True, [25, 25],
                                     O.getMaximalFrequency(m, M), True)
    k2 = w * w - 1j * 0.01 * w
    if shifted:
        H = (H + O.GetHelmholtzShiftOP(m, w, 0.1)).tocsr()
        k2 -= 0.1j * w * w
    k = np.sqrt(k2)
    k = k if k.imag < 0 else -k
    q, src = O.getAcousticPointSource(M, np.complex128)
    assert src == [128, 1] and q.max() == pytest.approx(1.0 / (M.h[0] ** 2 + M.h[1] ** 2))
    u = O.direct_solve(H, q[:, None])[:, 0]
    xn = O.getNodalGrid(M)
    r = np.hypot(xn[:, 0] - (src[0] - 1) * M.h[0], xn[:, 1] - (src[1] - 1) * M.h[1])
    sel = (r >= 0.5) & (r <= 2.5)
    g = -0.25j * hankel2(0, k * r[sel]) * q.max() * M.h[0] * M.h[1]
    assert np.linalg.norm(u[sel] - g) / np.linalg.norm(g) < 0.05


@pytest.fixture(scope="module")
def shifted_laplacian_example(O):
    """test/ShiftedLaplacianTest.jl:14-83 restated: v = 1.5 on 257x129 nodes of
    [0,13.5]x[0,4.2], f = 2.5, gamma = 0.01 w plus the absorbing layer (pad 16,
    getMaximalFrequency), Neumann top, Sommerfeld; q = 1/h1^2 at (div(n1, 2), 1)."""
    M = O.getRegularMesh([0.0, 13.5, 0.0, 4.2], [256, 128])
    m = np.full(257 * 129, 1 / 1.5**2)
    w = 2 * np.pi * 2.5
    H, gamma = O.GetHelmholtzOperatorABL(M, m, w, w * 0.01 * np.ones(m.size), True, [16, 16],
                                         O.getMaximalFrequency(m, M), True)
    n = M.n + 1
    q = np.zeros(int(np.prod(n)), dtype=complex)
    q[O.loc2cs(n, [n[0] // 2, 1]) - 1] = 1.0 / M.h[0] ** 2
    rng = np.random.default_rng(0)
    B2 = rng.random((q.size, 2)) + 1j * rng.random((q.size, 2))  # rand(ComplexF64, n, 2)
    return M, m, np.ravel(gamma, order="F"), w, H, q, B2


@pytest.mark.parametrize("krylov,cycle,restart,rhs,relax", [
    ("GMRES", "W", 20, "point", "Jac"),      # :63-73  getMGparam(levels 2, Jac 0.75, 2/2, 'W'), GMRES(20)
    ("BiCGSTAB", "W", 0, "point", "Jac"),    # :75-78
    ("BiCGSTAB", "W", 0, "random", "Jac"),   # :121-135 two random right-hand sides
    ("GMRES", "K", 5, "random", "Jac-GMRES"),  # :137-142 relaxType "Jac-GMRES", K-cycle, GMRES(5)
    ("GMRES", "K", 5, "random", "Jac"),      # the same with damped Jacobi (the relaxation the GPU path builds)
])
def test_shifted_laplacian_example(O, shifted_laplacian_example, krylov, cycle, restart, rhs, relax):
    """Each solve of the reference's shifted-Laplacian example (shift 0.2/10 on every
    level, maxIter 30, tolerance 1e-6) reaches the residual the example prints and
    the direct solution."""
    M, m, gamma, w, H, q, B2 = shifted_laplacian_example
    B = q if rhs == "point" else B2
    sol = O.slmg_solve(M, m, gamma, w, True, True, B, levels=2, shift=0.02, relax_w=0.75, pre=2, post=2,
                       restart=max(restart, 1), tol=1e-6, max_outer=30, cycle=cycle, krylov=krylov,
                       relax_type=relax)
    assert np.all(sol.result.converged)
    X = sol.X.reshape(q.size, -1)
    Bm = B.reshape(q.size, -1)
    assert np.all(np.linalg.norm(H @ X - Bm, axis=0) <= 1e-6 * np.linalg.norm(Bm, axis=0))
    Xd = O.direct_solve(H, Bm)
    assert np.linalg.norm(X - Xd) / np.linalg.norm(Xd) < 1e-4


def test_laplacian_rows_follow_reference_boundary_rule(O):
    """(2u_0 - 2u_1)/h^2 boundary rows (orderNeumannBC = 2), interior [-1 2 -1]/h^2."""
    D = O.dxxMat(5, 0.5).toarray()
    h2 = 0.25
    np.testing.assert_allclose(D[0, :2] * h2, [2, -2])
    np.testing.assert_allclose(D[-1, -2:] * h2, [-2, 2])
    np.testing.assert_allclose(D[2, 1:4] * h2, [-1, 2, -1])
    D1 = O.dxxMat(5, 0.5, 1).toarray()
    np.testing.assert_allclose(D1[0, :2] * h2, [1, -1])


@pytest.mark.parametrize("nc", [(24, 16), (8, 6, 10)])
def test_sommerfeld_term_keeps_order_two_with_first_order_laplacian(O, nc):
    """GetHelmholtzOperator(..., orderNeumannBC = 1) with Sommerfeld on: the
    Laplacian's boundary rows take BC = 1, the Sommerfeld term keeps BC = 2
    (src/GetHelmholtz.jl:45 passes no order to getSommerfeldBC)."""
    import problems as PB
    P = PB.layered(nc, seed=2, pad=2, neumann=False, ellipsoid=len(nc) == 3)
    H1 = O.GetHelmholtzOperator(P["M"], P["m"], P["w"], P["gamma"], False, True, 1)
    ref = PB.operator_from_parts(P, 1)
    assert abs(H1 - ref).max() <= 1e-14 * abs(ref).max()
    # and it differs from the operator a BC = 1 Sommerfeld term would give
    somm1 = O.getSommerfeldBC(P["M"], P["m"], P["w"], False, 1).ravel(order="F")
    somm2 = O.getSommerfeldBC(P["M"], P["m"], P["w"], False, 2).ravel(order="F")
    assert np.abs(somm2 - somm1).max() > 0.1 * np.abs(somm2).max()


def test_abl_corner_rule_2d(O):
    """2D absorbing layer corners combine as a + b - ab (src/GetHelmholtz.jl:141-163)."""
    g = O.getABL([20, 12], False, [4, 3], 1.0)
    a = (4.0**2) / 16  # b_bwd1[0]
    b = (3.0**2) / 9   # b_bwd2[0]
    assert g[0, 0] == pytest.approx(a + b - a * b)
    assert g[10, 6] == 0.0
    gn = O.getABL([20, 12], True, [4, 3], 1.0)
    assert gn[10, 0] == 0.0  # no layer on top with NeumannAtFirstDim


def test_oracle_slmg_matches_direct_solve(O):
    P = PB.gradient_2d((64, 64))
    B = PB.rhs(P["H"].shape[0], 3, seed=3)
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=3, tol=1e-10, max_outer=60)
    X = O.direct_solve(P["H"], B)
    assert np.all(sol.result.converged)
    assert np.linalg.norm(sol.X - X) / np.linalg.norm(X) < 1e-7


def test_oracle_transpose_solve(O):
    P = PB.gradient_2d((32, 32))
    B = PB.rhs(P["H"].shape[0], 2, seed=5)
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=2, tol=1e-10, max_outer=60,
                       transpose=True)
    X = O.direct_solve(P["H"].conj().T.tocsr(), B)
    assert np.linalg.norm(sol.X - X) / np.linalg.norm(X) < 1e-7


def test_c_oracle_restart_cycles_continue_one_solve(O, cpu_slmg):
    """A restarted FGMRES solve continued one restart cycle per call from the last
    X takes the same iterates as one call (the CPU baseline times such cycles)."""
    P = PB.gradient_2d((64, 64))
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    B = PB.rhs(P["H"].shape[0], 2, seed=9)
    cpu = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 3)
    whole = cpu.solve(B, tol=1e-8, max_outer=60, cycle="K")
    X = np.zeros_like(B)
    iters = np.zeros(2, dtype=np.int64)
    for _ in range(60):
        r = cpu.solve(B, tol=1e-8, max_outer=1, cycle="K", X0=X)
        X = r.X
        iters += r.iters
        if np.all(r.relres <= 1e-8):
            break
    np.testing.assert_array_equal(iters, whole.iters)
    assert np.linalg.norm(X - whole.X) <= 1e-12 * np.linalg.norm(whole.X)


def test_c_oracle_matches_numpy_oracle(O, cpu_slmg):
    P = PB.gradient_2d((64, 64))
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    B = PB.rhs(P["H"].shape[0], 3, seed=7)
    B[:, 1] = 0.0  # a zero column stays zero
    cpu = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 3)
    r = cpu.solve(B, tol=1e-8, max_outer=60)
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=3, tol=1e-8, max_outer=60)
    np.testing.assert_array_equal(r.iters, sol.result.iters)
    assert np.linalg.norm(r.X - sol.X) <= 1e-12 * np.linalg.norm(sol.X)
    assert np.all(r.X[:, 1] == 0)


def test_c_oracle_w_cycle_3d(O, cpu_slmg):
    P = PB.layered((16, 16, 16), seed=2, pad=3, ellipsoid=True)
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    B = PB.rhs(P["H"].shape[0], 2, seed=9)
    cpu = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 3)
    r = cpu.solve(B, tol=1e-8, max_outer=60, cycle="W")
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=3, tol=1e-8, max_outer=60,
                       cycle="W")
    np.testing.assert_array_equal(r.iters, sol.result.iters)
    X = O.direct_solve(P["H"], B)
    assert np.linalg.norm(r.X - X) / np.linalg.norm(X) < 1e-6


def test_oracle_kcycle_converges_faster_than_v(O):
    """The oracle's K-cycle (two preconditioned FGMRES steps per coarse level) solves
    to the same residual as the V-cycle in fewer outer iterations."""
    import problems as PB
    P = PB.layered((64, 64), seed=3, pad=8)
    B = PB.rhs(P["m"].size, 2, seed=1)
    it = {}
    for cyc in ("V", "K"):
        sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=4, tol=1e-8, max_outer=60,
                           cycle=cyc)
        r = np.linalg.norm(P["H"] @ sol.result.X - B, axis=0) / np.linalg.norm(B, axis=0)
        assert np.all(r <= 1e-8 * 1.0001)
        it[cyc] = int(sol.result.iters.max())
    assert it["K"] < it["V"], it


@pytest.mark.parametrize("cycle", ["W", "K"])
def test_c_oracle_cycles_match_numpy_oracle(O, cpu_slmg, cycle):
    """The two restatements of the solve (NumPy and threaded C) take the same
    iterations per column with the W- and the K-cycle and agree on the solution."""
    P = PB.layered((64, 64), seed=3, pad=8)
    B = PB.rhs(P["m"].size, 3, seed=1)
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    r = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 4).solve(B, tol=1e-8, max_outer=60, cycle=cycle)
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=4, tol=1e-8, max_outer=60,
                       cycle=cycle)
    np.testing.assert_array_equal(r.iters, sol.result.iters)
    assert np.abs(r.X - sol.result.X).max() <= 1e-12 * np.abs(sol.result.X).max()


@pytest.mark.parametrize("cycle", ["V", "K"])
def test_c_oracle_rediscretized_matches_numpy_oracle(O, cpu_slmg, cycle):
    """The C solve on a prebuilt re-discretised hierarchy takes the NumPy
    oracle's iterations (coarse_op = re-discretise, the CPU baseline of that option)."""
    P = PB.layered((64, 64), seed=4, pad=8)
    B = PB.rhs(P["m"].size, 2, seed=2)
    hier = O.build_hierarchy_rediscretized(P["M"], P["m"], P["gamma"], P["w"], 0.5, True, True, 4)
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    r = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 4, hier=hier).solve(B, tol=1e-8, max_outer=60, cycle=cycle)
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=4, tol=1e-8, max_outer=60,
                       cycle=cycle, coarse="rediscretize")
    np.testing.assert_array_equal(r.iters, sol.result.iters)
    assert np.abs(r.X - sol.result.X).max() <= 1e-12 * np.abs(sol.result.X).max()


def test_kcycle_depth_galerkin_vs_rediscretized_3d(O, cpu_slmg):
    """3D layered+ellipsoid at 10 points per wavelength: with four levels the
    Galerkin K-cycle converges, but a fifth level (0.625 points per wavelength)
    stalls it; the re-discretised K-cycle is unaffected by the extra level.
    This is why the 257^3 solve needs re-discretised coarse levels (or four
    Galerkin levels) with its five-level hierarchy."""
    P = PB.layered((64, 64, 64), seed=7, pad=8, ellipsoid=True)
    B = np.zeros((P["m"].size, 1), dtype=complex)
    B[32 + 65 * (32 + 65 * 1), 0] = 1.0
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    it = {}
    for coarse in ("galerkin", "rediscretize"):
        for levels in (4, 5):
            hier = None
            if coarse == "rediscretize":
                hier = O.build_hierarchy_rediscretized(P["M"], P["m"], P["gamma"], P["w"], 0.5, True, True, levels)
            r = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], levels, hier=hier).solve(B, tol=1e-6, max_outer=15, cycle="K")
            it[coarse, levels] = (int(r.iters[0]), float(r.relres[0]))
    assert it["galerkin", 4][0] < 60 and it["galerkin", 4][1] <= 1e-6, it
    assert it["galerkin", 5][1] > 1e-6, it          # not converged in 15 restarts of 10
    assert it["rediscretize", 5][0] <= 1.2 * it["rediscretize", 4][0] and it["rediscretize", 5][1] <= 1e-6, it


@pytest.mark.parametrize("cycle,pre,post,gmres_from", [("V", 1, 1, 0), ("V", 2, 2, 0), ("K", 3, 1, 0), ("W", 2, 2, 0),
                                                         ("K", 1, 1, 1), ("V", 2, 1, 2)])
def test_c_oracle_jac_gmres_matches_numpy_oracle(O, cpu_slmg, cycle, pre, post, gmres_from):
    """relaxType "Jac-GMRES" (on every level, or from a coarse level down): the
    NumPy and the threaded C restatements take the same iterations per column and
    agree on the solution."""
    P = PB.layered((64, 64), seed=3, pad=8)
    B = PB.rhs(P["m"].size, 3, seed=1)
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    r = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 4).solve(B, tol=1e-8, max_outer=60, cycle=cycle, pre=pre, post=post,
                                                       relax="Jac-GMRES", gmres_from=gmres_from)
    sol = O.slmg_solve(P["M"], P["m"], P["gamma"], P["w"], True, True, B, levels=4, tol=1e-8, max_outer=60,
                       cycle=cycle, pre=pre, post=post, relax_type="Jac-GMRES", gmres_from=gmres_from)
    np.testing.assert_array_equal(r.iters, sol.result.iters)
    assert np.abs(r.X - sol.result.X).max() <= 1e-12 * np.abs(sol.result.X).max()


def test_jac_gmres_step_properties(O):
    """One Jac-GMRES smoothing never raises a column's residual (GMRES minimises it
    over a space that contains the old iterate); as many steps as unknowns solve
    the level exactly; a zero-residual column is left as it is."""
    P = PB.gradient_2d((8, 8))
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    L = O.build_hierarchy(SH, P["M"], 1).levels[0]
    rng = np.random.default_rng(0)
    n = SH.shape[0]
    b = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    x = rng.standard_normal((n, 3)) + 0j
    r0 = np.linalg.norm(b - SH @ x, axis=0)
    for steps in (1, 2, 5):
        x1 = O.gmres_relax(L, x.copy(), b, 0.8, steps)
        assert np.all(np.linalg.norm(b - SH @ x1, axis=0) <= r0 * (1 + 1e-12))
    xs = O.gmres_relax(L, np.zeros((n, 1), complex), b[:, :1], 0.8, n)
    assert np.linalg.norm(b[:, :1] - SH @ xs) <= 1e-8 * np.linalg.norm(b[:, :1])
    xe = np.linalg.solve(SH.toarray(), b[:, :1])
    be = SH @ xe  # the residual b - A x is exactly zero for this pair
    np.testing.assert_array_equal(O.gmres_relax(L, xe.copy(), be, 0.8, 2), xe)


def test_jac_gmres_rescues_deep_galerkin_3d(O, cpu_slmg):
    """3D layered+ellipsoid at 10 points per wavelength, five Galerkin levels (the
    fifth at 0.625 points per wavelength): the K-cycle with damped Jacobi does not
    converge in 15 restarts of 10, with one Jac-GMRES step per smoothing it does,
    well within them, and as well with GMRES smoothing on the coarse levels only
    (damped Jacobi kept on the fine level, where the smoothing costs the most)."""
    P = PB.layered((64, 64, 64), seed=7, pad=8, ellipsoid=True)
    B = np.zeros((P["m"].size, 1), dtype=complex)
    B[32 + 65 * (32 + 65 * 1), 0] = 1.0
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    S = cpu_slmg.CpuSLMG(P["H"], SH, P["M"], 5)
    jac = S.solve(B, tol=1e-6, max_outer=15, cycle="K")
    jg = S.solve(B, tol=1e-6, max_outer=15, cycle="K", relax="Jac-GMRES")
    assert jac.relres[0] > 1e-6, jac.relres
    assert jg.relres[0] <= 1e-6 and jg.iters[0] <= 60, (jg.iters, jg.relres)
    jc = S.solve(B, tol=1e-6, max_outer=15, cycle="K", relax="Jac-GMRES", gmres_from=1)
    assert jc.relres[0] <= 1e-6 and jc.iters[0] <= 1.1 * jg.iters[0], (jc.iters, jg.iters)


# ---------------------------------------------------------------------------
# The multigrid and Krylov internals (Multigrid.jl and KrylovMethods.jl, absent
# from the reference tree) pinned against formulations independent of the
# oracle's code: SciPy's GMRES and BiCGSTAB, and the algebraic error
# propagation operator of a multigrid cycle.
# ---------------------------------------------------------------------------
def _pin_problem(O, dims=(32, 32), levels=3, pad=4):
    P = PB.layered(dims, seed=3, pad=pad, ellipsoid=len(dims) == 3)
    SH = (P["H"] + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    return P, SH, O.build_hierarchy(SH, P["M"], levels)


def _gmres_scipy(A, prec, b, restart, maxiter, tol):
    """SciPy's restarted GMRES (modified Gram-Schmidt, LAPACK Givens rotations) on
    the right-preconditioned operator A M from a zero guess; returns x = M u, the
    inner iterations taken and SciPy's exit code."""
    import scipy.sparse.linalg as spla
    n = A.shape[0]
    AM = spla.LinearOperator((n, n), matvec=lambda u: A @ prec(u.reshape(n, 1))[:, 0], dtype=np.complex128)
    hist = []
    u, info = spla.gmres(AM, b, rtol=tol, atol=0.0, restart=restart, maxiter=maxiter, callback=hist.append,
                         callback_type="pr_norm")
    return prec(u.reshape(n, 1))[:, 0], len(hist), info


@pytest.mark.parametrize("cycle,sweeps,tol", [("V", 1, 1e-6), ("V", 1, 1e-10), ("W", 2, 1e-8)])
def test_fgmres_matches_scipy_gmres_on_the_preconditioned_operator(O, cycle, sweeps, tol):
    """With a linear preconditioner M (a V or W cycle from a zero guess), FGMRES(10)
    right-preconditioned by M takes the iterates x_k = M u_k of GMRES(10) on H M:
    SciPy's GMRES must stop after as many iterations, across restarts, at the same
    solution to rounding."""
    P, SH, hier = _pin_problem(O)
    H = P["H"]
    prec = lambda V: O.mg_cycle(hier, 0, V, 0.8, sweeps, sweeps, cycle)
    b = PB.rhs(H.shape[0], 1, seed=4)[:, 0]
    res = O.fgmres(lambda X: H @ X, prec, b[:, None], 10, tol, 50)
    x, its, info = _gmres_scipy(H, prec, b, 10, 50, tol)
    assert info == 0 and res.converged[0]
    assert res.outer >= 2  # the comparison spans restarts
    assert its == res.iters[0]
    assert np.linalg.norm(x - res.X[:, 0]) <= 1e-12 * np.linalg.norm(res.X[:, 0])


@pytest.mark.parametrize("k", [1, 3, 8])
def test_bicgstab_matches_scipy_bicgstab_iterates(O, k):
    """The oracle's right-preconditioned BiCGSTAB (the Krylov method of
    solveBiCGSTAB_MG) and SciPy's BiCGSTAB, both van der Vorst's recurrences with
    the preconditioner applied to p and s, agree after every number of iterations."""
    import scipy.sparse.linalg as spla
    P, SH, hier = _pin_problem(O)
    H = P["H"]
    n = H.shape[0]
    prec = lambda V: O.mg_cycle(hier, 0, V, 0.8, 1, 1, "V")
    b = PB.rhs(n, 1, seed=6)[:, 0]
    r = O.bicgstab(lambda X: H @ X, prec, b[:, None], 1e-30, k)
    M = spla.LinearOperator((n, n), matvec=lambda v: prec(v.reshape(n, 1))[:, 0], dtype=np.complex128)
    x, _ = spla.bicgstab(H, b, rtol=1e-30, atol=0.0, maxiter=k, M=M)
    assert r.iters[0] == k
    assert np.linalg.norm(x - r.X[:, 0]) <= 1e-12 * np.linalg.norm(r.X[:, 0])


def _interp_1d(c):
    """Nodal linear interpolation from c coarse cells to 2c fine cells, from its
    stencil: 1 at the coincident nodes, 1/2 from both neighbours in between."""
    P = np.zeros((2 * c + 1, c + 1))
    for i in range(c + 1):
        P[2 * i, i] = 1.0
    for i in range(c):
        P[2 * i + 1, i] = P[2 * i + 1, i + 1] = 0.5
    return P


@pytest.mark.parametrize("dims,cycle,sweeps", [((16, 16), "V", 1), ((16, 16), "W", 2), ((16, 8), "W", 1),
                                               ((8, 8, 8), "V", 1)])
def test_cycle_is_its_error_propagation_operator(O, dims, cycle, sweeps):
    """A V or W cycle from a zero guess is the linear map B_l = (I - E_l) A_l^-1,
    E_l = S^s (I - P_l B_{l+1} R_l A_l)^c S^s with damped Jacobi S = I - w D^-1 A_l,
    c = 1 (V) or 2 (W; above the coarsest level the exact correction is a projection,
    so squaring it changes nothing there), B = A^-1 on the coarsest level.  P_l is
    the Kronecker product (axis 1 fastest) of the 1D interpolation built here,
    R_l = P_l^T / 2^d and A_{l+1} = R_l A_l P_l.  The oracle's hierarchy must hold
    these matrices and its cycle applied to the identity must be B_0."""
    levels = 3
    P, SH, hier = _pin_problem(O, dims, levels, pad=2)
    d, w, c = len(dims), 0.8, 2 if cycle == "W" else 1
    A, Ps, Rs = [SH.toarray()], [], []
    cells = list(dims)
    for _ in range(levels - 1):
        Pl = _interp_1d(cells[0] // 2)
        for ck in cells[1:]:
            Pl = np.kron(_interp_1d(ck // 2), Pl)
        Ps.append(Pl)
        Rs.append(Pl.T / 2.0**d)
        A.append(Rs[-1] @ A[-1] @ Pl)
        cells = [ck // 2 for ck in cells]
    for lev in range(levels):
        Ao = hier.levels[lev].A.toarray()
        assert np.linalg.norm(Ao - A[lev]) <= 1e-13 * np.linalg.norm(A[lev])
    B = np.linalg.inv(A[-1])
    for lev in range(levels - 2, -1, -1):
        I = np.eye(A[lev].shape[0])
        S = np.linalg.matrix_power(I - w * A[lev] / np.diag(A[lev])[:, None], sweeps)
        E = S @ np.linalg.matrix_power(I - Ps[lev] @ B @ Rs[lev] @ A[lev], c) @ S
        B = (I - E) @ np.linalg.inv(A[lev])
    Bo = O.mg_cycle(hier, 0, np.eye(A[0].shape[0], dtype=np.complex128), w, sweeps, sweeps, cycle)
    assert np.linalg.norm(Bo - B) <= 1e-12 * np.linalg.norm(B)


def test_kcycle_correction_is_two_gmres_steps(O):
    """The K-cycle's coarse correction on a level (Multigrid.jl cycleType 'K') is two
    FGMRES steps from a zero guess right-preconditioned by the level's cycle; with
    the exact solve below, that cycle is linear and the correction equals one
    GMRES(2) cycle of SciPy's on A_l M_l."""
    P, SH, hier = _pin_problem(O)
    A1 = hier.levels[1].A
    b = PB.rhs(A1.shape[0], 2, seed=8)
    out = O.kcycle(hier, 1, b, 0.8, 1, 1)
    prec = lambda V: O.mg_cycle(hier, 1, V, 0.8, 1, 1, "K")
    for c in range(2):
        x, its, _ = _gmres_scipy(A1, prec, b[:, c], 2, 1, 1e-30)
        assert its == 2
        assert np.linalg.norm(x - out[:, c]) <= 1e-12 * np.linalg.norm(out[:, c])


@pytest.mark.parametrize("steps", [1, 2, 3])
def test_jac_gmres_smoother_is_gmres_on_the_correction(O, steps):
    """relaxType "Jac-GMRES" from an iterate x0: x0 plus `steps` GMRES steps on the
    correction A e = b - A x0, right-preconditioned by one damped-Jacobi sweep
    (M = w D^-1); SciPy's GMRES(steps) on A M for that residual gives the same x."""
    P, SH, hier = _pin_problem(O)
    L0 = hier.levels[0]
    A0 = L0.A
    b = PB.rhs(A0.shape[0], 2, seed=9)
    x0 = 0.1 * PB.rhs(A0.shape[0], 2, seed=10)
    xr = O.gmres_relax(L0, x0.copy(), b, 0.8, steps)
    prec = lambda V: 0.8 * L0.dinv[:, None] * V
    for c in range(2):
        e, its, _ = _gmres_scipy(A0, prec, b[:, c] - A0 @ x0[:, c], steps, 1, 1e-30)
        assert its == steps
        assert np.linalg.norm(x0[:, c] + e - xr[:, c]) <= 1e-12 * np.linalg.norm(xr[:, c])
