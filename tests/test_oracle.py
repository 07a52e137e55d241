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
