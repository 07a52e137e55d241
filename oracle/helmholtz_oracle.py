"""CPU oracle for the shifted-Laplacian multigrid (SLMG) Helmholtz solve.

TEST INFRASTRUCTURE ONLY.  This module is the checker: it is imported by
``tests/``, by ``__graft_entry__.smoke()`` and by the ``cpu_baseline`` leg of
``bench.py``.  The product (the CUDA library and its host mirror) never calls
it, and nothing here is ever measured as the product.

It restates, in NumPy/SciPy and complex FP64, the reference algorithm of
JuliaInv/Helmholtz.jl for the acoustic nodal Helmholtz operator and the
shifted-Laplacian multigrid preconditioned FGMRES solve:

* operator assembly      -- src/GetHelmholtz.jl:22-50, 75-83, 97-247
* nodal Laplacian        -- src/PlainNodalLaplacian.jl:4-46
* point sources          -- src/getPointSource.jl:63-111
* solver adapter         -- src/ShiftedLaplacianMultigridSolver.jl:33-102

The multigrid cycle, the transfer operators, the coarsest direct solve and
FGMRES live in Multigrid.jl v0.8.0 (git-tree 70508e009fd168c5dbe3b0cb274f85173c3e7928)
and KrylovMethods.jl v0.6.0 (git-tree ceb12d552f1d...), pinned in the
reference's Manifest.toml:46-52,91-97 and not vendored.  Their published
algorithms are restated here from the mathematics:

* geometric coarsening by a factor 2 per axis (cells n -> n/2),
* bi/trilinear nodal prolongation P, full-weighting restriction R = P^T / 2^d,
* Galerkin coarse operators A_{l+1} = R A_l P (the RAP path that
  src/ShiftedLaplacianMultigridSolver.jl:64-65 takes),
* damped Jacobi relaxation x <- x + w D^{-1} (b - A x),
* V/W cycles with a direct solve on the coarsest level,
* right-preconditioned flexible GMRES(restart) per right-hand-side column,
  classical Gram-Schmidt with DGKS selective reorthogonalisation, Givens rotations,
  relative-residual stopping test ||r_j|| <= tol * ||b_j||.

Parity status: the operator assembly is pinned by the reference's own
known-answer test (the manufactured-solution O(h^2) convergence check of
test/testFictitiousSource2D.jl:10-70, restated in tests/test_oracle.py).  The
multigrid/Krylov internals are not pinned by any reference test (the reference
tests print residuals only); the solve is anchored on the unique solution of
H X = B, computed here by a sparse direct solve exactly as the reference tests
do (test/HelmholtzTest.jl:42).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


# ---------------------------------------------------------------------------
# Mesh (the jInv RegularMesh fields the path uses: domain, n cells, h, dim)
# ---------------------------------------------------------------------------
@dataclass
class RegularMesh:
    domain: np.ndarray
    n: np.ndarray  # cells per axis
    h: np.ndarray
    dim: int

    @property
    def nodes(self) -> np.ndarray:
        return self.n + 1


def getRegularMesh(domain, n) -> RegularMesh:
    """jInv getRegularMesh: h = (domain[2k+1] - domain[2k]) / n[k]."""
    domain = np.asarray(domain, dtype=np.float64).ravel()
    n = np.asarray(n, dtype=np.int64).ravel()
    h = (domain[1::2] - domain[0::2]) / n
    return RegularMesh(domain=domain, n=n, h=h, dim=len(n))


def getNodalGrid(M: RegularMesh) -> np.ndarray:
    """Node coordinates, column-major (axis 1 fastest), one row per node."""
    axes = [M.domain[2 * k] + M.h[k] * np.arange(M.n[k] + 1) for k in range(M.dim)]
    grids = np.meshgrid(*axes, indexing="ij")
    return np.stack([g.ravel(order="F") for g in grids], axis=1)


# ---------------------------------------------------------------------------
# Discretisation (src/GetHelmholtz.jl, src/PlainNodalLaplacian.jl)
# ---------------------------------------------------------------------------
def getMaximalFrequency(m, M: RegularMesh) -> float:
    """src/GetHelmholtz.jl:75-79 -- 10 points per wavelength at max slowness."""
    return (0.1 * 2 * math.pi) / (float(np.max(M.h)) * math.sqrt(float(np.max(m))))


def getBC(orderNeumannBC: int = 2) -> float:
    """src/PlainNodalLaplacian.jl:4-15."""
    return 1.0 if orderNeumannBC == 1 else 2.0


def dxxMat(n: int, h: float, orderNeumannBC: int = 2) -> sp.csr_matrix:
    """src/PlainNodalLaplacian.jl:18-30: [-1 2 -1]/h^2 with ghost-reflection
    boundary rows (BC u_1 - BC u_2)/h^2 (non-symmetric for BC=2)."""
    BC = getBC(orderNeumannBC)
    O1 = -np.ones(n - 1)
    O1[n - 2] = -BC
    O2 = 2.0 * np.ones(n)
    O2[0] = BC
    O2[n - 1] = BC
    O3 = -np.ones(n - 1)
    O3[0] = -BC
    return sp.diags([O1 / h**2, O2 / h**2, O3 / h**2], [-1, 0, 1], format="csr")


def getNodalLaplacianMatrix(M: RegularMesh, orderNeumannBC: int = 2) -> sp.csr_matrix:
    """src/PlainNodalLaplacian.jl:32-46: Kronecker sum, axis 1 fastest."""
    nodes = M.n + 1
    I1 = sp.identity(nodes[0], format="csr")
    I2 = sp.identity(nodes[1], format="csr")
    D1 = dxxMat(int(nodes[0]), float(M.h[0]), orderNeumannBC)
    D2 = dxxMat(int(nodes[1]), float(M.h[1]), orderNeumannBC)
    if M.dim == 2:
        return (sp.kron(I2, D1) + sp.kron(D2, I1)).tocsr()
    I3 = sp.identity(nodes[2], format="csr")
    D3 = dxxMat(int(nodes[2]), float(M.h[2]), orderNeumannBC)
    return (sp.kron(I3, sp.kron(I2, D1) + sp.kron(D2, I1)) + sp.kron(D3, sp.kron(I2, I1))).tocsr()


def getABL(n, NeumannAtFirstDim: bool, ABLpad, ABLamp: float) -> np.ndarray:
    """src/GetHelmholtz.jl:97-220 (the active impl=1 branch in 2D).

    ``n`` are node counts.  Returns gamma with shape ``tuple(n)`` (Fortran
    order semantics: axis 0 is the fastest-varying index)."""
    n = [int(v) for v in np.ravel(n)]
    pad = [int(v) for v in np.ravel(ABLpad)]
    if len(n) == 2:
        gamma = np.zeros(n)
        p1, p2 = pad
        b_bwd1 = (np.arange(p1, 0, -1) ** 2) / p1**2
        b_bwd2 = (np.arange(p2, 0, -1) ** 2) / p2**2
        b_fwd1 = (np.arange(1, p1 + 1) ** 2) / p1**2
        b_fwd2 = (np.arange(1, p2 + 1) ** 2) / p2**2
        I1 = slice(n[0] - p1, n[0])
        I2 = slice(n[1] - p2, n[1])
        if not NeumannAtFirstDim:
            gamma[:, 0:p2] += np.ones((n[0], 1)) * b_bwd2[None, :]
            gamma[0:p1, 0:p2] -= np.outer(b_bwd1, b_bwd2)
            gamma[I1, 0:p2] -= np.outer(b_fwd1, b_bwd2)
        gamma[:, I2] += np.ones((n[0], 1)) * b_fwd2[None, :]
        gamma[0:p1, :] += b_bwd1[:, None] * np.ones((1, n[1]))
        gamma[I1, :] += b_fwd1[:, None] * np.ones((1, n[1]))
        gamma[0:p1, I2] -= np.outer(b_bwd1, b_fwd2)
        gamma[I1, I2] -= np.outer(b_fwd1, b_fwd2)
        gamma *= ABLamp
        return gamma
    # 3D branch
    x1 = np.linspace(-1.0, 1.0, n[0])
    x2 = np.linspace(-1.0, 1.0, n[1])
    x3 = np.linspace(0.0, 1.0, n[2])
    X1, X2, X3 = np.meshgrid(x1, x2, x3, indexing="ij")
    p1, p2, p3 = pad

    def side(X, x, p, axis, lo: bool, hi: bool):
        g = np.zeros(X.shape)
        if lo:
            gl = (X - x[p - 1]) ** 2
            idx = [slice(None)] * 3
            idx[axis] = slice(p, None)
            gl[tuple(idx)] = 0.0
            g += gl
        if hi:
            gr = (X - x[len(x) - p]) ** 2
            idx = [slice(None)] * 3
            idx[axis] = slice(0, len(x) - p)
            gr[tuple(idx)] = 0.0
            g += gr
        return g / (np.max(g) + 1e-5)

    gx = side(X1, x1, p1, 0, True, True)
    gy = side(X2, x2, p2, 1, True, True)
    gz = side(X3, x3, p3, 2, not NeumannAtFirstDim, True)
    gamma = (gx + gy + gz) * ABLamp
    gamma[gamma >= ABLamp] = ABLamp
    return gamma


def getSommerfeldBC(M: RegularMesh, mNodal, omega: float, NeumannOnTop: bool, orderNeumannBC: int = 2) -> np.ndarray:
    """src/GetHelmholtz.jl:222-247: -i w (BC/h_d) sqrt(m) summed over the
    boundary faces (top face skipped when NeumannOnTop).  Returns a complex
    array of node shape."""
    BC = getBC(orderNeumannBC)
    shp = tuple(int(v) for v in (M.n + 1))
    S = np.zeros(shp, dtype=np.complex128)
    m = np.reshape(np.asarray(mNodal, dtype=np.float64), shp, order="F")
    h = M.h
    c = -1j * omega * BC
    if M.dim == 2:
        if not NeumannOnTop:
            S[:, 0] += (c / h[1]) * np.sqrt(m[:, 0])
        S[:, -1] += (c / h[1]) * np.sqrt(m[:, -1])
        S[-1, :] += (c / h[0]) * np.sqrt(m[-1, :])
        S[0, :] += (c / h[0]) * np.sqrt(m[0, :])
    else:
        if not NeumannOnTop:
            S[:, :, 0] += (c / h[2]) * np.sqrt(m[:, :, 0])
        S[:, :, -1] += (c / h[2]) * np.sqrt(m[:, :, -1])
        S[:, 0, :] += (c / h[1]) * np.sqrt(m[:, 0, :])
        S[:, -1, :] += (c / h[1]) * np.sqrt(m[:, -1, :])
        S[0, :, :] += (c / h[0]) * np.sqrt(m[0, :, :])
        S[-1, :, :] += (c / h[0]) * np.sqrt(m[-1, :, :])
    return S


def helmholtz_mass(M: RegularMesh, mNodal, omega, gamma, NeumannOnTop: bool, Sommerfeld: bool,
                   orderNeumannBC: int = 2) -> np.ndarray:
    """Diagonal (mass) part of H, src/GetHelmholtz.jl:41-47, flattened column-major.

    orderNeumannBC does not reach the Sommerfeld term: src/GetHelmholtz.jl:45 calls
    getSommerfeldBC(Msh, mNodal, real(omega), NeumannAtFirstDim) without it, so the
    term takes getSommerfeldBC's default order 2 (:222) for either Laplacian."""
    m = np.asarray(mNodal, dtype=np.float64).ravel(order="F")
    g = np.asarray(gamma, dtype=np.float64).ravel(order="F")
    w = complex(omega)
    mass = -(w**2) * m * (1.0 - 1j * g / w.real)
    if Sommerfeld:
        mass = mass - getSommerfeldBC(M, m, w.real, NeumannOnTop).ravel(order="F")
    return mass


def GetHelmholtzOperator(M: RegularMesh, mNodal, omega, gamma, NeumannAtFirstDim: bool, Sommerfeld: bool,
                         orderNeumannBC: int = 2) -> sp.csr_matrix:
    """src/GetHelmholtz.jl:33-50: H = Lap + diag(mass)."""
    L = getNodalLaplacianMatrix(M, orderNeumannBC)
    mass = helmholtz_mass(M, mNodal, omega, gamma, NeumannAtFirstDim, Sommerfeld, orderNeumannBC)
    return (L.astype(np.complex128) + sp.diags(mass)).tocsr()


def GetHelmholtzOperatorABL(M: RegularMesh, mNodal, omega, gamma, NeumannAtFirstDim: bool, ABLpad, ABLamp: float,
                            Sommerfeld: bool, orderNeumannBC: int = 2):
    """src/GetHelmholtz.jl:22-31: adds the absorbing layer to gamma, returns (H, gamma)."""
    abl = getABL(M.n + 1, NeumannAtFirstDim, ABLpad, ABLamp)
    if gamma is None or np.size(gamma) == 0:
        g = abl
    else:
        g = np.reshape(np.asarray(gamma, dtype=np.float64), abl.shape, order="F") + abl
    H = GetHelmholtzOperator(M, mNodal, omega, g, NeumannAtFirstDim, Sommerfeld, orderNeumannBC)
    return H, g


def GetHelmholtzShiftOP(mNodal, omega: float, shift: float) -> sp.csr_matrix:
    """src/GetHelmholtz.jl:81-83: diag(m * i * shift * w^2)."""
    m = np.asarray(mNodal, dtype=np.float64).ravel(order="F")
    return sp.diags(m * (1j * shift * omega**2)).tocsr()


# ---------------------------------------------------------------------------
# Point sources (src/getPointSource.jl:63-111)
# ---------------------------------------------------------------------------
def getTopPointSrc(M: RegularMesh):
    """1-based source position (div(n1+1,2), [div(n2+1,2),] 1)."""
    if M.dim == 3:
        return [(int(M.n[0]) + 1) // 2, (int(M.n[1]) + 1) // 2, 1]
    return [(int(M.n[0]) + 1) // 2, 1]


def loc2cs(n, sub) -> int:
    """1-based column-major linear index (src/getPointSource.jl:82-100)."""
    n = [int(v) for v in n]
    if len(sub) == 2:
        return int(sub[0]) + (int(sub[1]) - 1) * n[0]
    return int(sub[0]) + (int(sub[1]) - 1) * n[0] + (int(sub[2]) - 1) * n[0] * n[1]


def getAcousticPointSource(M: RegularMesh, dtype=np.complex128, src=None):
    """q[src] = 1/||h||^2 on the node grid; returns (q, src) with q column-major flat."""
    if src is None:
        src = getTopPointSrc(M)
    nn = M.n + 1
    q = np.zeros(int(np.prod(nn)), dtype=dtype)
    q[loc2cs(nn, src) - 1] = 1.0 / (float(np.linalg.norm(M.h)) ** 2)
    return q, src


# ---------------------------------------------------------------------------
# Multigrid hierarchy (Multigrid.jl restated: geometric RAP, FW/bilinear)
# ---------------------------------------------------------------------------
def prolongation_1d(nc_cells: int) -> sp.csr_matrix:
    """Linear nodal interpolation from nc_cells coarse cells to 2*nc_cells fine cells."""
    ncn = nc_cells + 1
    nfn = 2 * nc_cells + 1
    rows, cols, vals = [], [], []
    for i in range(ncn):
        rows.append(2 * i); cols.append(i); vals.append(1.0)
    for i in range(nc_cells):
        rows += [2 * i + 1, 2 * i + 1]; cols += [i, i + 1]; vals += [0.5, 0.5]
    return sp.csr_matrix((vals, (rows, cols)), shape=(nfn, ncn))


def prolongation(fine_cells) -> sp.csr_matrix:
    """Bi/trilinear nodal prolongation, Kronecker product with axis 1 fastest."""
    fine_cells = [int(c) for c in fine_cells]
    for c in fine_cells:
        if c % 2:
            raise ValueError("cell count must be even to coarsen: %r" % (fine_cells,))
    Ps = [prolongation_1d(c // 2) for c in fine_cells]
    P = Ps[0]
    for Pk in Ps[1:]:
        P = sp.kron(Pk, P)
    return P.tocsr()


@dataclass
class Level:
    cells: np.ndarray
    A: sp.csr_matrix          # shifted operator at this level
    dinv: np.ndarray          # 1 / diag(A)
    P: sp.csr_matrix | None = None   # prolongation from the next coarser level
    R: sp.csr_matrix | None = None   # restriction to the next coarser level


@dataclass
class Hierarchy:
    levels: list = field(default_factory=list)
    lu: object = None


def build_hierarchy(SH: sp.csr_matrix, M: RegularMesh, nlevels: int) -> Hierarchy:
    """Galerkin hierarchy A_{l+1} = R A_l P with R = P^T / 2^d."""
    hier = Hierarchy()
    A = SH.tocsr()
    cells = np.array(M.n, dtype=np.int64)
    d = M.dim
    for lev in range(nlevels):
        L = Level(cells=cells.copy(), A=A, dinv=1.0 / A.diagonal())
        if lev < nlevels - 1:
            P = prolongation(cells)
            R = (P.T / (2.0**d)).tocsr()
            L.P, L.R = P, R
            A = (R @ A @ P).tocsr()
            cells = cells // 2
        hier.levels.append(L)
    hier.lu = spla.splu(hier.levels[-1].A.tocsc())
    return hier


def restrict_nodal(v: np.ndarray, fine_cells) -> np.ndarray:
    """Full-weighting average of a nodal field: (P^T v) / (P^T 1)."""
    P = prolongation(fine_cells)
    return (P.T @ v) / (P.T @ np.ones(P.shape[0]))


def build_hierarchy_rediscretized(M: RegularMesh, m, gamma, omega: float, shift: float, NeumannOnTop: bool,
                                  Sommerfeld: bool, nlevels: int, transpose: bool = False) -> Hierarchy:
    """The alternative MGsetup path of src/ShiftedLaplacianMultigridSolver.jl:51-62:
    the shift is folded into gamma (getShiftedHelmholtzParam, src/Helmholtz.jl:32-34),
    m and gamma are restricted to every coarse mesh and the operator is
    re-assembled there with GetHelmholtzOperator; P and R as in the Galerkin path."""
    hier = Hierarchy()
    m_l = np.asarray(m, dtype=np.float64).ravel(order="F")
    g_l = np.asarray(gamma, dtype=np.float64).ravel(order="F") + shift * float(np.real(omega))
    M_l = M
    for lev in range(nlevels):
        A = GetHelmholtzOperator(M_l, m_l, omega, g_l, NeumannOnTop, Sommerfeld)
        if transpose:
            A = A.conj().T.tocsr()
        L = Level(cells=np.array(M_l.n), A=A, dinv=1.0 / A.diagonal())
        if lev < nlevels - 1:
            P = prolongation(M_l.n)
            L.P, L.R = P, (P.T / (2.0 ** M.dim)).tocsr()
            m_l = restrict_nodal(m_l, M_l.n)
            g_l = restrict_nodal(g_l, M_l.n)
            M_l = getRegularMesh(M_l.domain, M_l.n // 2)
        hier.levels.append(L)
    hier.lu = spla.splu(hier.levels[-1].A.tocsc())
    return hier


def jacobi(L: Level, x: np.ndarray, b: np.ndarray, w: float, sweeps: int) -> np.ndarray:
    for _ in range(sweeps):
        x = x + w * (L.dinv[:, None] * (b - L.A @ x))
    return x


def gmres_relax(L: Level, x: np.ndarray, b: np.ndarray, w: float, steps: int) -> np.ndarray:
    """relaxType "Jac-GMRES" (set by test/ShiftedLaplacianTest.jl:138 for its
    K-cycle; Multigrid.jl v0.8.0, not vendored, restated from the published
    method): `steps` Arnoldi steps of GMRES on the level's operator, started
    from the current iterate and right-preconditioned by one damped-Jacobi sweep
    (M^-1 = w D^-1), classical Gram-Schmidt, then the least-squares update
    x += Z y per column.  A column with zero residual is left unchanged."""
    if steps <= 0:
        return x
    b = b.reshape(b.shape[0], -1)
    x = np.array(x, dtype=np.complex128).reshape(b.shape)
    r = b - L.A @ x
    beta = np.linalg.norm(r, axis=0)
    V = [r / np.where(beta > 0, beta, 1.0)]
    Z = []
    Hm = np.zeros((steps + 1, steps, b.shape[1]), dtype=np.complex128)
    for j in range(steps):
        Z.append(w * (L.dinv[:, None] * V[j]))
        u = L.A @ Z[j]
        h = [np.sum(np.conj(V[i]) * u, axis=0) for i in range(j + 1)]
        for i in range(j + 1):
            Hm[i, j] = h[i]
            u = u - h[i] * V[i]
        hn = np.linalg.norm(u, axis=0)
        Hm[j + 1, j] = hn
        V.append(u / np.where(hn > 0, hn, 1.0) * (hn > 0))
    for c in range(b.shape[1]):
        if beta[c] == 0:
            continue
        e = np.zeros(steps + 1, dtype=np.complex128)
        e[0] = beta[c]
        y = np.linalg.lstsq(Hm[:, :, c], e, rcond=None)[0]
        for j in range(steps):
            x[:, c] += y[j] * Z[j][:, c]
    return x


def relax(L: Level, x: np.ndarray, b: np.ndarray, w: float, sweeps: int, relax_type: str = "Jac",
          lev: int = 0, gmres_from: int = 0) -> np.ndarray:
    """The smoother of relaxType on level ``lev``: damped Jacobi ("Jac") or
    "Jac-GMRES"; with "Jac-GMRES", levels above ``gmres_from`` keep damped Jacobi
    (gmres_from = 0, every level, is the reference's option)."""
    if relax_type == "Jac-GMRES" and lev >= gmres_from:
        return gmres_relax(L, x, b, w, sweeps)
    if relax_type == "Jac-GMRES":
        return jacobi(L, x, b, w, sweeps)
    if relax_type != "Jac":
        raise ValueError(f"relaxType {relax_type!r}")
    return jacobi(L, x, b, w, sweeps)


def kcycle(hier: Hierarchy, lev: int, b: np.ndarray, w: float, pre: int, post: int,
           relax_type: str = "Jac", gmres_from: int = 0) -> np.ndarray:
    """K-cycle coarse correction on level ``lev`` (Multigrid.jl cycleType 'K',
    used by test/ShiftedLaplacianTest.jl:137-140, restated): two steps of FGMRES
    on that level's operator from a zero guess, right-preconditioned by the
    level's own cycle, per column (least squares of the 3x2 Hessenberg matrix)."""
    A = hier.levels[lev].A
    b = b.reshape(b.shape[0], -1)
    out = np.zeros_like(b)
    beta = np.linalg.norm(b, axis=0)
    V0 = b / np.where(beta > 0, beta, 1.0)
    Z0 = mg_cycle(hier, lev, V0, w, pre, post, "K", relax_type, gmres_from)
    W = A @ Z0
    h00 = np.sum(np.conj(V0) * W, axis=0)
    W = W - h00 * V0
    h10 = np.linalg.norm(W, axis=0)
    V1 = W / np.where(h10 > 0, h10, 1.0) * (h10 > 0)
    Z1 = mg_cycle(hier, lev, V1, w, pre, post, "K", relax_type, gmres_from)
    W = A @ Z1
    h01 = np.sum(np.conj(V0) * W, axis=0)
    h11 = np.sum(np.conj(V1) * W, axis=0)
    W = W - h01 * V0 - h11 * V1
    h21 = np.linalg.norm(W, axis=0)
    for c in range(b.shape[1]):
        if beta[c] == 0:
            continue
        Hm = np.array([[h00[c], h01[c]], [h10[c], h11[c]], [0.0, h21[c]]], dtype=np.complex128)
        y = np.linalg.lstsq(Hm, np.array([beta[c], 0.0, 0.0], dtype=np.complex128), rcond=None)[0]
        out[:, c] = y[0] * Z0[:, c] + y[1] * Z1[:, c]
    return out


def mg_cycle(hier: Hierarchy, lev: int, b: np.ndarray, w: float, pre: int, post: int, cycle: str = "V",
             relax_type: str = "Jac", gmres_from: int = 0) -> np.ndarray:
    """One V, W or K cycle with zero initial guess on level ``lev``."""
    L = hier.levels[lev]
    if lev == len(hier.levels) - 1:
        return hier.lu.solve(b)
    x = np.zeros_like(b)
    x = relax(L, x, b, w, pre, relax_type, lev, gmres_from)
    ncalls = 2 if cycle == "W" and lev < len(hier.levels) - 2 else 1
    for _ in range(ncalls):
        r = b - L.A @ x
        bc = L.R @ r
        if cycle == "K" and lev + 1 < len(hier.levels) - 1:
            xc = kcycle(hier, lev + 1, bc, w, pre, post, relax_type, gmres_from).reshape(bc.shape)
        else:
            xc = mg_cycle(hier, lev + 1, bc, w, pre, post, cycle, relax_type, gmres_from)
        x = x + L.P @ xc
    x = relax(L, x, b, w, post, relax_type, lev, gmres_from)
    return x


# ---------------------------------------------------------------------------
# FGMRES (KrylovMethods / Multigrid.jl solveGMRES_MG restated), per column
# ---------------------------------------------------------------------------
@dataclass
class FGMRESResult:
    X: np.ndarray
    iters: np.ndarray        # inner iterations (preconditioner applications) per column
    outer: int               # restart cycles performed
    relres: np.ndarray       # true relative residual per column
    converged: np.ndarray


def fgmres(Hmul, prec, B: np.ndarray, restart: int, tol: float, max_outer: int) -> FGMRESResult:
    """Right-preconditioned flexible GMRES(restart), all columns batched but
    mathematically independent; per-column Givens rotations; a column
    stops when its Arnoldi residual estimate drops to tol*||b_j||; the true
    residual is recomputed at each restart.  Gram-Schmidt is classical with
    the DGKS criterion: a second pass where ||w'||^2 < ||w||^2 / 2."""
    B = np.asarray(B, dtype=np.complex128)
    n, R = B.shape
    X = np.zeros_like(B)
    bnorm = np.linalg.norm(B, axis=0)
    active = bnorm > 0
    iters = np.zeros(R, dtype=np.int64)
    conv = ~active
    Rr = B.copy()
    outer = 0
    for outer in range(1, max_outer + 1):
        cols = np.nonzero(active & ~conv)[0]
        if cols.size == 0:
            outer -= 1
            break
        beta = np.linalg.norm(Rr[:, cols], axis=0)
        m = restart
        V = np.zeros((m + 1, n, cols.size), dtype=np.complex128)
        Z = np.zeros((m, n, cols.size), dtype=np.complex128)
        Hh = np.zeros((m + 1, m, cols.size), dtype=np.complex128)
        cs = np.zeros((m, cols.size), dtype=np.complex128)
        sn = np.zeros((m, cols.size), dtype=np.complex128)
        g = np.zeros((m + 1, cols.size), dtype=np.complex128)
        g[0] = beta
        V[0] = Rr[:, cols] / beta
        kcol = np.zeros(cols.size, dtype=np.int64)      # Arnoldi steps taken per column
        live = np.ones(cols.size, dtype=bool)
        for j in range(m):
            lc = np.nonzero(live)[0]
            if lc.size == 0:
                break
            Z[j][:, lc] = prec(V[j][:, lc])
            w = Hmul(Z[j][:, lc])
            # classical Gram-Schmidt; a second pass only for the columns whose
            # squared norm dropped below half (DGKS test)
            Vl = V[: j + 1][:, :, lc]
            before = np.sum(np.abs(w) ** 2, axis=0)
            h = np.einsum("knc,nc->kc", Vl.conj(), w)
            w = w - np.einsum("knc,kc->nc", Vl, h)
            after = np.sum(np.abs(w) ** 2, axis=0)
            redo = after < 0.5 * before
            if redo.any():
                h2 = np.einsum("knc,nc->kc", Vl[:, :, redo].conj(), w[:, redo])
                w[:, redo] = w[:, redo] - np.einsum("knc,kc->nc", Vl[:, :, redo], h2)
                h[:, redo] += h2
            hn = np.linalg.norm(w, axis=0)
            V[j + 1][:, lc] = w / np.where(hn > 0, hn, 1.0)
            col = np.zeros((j + 2, lc.size), dtype=np.complex128)
            col[: j + 1] = h
            col[j + 1] = hn
            # rotation i maps (u, v) -> (conj(c) u + conj(s) v, -s u + c v)
            for i in range(j):
                t = np.conj(cs[i, lc]) * col[i] + np.conj(sn[i, lc]) * col[i + 1]
                col[i + 1] = -sn[i, lc] * col[i] + cs[i, lc] * col[i + 1]
                col[i] = t
            a, bb = col[j], col[j + 1]
            den = np.sqrt(np.abs(a) ** 2 + np.abs(bb) ** 2)
            den = np.where(den > 0, den, 1.0)
            c = a / den
            s = bb / den
            cs[j, lc], sn[j, lc] = c, s
            col[j] = c.conj() * a + s.conj() * bb
            col[j + 1] = 0
            Hh[: j + 2, j][:, lc] = col
            gj = g[j, lc]
            g[j, lc] = c.conj() * gj
            g[j + 1, lc] = -s * gj
            kcol[lc] = j + 1
            iters[cols[lc]] += 1
            est = np.abs(g[j + 1, lc]) / bnorm[cols[lc]]
            live[lc[est <= tol]] = False
        # solve the triangular systems and update x per column
        for ci, c_ in enumerate(cols):
            k = int(kcol[ci])
            if k == 0:
                continue
            Hk = Hh[:k, :k, ci]
            y = np.linalg.solve(np.triu(Hk), g[:k, ci])
            X[:, c_] += Z[:k, :, ci].T @ y
        Rr[:, cols] = B[:, cols] - Hmul(X[:, cols])
        rel = np.linalg.norm(Rr[:, cols], axis=0) / bnorm[cols]
        conv[cols[rel <= tol]] = True
    relres = np.zeros(R)
    nz = bnorm > 0
    if nz.any():
        relres[nz] = np.linalg.norm(B[:, nz] - Hmul(X[:, nz]), axis=0) / bnorm[nz]
    return FGMRESResult(X=X, iters=iters, outer=outer, relres=relres, converged=conv)


def bicgstab(Hmul, prec, B: np.ndarray, tol: float, max_iter: int) -> FGMRESResult:
    """Right-preconditioned BiCGSTAB (van der Vorst 1992), the Krylov method
    of solveBiCGSTAB_MG (src/ShiftedLaplacianMultigridSolver.jl:91-93, the
    reference's default), all columns batched but independent.  Two
    preconditioner applications per iteration; a column stops when
    ||r||/||b|| <= tol (r updated recursively, true residual at the end).
    ``iters`` counts iterations, ``outer`` the maximum over the columns."""
    B = np.asarray(B, dtype=np.complex128)
    n, R = B.shape
    X = np.zeros_like(B)
    bnorm = np.linalg.norm(B, axis=0)
    live = bnorm > 0
    r = B.copy()
    rh = r.copy()
    p = np.zeros_like(B)
    v = np.zeros_like(B)
    rho_prev = np.ones(R, dtype=np.complex128)
    alpha = np.ones(R, dtype=np.complex128)
    omega = np.ones(R, dtype=np.complex128)
    iters = np.zeros(R, dtype=np.int64)
    for _ in range(max_iter):
        c = np.nonzero(live)[0]
        if c.size == 0:
            break
        rho = np.sum(rh[:, c].conj() * r[:, c], axis=0)
        beta = (rho / rho_prev[c]) * (alpha[c] / omega[c])
        p[:, c] = r[:, c] + beta * (p[:, c] - omega[c] * v[:, c])
        ph = prec(p[:, c])
        v[:, c] = Hmul(ph)
        alpha[c] = rho / np.sum(rh[:, c].conj() * v[:, c], axis=0)
        s = r[:, c] - alpha[c] * v[:, c]
        sh = prec(s)
        t = Hmul(sh)
        omega[c] = np.sum(t.conj() * s, axis=0) / np.sum(np.abs(t) ** 2, axis=0)
        X[:, c] += alpha[c] * ph + omega[c] * sh
        r[:, c] = s - omega[c] * t
        rho_prev[c] = rho
        iters[c] += 1
        rel = np.linalg.norm(r[:, c], axis=0) / bnorm[c]
        live[c[rel <= tol]] = False
    relres = np.zeros(R)
    nz = bnorm > 0
    if nz.any():
        relres[nz] = np.linalg.norm(B[:, nz] - Hmul(X[:, nz]), axis=0) / bnorm[nz]
    return FGMRESResult(X=X, iters=iters, outer=int(iters.max(initial=0)), relres=relres,
                        converged=relres <= tol * 1.0001)


@dataclass
class SLMGSolution:
    X: np.ndarray
    result: FGMRESResult
    hier: Hierarchy


def slmg_solve(M: RegularMesh, m, gamma, omega: float, NeumannOnTop: bool, Sommerfeld: bool, B: np.ndarray,
               levels: int, shift: float = 0.5, relax_w: float = 0.8, pre: int = 1, post: int = 1,
               restart: int = 10, tol: float = 1e-8, max_outer: int = 100, cycle: str = "V",
               transpose: bool = False, krylov: str = "GMRES", coarse: str = "galerkin",
               relax_type: str = "Jac", gmres_from: int = 0) -> SLMGSolution:
    """Plain FP64 SLMG: FGMRES(restart) on H (or H^H when ``transpose``),
    right-preconditioned by one multigrid cycle on SH = H + i*s*w^2*diag(m)
    (or SH^H), src/ShiftedLaplacianMultigridSolver.jl:33-102.  relax_type
    "Jac-GMRES" smooths levels >= gmres_from by GMRES steps (gmres_relax)."""
    H = GetHelmholtzOperator(M, m, omega, gamma, NeumannOnTop, Sommerfeld)
    SH = (H + GetHelmholtzShiftOP(m, omega, shift)).tocsr()
    if transpose:
        H = H.conj().T.tocsr()
        SH = SH.conj().T.tocsr()
    if coarse == "rediscretize":
        hier = build_hierarchy_rediscretized(M, m, gamma, omega, shift, NeumannOnTop, Sommerfeld, levels, transpose)
    else:
        hier = build_hierarchy(SH, M, levels)
    B2 = np.asarray(B, dtype=np.complex128)
    vec = B2.ndim == 1
    if vec:
        B2 = B2[:, None]
    if krylov == "BiCGSTAB":
        res = bicgstab(lambda X: H @ X, lambda V: mg_cycle(hier, 0, V, relax_w, pre, post, cycle, relax_type,
                                                           gmres_from), B2, tol, max_outer)
    else:
        res = fgmres(lambda X: H @ X, lambda V: mg_cycle(hier, 0, V, relax_w, pre, post, cycle, relax_type,
                                                         gmres_from), B2, restart, tol, max_outer)
    X = res.X[:, 0] if vec else res.X
    return SLMGSolution(X=X, result=res, hier=hier)


def direct_solve(H: sp.csr_matrix, B: np.ndarray) -> np.ndarray:
    """Sparse LU solve H X = B, as test/HelmholtzTest.jl:42 does with H\\q."""
    lu = spla.splu(H.tocsc())
    return lu.solve(np.asarray(B, dtype=np.complex128))


# ---------------------------------------------------------------------------
# Seeded synthetic velocity models (the workloads the solver is measured on)
# ---------------------------------------------------------------------------
def model_gradient_ellipse(nodes, h):
    """2D: v = 1.5 + 3 z plus an ellipse v=4.5 at (0.5,0.6), semi-axes 0.15/0.08."""
    x = h[0] * np.arange(nodes[0])
    z = h[1] * np.arange(nodes[1])
    X, Z = np.meshgrid(x, z, indexing="ij")
    v = 1.5 + 3.0 * Z
    inside = ((X - 0.5) / 0.15) ** 2 + ((Z - 0.6) / 0.08) ** 2 <= 1.0
    v[inside] = 4.5
    return v


def model_layered(nodes, seed: int, nlayers: int = 12, vmin: float = 1.5, vmax: float = 4.5,
                  ellipsoid: bool = False):
    """Layered velocity (last axis = depth), layer thicknesses seeded, velocities
    uniform in [vmin, vmax] sorted to increase with depth; optional seeded
    ellipsoidal v=4.5 body.  Returns v with node shape."""
    rng = np.random.default_rng(seed)
    nodes = [int(v) for v in nodes]
    nz = nodes[-1]
    w = rng.uniform(0.5, 1.5, size=nlayers)
    bounds = np.concatenate([[0], np.cumsum(w) / np.sum(w) * nz]).astype(np.int64)
    bounds[-1] = nz
    vel = np.sort(rng.uniform(vmin, vmax, size=nlayers))
    vz = np.empty(nz)
    for k in range(nlayers):
        vz[bounds[k]:bounds[k + 1]] = vel[k]
    shape = tuple(nodes)
    v = np.broadcast_to(vz.reshape((1,) * (len(nodes) - 1) + (nz,)), shape).copy()
    if ellipsoid:
        grids = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in nodes], indexing="ij")
        c = rng.uniform(0.3, 0.7, size=len(nodes))
        ax = rng.uniform(0.08, 0.2, size=len(nodes))
        r = sum(((g - ci) / ai) ** 2 for g, ci, ai in zip(grids, c, ax))
        v[r <= 1.0] = 4.5
    return v
