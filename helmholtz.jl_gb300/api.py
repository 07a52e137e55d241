"""Host-side mirror of the Helmholtz.jl API for the shifted-Laplacian
multigrid path, running on the helmgpu CUDA library.

Names, argument order and semantics follow the reference so that code and
tests written against Helmholtz.jl read the same here:

* ``getRegularMesh``, ``HelmholtzParam``                       (jInv, src/Helmholtz.jl:13-20)
* ``getMaximalFrequency``, ``getABL``, ``getSommerfeldBC``,
  ``GetHelmholtzOperator``, ``GetHelmholtzShiftOP``,
  ``getHelmholtzFun``                                           (src/GetHelmholtz.jl)
* ``getMGparam``                                                (Multigrid.jl, positional form of
                                                                 test/ShiftedLaplacianTest.jl:63-64)
* ``getShiftedLaplacianMultigridSolver``, ``solveLinearSystem``,
  ``solveLinearSystemInPlace`` (jInv's ``solveLinearSystem!``),
  ``copySolver``, ``clear_`` (``clear!``)                       (src/ShiftedLaplacianMultigridSolver.jl)
* ``getAcousticPointSource``, ``getTopPointSrc``, ``loc2cs``    (src/getPointSource.jl:63-111)

Operators are matrix-free and live on the GPU; ``GetHelmholtzOperator``
returns an operator object (not a sparse matrix) whose products run the
library's stencil kernel.  Arrays are column-major node vectors (axis 1
fastest), as in the reference.  There is no CPU fallback: without the
compiled library or a GPU every compute call raises.
"""
from __future__ import annotations

import ctypes as C
import sys
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i64(vals):
    arr = (C.c_int64 * len(vals))(*[int(v) for v in vals])
    return arr


# ---------------------------------------------------------------------------
# Mesh and parameters
# ---------------------------------------------------------------------------
@dataclass
class RegularMesh:
    """jInv RegularMesh fields used on this path: domain, n (cells), h, dim."""
    domain: np.ndarray
    n: np.ndarray
    h: np.ndarray
    dim: int


def getRegularMesh(domain, n) -> RegularMesh:
    domain = np.asarray(domain, dtype=np.float64).ravel()
    n = np.asarray(n, dtype=np.int64).ravel()
    if domain.size != 2 * n.size:
        raise ValueError("domain needs two entries per axis")
    h = (domain[1::2] - domain[0::2]) / n
    return RegularMesh(domain=domain, n=n, h=h, dim=int(n.size))


@dataclass
class HelmholtzParam:
    """src/Helmholtz.jl:13-20."""
    Mesh: RegularMesh
    gamma: np.ndarray
    m: np.ndarray
    omega: complex | float
    NeumannOnTop: bool
    Sommerfeld: bool


def getShiftedHelmholtzParam(p: HelmholtzParam, s: float) -> HelmholtzParam:
    """src/Helmholtz.jl:32-34: gamma + s * Re(omega)."""
    return HelmholtzParam(p.Mesh, np.asarray(p.gamma) + s * complex(p.omega).real, p.m, p.omega, p.NeumannOnTop,
                          p.Sommerfeld)


def _nodes(M: RegularMesh):
    return [int(v) + 1 for v in M.n]


def _flat(a, N: int, name: str) -> np.ndarray:
    v = np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))
    if v.size != N:
        raise ValueError(f"{name} has {v.size} values, the mesh has {N} nodes")
    return v


# ---------------------------------------------------------------------------
# Discretisation helpers (host, through the C ABI)
# ---------------------------------------------------------------------------
def getMaximalFrequency(m, M: RegularMesh) -> float:
    """src/GetHelmholtz.jl:75-79 (10 points per wavelength)."""
    mm = np.ascontiguousarray(np.asarray(m, dtype=np.float64).ravel())
    h = np.ascontiguousarray(M.h, dtype=np.float64)
    return float(L.load().hz_max_frequency(_dp(mm), mm.size, _dp(h), M.dim))


def getABL(n, NeumannAtFirstDim: bool, ABLpad, ABLamp: float) -> np.ndarray:
    """src/GetHelmholtz.jl:97-220; n are node counts.  Returns gamma with node
    shape (Fortran order)."""
    n = [int(v) for v in np.ravel(n)]
    pad = [int(v) for v in np.ravel(ABLpad)]
    if len(pad) == 1:
        pad = pad * len(n)
    out = np.zeros(int(np.prod(n)), dtype=np.float64)
    L.check(L.load().hz_abl(len(n), _i64(n), int(bool(NeumannAtFirstDim)), _i64(pad), float(ABLamp), _dp(out)))
    return out.reshape(n, order="F")


def getSommerfeldBC(Msh: RegularMesh, mNodal, omega: float, NeumannOnTop: bool, orderNeumannBC: int = 2):
    """src/GetHelmholtz.jl:222-247."""
    nn = _nodes(Msh)
    N = int(np.prod(nn))
    m = _flat(mNodal, N, "m")
    out = np.zeros(2 * N, dtype=np.float64)
    h = np.ascontiguousarray(Msh.h, dtype=np.float64)
    L.check(L.load().hz_sommerfeld(Msh.dim, _i64(Msh.n), _dp(h), _dp(m), float(omega), int(bool(NeumannOnTop)),
                                   int(orderNeumannBC), _dp(out)))
    return out.view(np.complex128).reshape(nn, order="F")


def _problem(param: HelmholtzParam, orderNeumannBC: int = 2):
    M = param.Mesh
    N = int(np.prod(_nodes(M)))
    m = _flat(param.m, N, "m")
    g = _flat(param.gamma, N, "gamma")
    p = L.hz_problem()
    p.dim = M.dim
    for d in range(M.dim):
        p.n[d] = int(M.n[d])
        p.h[d] = float(M.h[d])
    w = complex(param.omega)
    p.omega_re, p.omega_im = w.real, w.imag
    p.m = _dp(m)
    p.gamma = _dp(g)
    p.neumann_on_top = int(bool(param.NeumannOnTop))
    p.sommerfeld = int(bool(param.Sommerfeld))
    p.order_neumann_bc = int(orderNeumannBC)
    return p, (m, g)  # keep the arrays alive with the struct


def helmholtz_mass(param: HelmholtzParam, orderNeumannBC: int = 2) -> np.ndarray:
    """Diagonal mass term of H (src/GetHelmholtz.jl:41-47)."""
    p, keep = _problem(param, orderNeumannBC)
    N = keep[0].size
    out = np.zeros(2 * N, dtype=np.float64)
    L.check(L.load().hz_helmholtz_mass(C.byref(p), _dp(out)))
    return out.view(np.complex128)


# ---------------------------------------------------------------------------
# Matrix-free operators
# ---------------------------------------------------------------------------
class _Device:
    """A helmgpu handle built for operator products (no hierarchy until a solve)."""

    def __init__(self, param: HelmholtzParam, shift: float, orderNeumannBC: int = 2, opts: L.hz_options | None = None):
        lib = L.load()
        p, self._keep = _problem(param, orderNeumannBC)
        o = opts if opts is not None else _default_options()
        o.shift = float(shift)
        h = C.c_void_p()
        L.check(lib.hz_create(C.byref(p), C.byref(o), C.byref(h)))
        self.handle = h
        self.N = self._keep[0].size
        self.shift = float(shift)

    def apply(self, op: int, adj: bool, X):
        return _apply(self, op, adj, X)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                L.load().hz_destroy(h)
            except Exception:
                pass
            self.handle = None


def current_device() -> int:
    """The CUDA device new handles are built on: the one this process selected
    with torch.cuda.set_device (one process per GPU under torchrun), or device 0
    when torch is not loaded or sees no GPU."""
    torch = sys.modules.get("torch")
    if torch is not None and torch.cuda.is_available():
        return int(torch.cuda.current_device())
    return 0


def _default_options() -> L.hz_options:
    o = L.hz_options()
    L.load().hz_default_options(C.byref(o))
    o.device = current_device()
    return o


def _is_device_array(x) -> bool:
    return hasattr(x, "data_ptr") and getattr(getattr(x, "device", None), "type", "cpu") == "cuda"


def _device_inputs_ready() -> None:
    """Make the work queued for the tensors handed to the library complete
    before the library reads them.  The library orders its own stream after the
    legacy default stream (torch's default stream); work queued on another
    current torch stream is waited for here."""
    import torch
    cur = torch.cuda.current_stream()
    if cur.cuda_stream != 0:
        cur.synchronize()


def _apply(dev: _Device, op: int, adj: bool, X):
    lib = L.load()
    if _is_device_array(X):
        import torch
        Xt = X if X.dim() == 2 else X.reshape(-1, 1)
        if Xt.dtype != torch.complex128:
            raise TypeError("device arrays must be complex128")
        # column-major n x nrhs: a (nrhs, n) row-major tensor has that layout
        Xc = Xt.t().contiguous()
        Yc = torch.empty_like(Xc)
        _device_inputs_ready()
        L.check(lib.hz_apply(dev.handle, op, int(adj), Xc.data_ptr(), Yc.data_ptr(), Xc.shape[1], Xc.shape[0],
                             L.HZ_MEM_DEVICE), dev.handle)
        Y = Yc.t()
        return Y if X.dim() == 2 else Y.reshape(-1)
    Xa = np.asarray(X, dtype=np.complex128)
    vec = Xa.ndim == 1
    X2 = Xa.reshape(-1, 1) if vec else Xa
    n, nrhs = X2.shape
    Xf = np.asfortranarray(X2)
    Yf = np.empty((n, nrhs), dtype=np.complex128, order="F")
    L.check(lib.hz_apply(dev.handle, op, int(adj), Xf.ctypes.data, Yf.ctypes.data, n, nrhs, L.HZ_MEM_HOST),
            dev.handle)
    return Yf[:, 0] if vec else Yf


class HelmholtzOperator:
    """Matrix-free A = base + i*sigma*w^2*diag(m) with base = H, H^H or nothing.

    ``GetHelmholtzOperator`` returns H (adj=False, sigma=0);
    ``GetHelmholtzShiftOP(m, w, s)`` returns the pure shift term (no base,
    sigma=s); their sum is SH; ``.H`` / ``adjoint()`` conjugate-transpose
    (adj flips, sigma changes sign).  ``A @ X`` runs the GPU stencil for H,
    H^H, SH and SH^H."""

    def __init__(self, param: HelmholtzParam | None, orderNeumannBC: int = 2, adj: bool = False,
                 sigma: float = 0.0, base: bool = True, devices: dict | None = None, m=None, omega=None):
        self.param = param
        self.orderNeumannBC = orderNeumannBC
        self.adj = bool(adj)
        self.sigma = float(sigma)
        self.base = bool(base)
        self._devices = devices if devices is not None else {}
        self._m = np.asarray(param.m if m is None else m, dtype=np.float64).ravel(order="F")
        self._omega = complex(param.omega if omega is None else omega)
        N = self._m.size
        self.shape = (N, N)

    def _with(self, **kw) -> "HelmholtzOperator":
        d = dict(param=self.param, orderNeumannBC=self.orderNeumannBC, adj=self.adj, sigma=self.sigma,
                 base=self.base, devices=self._devices, m=self._m, omega=self._omega)
        d.update(kw)
        return HelmholtzOperator(**d)

    def adjoint(self) -> "HelmholtzOperator":
        return self._with(adj=not self.adj, sigma=-self.sigma)

    @property
    def H(self) -> "HelmholtzOperator":
        return self.adjoint()

    def __add__(self, other):
        if not isinstance(other, HelmholtzOperator):
            return NotImplemented
        if self.base and other.base:
            raise ValueError("the sum of two Helmholtz operators is not built")
        if not np.array_equal(self._m, other._m) or self._omega.real != other._omega.real:
            raise ValueError("operators built from a different m or omega")
        if self.base or other.base:
            b = self if self.base else other
            return b._with(sigma=self.sigma + other.sigma)
        return self._with(sigma=self.sigma + other.sigma)

    __radd__ = __add__

    def __neg__(self):
        if self.base:
            raise ValueError("only the shift term can be negated")
        return self._with(sigma=-self.sigma)

    def _device(self, shift: float) -> _Device:
        key = round(shift, 15)
        dev = self._devices.get(key)
        if dev is None:
            dev = _Device(self.param, shift, self.orderNeumannBC)
            self._devices[key] = dev
        return dev

    def __matmul__(self, X):
        if not self.base or self.param is None:
            raise TypeError("the shift term alone is not applied on the device; add it to H")
        if self.sigma == 0.0:  # H or H^H: the handle's shift does not enter
            dev = next(iter(self._devices.values()), None) or self._device(0.5)
            return dev.apply(L.HZ_OP_H, self.adj, X)
        s = -self.sigma if self.adj else self.sigma   # SH has sigma=s, SH^H has sigma=-s
        return self._device(s).apply(L.HZ_OP_SH, self.adj, X)

    def diagonal_shift(self) -> np.ndarray:
        return self._m * (1j * self.sigma * self._omega.real ** 2)


def GetHelmholtzOperator(*args, **kw):
    """Three methods of src/GetHelmholtz.jl:
    (Hparam, orderNeumannBC=2) -> H
    (Msh, m, omega, gamma, NeumannAtFirstDim, ABLpad, ABLamp, Sommerfeld, orderNeumannBC=2) -> (H, gamma)
    (Msh, m, omega, gamma, NeumannAtFirstDim, Sommerfeld, orderNeumannBC=2) -> H
    """
    if isinstance(args[0], HelmholtzParam):
        order = args[1] if len(args) > 1 else kw.get("orderNeumannBC", 2)
        return HelmholtzOperator(args[0], order)
    Msh, m, omega, gamma, neumann = args[:5]
    rest = args[5:]
    if len(rest) >= 3 and not isinstance(rest[0], (bool, np.bool_)):
        pad, amp, somm = rest[0], rest[1], rest[2]
        order = rest[3] if len(rest) > 3 else kw.get("orderNeumannBC", 2)
        abl = getABL(_nodes(Msh), neumann, pad, amp)
        if gamma is None or np.size(gamma) == 0:
            g = abl
        else:
            g = np.reshape(np.asarray(gamma, dtype=np.float64), abl.shape, order="F") + abl
        p = HelmholtzParam(Msh, g, np.asarray(m, dtype=np.float64), omega, bool(neumann), bool(somm))
        return HelmholtzOperator(p, order), g
    somm = rest[0]
    order = rest[1] if len(rest) > 1 else kw.get("orderNeumannBC", 2)
    p = HelmholtzParam(Msh, np.asarray(gamma, dtype=np.float64), np.asarray(m, dtype=np.float64), omega,
                       bool(neumann), bool(somm))
    return HelmholtzOperator(p, order)


def GetHelmholtzShiftOP(mNodal, omega: float, shift: float) -> HelmholtzOperator:
    """src/GetHelmholtz.jl:81-83: the shift term diag(i*shift*w^2*m); add it to
    a Helmholtz operator of the same problem to get SH."""
    return HelmholtzOperator(None, 2, False, float(shift), base=False, m=mNodal, omega=float(omega))


def getHelmholtzFun(ShiftedHelmholtT: HelmholtzOperator, ShiftMat: HelmholtzOperator, y=None, numCores: int = 1):
    """src/GetHelmholtz.jl:85-95: x -> ShiftedHT' x + ShiftMat' x, i.e. H x
    (or H^H x for the transposed pair), evaluated by the GPU stencil."""
    if ShiftMat.base:
        raise ValueError("ShiftMat must be a shift term (GetHelmholtzShiftOP)")
    total = ShiftedHelmholtT.adjoint() + ShiftMat.adjoint()

    def Hfun(x):
        return total @ x

    return Hfun


# ---------------------------------------------------------------------------
# Multigrid parameters and the SLMG solver
# ---------------------------------------------------------------------------
@dataclass
class MGparam:
    """The in-scope subset of Multigrid.jl's MGparam."""
    levels: int
    numCores: int
    maxOuterIter: int
    relativeTol: float
    relaxType: str
    relaxParam: float
    relaxPre: int
    relaxPost: int
    cycleType: str
    coarseSolveType: str
    low: float = 0.5
    high: float = 0.0
    transferType: str = "FullWeighting"
    precision: str = "fp64"  # "fp64" or "mixed" (complex-FP32 cycle)
    coarseOperator: str = "Galerkin"  # or "Rediscretize" (src/ShiftedLaplacianMultigridSolver.jl:51-62)
    outerArithmetic: str = "fp64"     # or "emulated": FP64 emulated with FP32 pairs (mixed form, FGMRES)
    cudaGraph: bool = True            # replay the FGMRES preconditioner applications from CUDA graphs
    autotune: bool = True             # time the stencils' launch shapes at the first solve
    relaxFrom: int = 0                # "Jac-GMRES": first level smoothed by GMRES steps (finer: "Jac")
    doTranspose: int = 0
    _hier: dict = field(default_factory=dict, repr=False)


_SUPPORTED_COARSE = {"Julia", "MUMPS", "NoMUMPS", "BandLU"}


def getMGparam(*args, transferType: str | None = None, precision: str = "fp64",
               coarseOperator: str = "Galerkin", outerArithmetic: str = "fp64", relaxFrom: int = 0) -> MGparam:
    """Positional forms of Multigrid.jl getMGparam:
    (TYPE, ITYPE, levels, numCores, maxIter, relativeTol, relaxType, relaxParam,
     relaxPre, relaxPost, cycleType, coarseSolveType[, low, high[, transferType]])
    or the same without the leading TYPE, ITYPE."""
    a = list(args)
    if a and isinstance(a[0], type):
        a = a[2:]
    if len(a) < 10:
        raise TypeError("getMGparam needs levels, numCores, maxIter, relativeTol, relaxType, relaxParam, "
                        "relaxPre, relaxPost, cycleType, coarseSolveType")
    (levels, numCores, maxIter, tol, relaxType, relaxParam, pre, post, cycle, coarse) = a[:10]
    low = a[10] if len(a) > 10 else 0.5
    high = a[11] if len(a) > 11 else 0.0
    tt = a[12] if len(a) > 12 else (transferType or "FullWeighting")
    mg = MGparam(int(levels), int(numCores), int(maxIter), float(tol), str(relaxType), float(relaxParam), pre, post,
                 str(cycle), str(coarse), float(low), float(high), str(tt), precision, coarseOperator,
                 outerArithmetic)
    mg.relaxFrom = int(relaxFrom)
    return mg


def _validate_mg(MG: MGparam):
    if MG.relaxType not in ("Jac", "Jac-GMRES"):
        raise NotImplementedError(f"relaxType {MG.relaxType!r}: damped Jacobi ('Jac') and 'Jac-GMRES' are built")
    if MG.cycleType not in ("V", "W", "K"):
        raise NotImplementedError(f"cycleType {MG.cycleType!r}: only 'V', 'W' and 'K' cycles are built")
    if MG.coarseSolveType not in _SUPPORTED_COARSE:
        raise NotImplementedError(f"coarseSolveType {MG.coarseSolveType!r} is not built (direct band LU only)")
    if MG.transferType != "FullWeighting":
        raise NotImplementedError(f"transferType {MG.transferType!r}: only full weighting is built")
    if callable(MG.relaxPre) or callable(MG.relaxPost):
        raise NotImplementedError("level-dependent relaxation counts are not built")
    if MG.precision not in ("fp64", "mixed"):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    if MG.coarseOperator not in ("Galerkin", "Rediscretize"):
        raise ValueError("coarseOperator must be 'Galerkin' or 'Rediscretize'")
    if MG.outerArithmetic not in ("fp64", "emulated"):
        raise ValueError("outerArithmetic must be 'fp64' or 'emulated'")


@dataclass
class ShiftedLaplacianMultigridSolver:
    """src/ShiftedLaplacianMultigridSolver.jl:4-15."""
    helmParam: HelmholtzParam
    MG: MGparam
    shift: np.ndarray
    Krylov: str
    inner: int
    doClear: int
    verbose: bool
    setupTime: float = 0.0
    nPrec: int = 0
    solveTime: float = 0.0
    _handle: object = field(default=None, repr=False)
    _key: tuple = field(default=(), repr=False)
    _device: int = field(default=0, repr=False)  # CUDA device of _handle
    last_stats: object = field(default=None, repr=False)
    last_relres: np.ndarray | None = field(default=None, repr=False)
    last_iters: np.ndarray | None = field(default=None, repr=False)
    learned: object = field(default=None, repr=False)  # (CoarseNet, level, stag_ratio): learned.attach

    def __del__(self):
        _release(self)


def _release(s: ShiftedLaplacianMultigridSolver):
    h = getattr(s, "_handle", None)
    if h is not None and h.value:
        try:
            L.load().hz_destroy(h)
        except Exception:
            pass
    s._handle = None


def getShiftedLaplacianMultigridSolver(helmParam: HelmholtzParam, MG: MGparam, shift, Krylov: str = "BiCGSTAB",
                                       inner: int = 5, verbose: bool = False) -> ShiftedLaplacianMultigridSolver:
    """src/ShiftedLaplacianMultigridSolver.jl:24-30 (scalar shift broadcast to every level)."""
    if np.isscalar(shift):
        shift = np.ones(MG.levels) * float(shift)
    return ShiftedLaplacianMultigridSolver(helmParam, MG, np.asarray(shift, dtype=np.float64), Krylov, int(inner), 0,
                                           bool(verbose))


def copySolver(s: ShiftedLaplacianMultigridSolver) -> ShiftedLaplacianMultigridSolver:
    """src/ShiftedLaplacianMultigridSolver.jl:18-22: a fresh solver, same parameters, no hierarchy."""
    mg = MGparam(**{k: getattr(s.MG, k) for k in s.MG.__dataclass_fields__ if k != "_hier"})
    return getShiftedLaplacianMultigridSolver(s.helmParam, mg, s.shift.copy(), s.Krylov, s.inner, s.verbose)


def clear_(s: ShiftedLaplacianMultigridSolver) -> None:
    """clear! (src/ShiftedLaplacianMultigridSolver.jl:105-109): drop the hierarchy."""
    if s._handle is not None:
        L.check(L.load().hz_clear(s._handle), s._handle)
    s.doClear = 0


def _options(s: ShiftedLaplacianMultigridSolver) -> L.hz_options:
    MG = s.MG
    o = _default_options()
    o.levels = MG.levels
    o.max_outer = MG.maxOuterIter
    o.rel_tol = MG.relativeTol
    o.relax_pre = int(MG.relaxPre)
    o.relax_post = int(MG.relaxPost)
    o.relax_param = MG.relaxParam
    o.cycle = ord(MG.cycleType)
    o.krylov = L.HZ_KRYLOV_BICGSTAB if s.Krylov == "BiCGSTAB" else L.HZ_KRYLOV_FGMRES
    o.inner = s.inner
    o.shift = float(s.shift[0])
    o.precision = L.HZ_PREC_MIXED if MG.precision == "mixed" else L.HZ_PREC_FP64
    o.coarse_op = L.HZ_COARSE_REDISCRETIZE if MG.coarseOperator == "Rediscretize" else L.HZ_COARSE_GALERKIN
    o.outer_arith = L.HZ_OUTER_EMULATED if MG.outerArithmetic == "emulated" else L.HZ_OUTER_FP64
    o.cuda_graph = int(bool(MG.cudaGraph))
    o.autotune = int(bool(MG.autotune))
    o.relax_type = L.HZ_RELAX_JAC_GMRES if MG.relaxType == "Jac-GMRES" else L.HZ_RELAX_JAC
    o.relax_from = int(MG.relaxFrom)
    o.verbose = int(bool(s.verbose))
    return o


def _ensure_handle(s: ShiftedLaplacianMultigridSolver):
    _validate_mg(s.MG)
    if s.Krylov not in ("GMRES", "BiCGSTAB"):
        raise NotImplementedError(f"Krylov {s.Krylov!r}: FGMRES ('GMRES') and 'BiCGSTAB' are built")
    if not np.all(s.shift == s.shift[0]):
        raise NotImplementedError("level-dependent shifts are not built")
    dev = current_device()
    key = (dev, id(s.helmParam), id(s.helmParam.m), id(s.helmParam.gamma), s.MG.levels, s.MG.maxOuterIter,
           s.MG.relativeTol, s.MG.relaxParam, int(s.MG.relaxPre), int(s.MG.relaxPost), s.MG.cycleType,
           s.MG.precision, s.inner, float(s.shift[0]), s.Krylov, s.MG.coarseOperator, s.MG.outerArithmetic,
           bool(s.MG.cudaGraph), bool(s.MG.autotune), s.MG.relaxType, int(s.MG.relaxFrom))
    if s._handle is not None and s._key == key:
        return s._handle
    _release(s)
    p, keep = _problem(s.helmParam)
    o = _options(s)
    h = C.c_void_p()
    L.check(L.load().hz_create(C.byref(p), C.byref(o), C.byref(h)))
    s._handle = h
    s._key = key
    s._device = int(o.device)
    if s.learned is not None:
        from .learned import _apply
        _apply(s)
    return h


def solveLinearSystem(ShiftedHT, B, param: ShiftedLaplacianMultigridSolver, doTranspose: int = 0):
    """src/ShiftedLaplacianMultigridSolver.jl:33-102.  Returns (X, param).

    ShiftedHT is the adjoint of the shifted operator as in the reference; its
    values are not read (the library rebuilds the operator matrix-free from
    helmParam) but its size is checked.  A one-column B comes back as a
    vector, an all-zero B returns zeros."""
    lib = L.load()
    on_device = _is_device_array(B)
    if on_device:
        import torch
        Bt = B if B.dim() == 2 else B.reshape(-1, 1)
        n, nrhs = Bt.shape
    else:
        Ba = np.asarray(B)
        if Ba.ndim == 2 and Ba.shape[1] == 1:
            Ba = Ba[:, 0]
        Bc = Ba.astype(np.complex128, copy=False)
        B2 = Bc.reshape(-1, 1) if Bc.ndim == 1 else Bc
        n, nrhs = B2.shape
    N = int(np.prod(_nodes(param.helmParam.Mesh)))
    if n != N:
        raise ValueError(f"B has {n} rows, the mesh has {N} nodes")
    if ShiftedHT is not None and hasattr(ShiftedHT, "shape") and tuple(ShiftedHT.shape) != (N, N):
        raise ValueError("ShiftedHT has the wrong size")
    if param.doClear == 1:
        clear_(param)
    zero = float(torch.linalg.vector_norm(Bt)) == 0.0 if on_device else np.linalg.norm(B2) == 0.0
    if zero:
        # zero solution, zero residual: the per-column results describe this call, not an earlier one
        param.last_relres = np.zeros(nrhs)
        param.last_iters = np.zeros(nrhs, dtype=np.int32)
        return (torch.zeros_like(B) if on_device else np.zeros_like(Bc)), param
    h = _ensure_handle(param)
    st = L.hz_stats()
    if on_device:
        Bc_ = Bt.t().contiguous()
        Xc_ = torch.empty_like(Bc_)
        _device_inputs_ready()
        code = lib.hz_solve(h, Bc_.data_ptr(), Xc_.data_ptr(), n, nrhs, int(doTranspose), L.HZ_MEM_DEVICE,
                            C.byref(st))
        L.check(code, h)
        X = Xc_.t()
        X = X if B.dim() == 2 else X.reshape(-1)
    else:
        Bf = np.asfortranarray(B2)
        Xf = np.empty((n, nrhs), dtype=np.complex128, order="F")
        code = lib.hz_solve(h, Bf.ctypes.data, Xf.ctypes.data, n, nrhs, int(doTranspose), L.HZ_MEM_HOST,
                            C.byref(st))
        L.check(code, h)
        X = Xf[:, 0] if Bc.ndim == 1 else Xf
    rr = np.zeros(nrhs)
    it = np.zeros(nrhs, dtype=np.int32)
    lib.hz_column_stats(h, _dp(rr), it.ctypes.data_as(C.POINTER(C.c_int32)), nrhs)
    param.setupTime = st.setup_time
    param.solveTime = st.solve_time
    param.nPrec += int(st.outer)
    param.MG.doTranspose = int(doTranspose)
    param.last_stats = st
    param.last_relres = rr
    param.last_iters = it
    if code == L.HZ_NOT_CONVERGED:
        print("WARNING: MG solver reached maximum iterations without convergence")
    return X, param


def solveLinearSystemInPlace(A, B, X, param: ShiftedLaplacianMultigridSolver, doTranspose: int = 0):
    """jInv's solveLinearSystem!(A, B, X, param, doTranspose): X is overwritten."""
    Y, param = solveLinearSystem(A, B, param, doTranspose)
    if _is_device_array(X):
        X.copy_(Y.reshape(X.shape))
    else:
        X[...] = np.reshape(Y, X.shape)
    return X, param


# ---------------------------------------------------------------------------
# Point sources (src/getPointSource.jl:63-111)
# ---------------------------------------------------------------------------
def getTopPointSrc(M: RegularMesh):
    if M.dim == 3:
        return [(int(M.n[0]) + 1) // 2, (int(M.n[1]) + 1) // 2, 1]
    return [(int(M.n[0]) + 1) // 2, 1]


def getMidPointSrc(M: RegularMesh):
    return [(int(v) + 1) // 2 for v in M.n]


def loc2cs(n, sub) -> int:
    n = [int(v) for v in n]
    cs = int(sub[0]) + (int(sub[1]) - 1) * n[0]
    if len(sub) == 3:
        cs += (int(sub[2]) - 1) * n[0] * n[1]
    return cs


def getAcousticPointSource(M: RegularMesh, TYPE=np.complex128, src=None):
    """q[src] = 1/||h||^2; returns (q with node shape, src)."""
    if src is None:
        src = getTopPointSrc(M)
    nn = _nodes(M)
    out = np.zeros(2 * int(np.prod(nn)), dtype=np.float64)
    h = np.ascontiguousarray(M.h, dtype=np.float64)
    L.check(L.load().hz_point_source(M.dim, _i64(M.n), _dp(h), _i64(src), _dp(out)))
    q = out.view(np.complex128).reshape(nn, order="F").astype(TYPE)
    return q, list(src)
