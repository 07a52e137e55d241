"""ctypes wrapper of the C oracle (oracle/slmg_cpu.c).

TEST INFRASTRUCTURE ONLY (checker and CPU baseline).  The hierarchy
(Galerkin A_l, prolongation P_l, restriction R_l) is assembled by
oracle/helmholtz_oracle.py with SciPy; the FGMRES + multigrid solve runs in
threaded C (OpenMP), as the reference's ParSpMatVec products do.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

import build_oracle
import helmholtz_oracle as O

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = C.CDLL(str(path))
        _lib.slmg_create.restype = C.c_void_p
        _lib.slmg_create.argtypes = [C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_void_p)]
        _lib.slmg_destroy.argtypes = [C.c_void_p]
        _lib.slmg_threads.restype = C.c_int
        _lib.slmg_solve.restype = C.c_int
        _lib.slmg_solve.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    return _lib


def _csr(M):
    M = sp.csr_matrix(M)
    M.sort_indices()
    return (np.ascontiguousarray(M.indptr, dtype=np.int64), np.ascontiguousarray(M.indices, dtype=np.int64),
            np.ascontiguousarray(M.data, dtype=np.complex128), M.shape)


@dataclass
class CpuSolveResult:
    X: np.ndarray
    iters: np.ndarray
    relres: np.ndarray
    outer: int
    setup_s: float
    solve_s: float
    threads: int


class CpuSLMG:
    """Plain FP64 SLMG on the CPU: hierarchy from SciPy, solve in threaded C."""

    def __init__(self, H, SH, M, levels: int, hier=None):
        """hier: a prebuilt hierarchy (e.g. O.build_hierarchy_rediscretized);
        by default the Galerkin hierarchy of SH."""
        t0 = time.perf_counter()
        self.hier = O.build_hierarchy(SH, M, levels) if hier is None else hier
        levels = len(self.hier.levels)
        self.H = _csr(H)
        mats = []
        for l, L in enumerate(self.hier.levels):
            mats.append(_csr(L.A))
            if l < levels - 1:
                mats.append(_csr(L.P))
                mats.append(_csr(L.R))
            else:
                mats += [None, None]
        self._mats = mats  # keep alive
        nslot = 3 * levels
        meta = (C.c_int64 * (2 * nslot))()
        ip = (C.c_void_p * nslot)()
        ix = (C.c_void_p * nslot)()
        dt = (C.c_void_p * nslot)()
        for s, mt in enumerate(mats):
            if mt is None:
                continue
            meta[2 * s], meta[2 * s + 1] = mt[3]
            ip[s] = mt[0].ctypes.data
            ix[s] = mt[1].ctypes.data
            dt[s] = mt[2].ctypes.data
        self.h = lib().slmg_create(levels, meta, ip, ix, dt)
        if not self.h:
            raise RuntimeError("C oracle setup failed")
        self.setup_s = time.perf_counter() - t0

    def solve(self, B, restart=10, tol=1e-8, max_outer=50, w=0.8, pre=1, post=1, cycle="V",
              relax="Jac", gmres_from=0, X0=None) -> CpuSolveResult:
        """relax: "Jac" (damped Jacobi sweeps) or "Jac-GMRES" (pre / post GMRES steps, at most 64,
        on the levels >= gmres_from; finer levels keep damped Jacobi).  X0: initial guess
        (default zero); continuing a restarted solve from its last X over several calls
        takes the same iterates as one call with the summed max_outer."""
        B2 = np.asfortranarray(np.asarray(B, dtype=np.complex128).reshape(B.shape[0], -1))
        n, nrhs = B2.shape
        if X0 is None:
            X = np.zeros((n, nrhs), dtype=np.complex128, order="F")
        else:
            X = np.array(np.asarray(X0, dtype=np.complex128).reshape(n, nrhs), order="F", copy=True)
        it = np.zeros(nrhs, dtype=np.int32)
        rr = np.zeros(nrhs, dtype=np.float64)
        hp, hi, hd, _ = self.H
        t0 = time.perf_counter()
        outer = lib().slmg_solve(self.h, n, hp.ctypes.data, hi.ctypes.data, hd.ctypes.data, B2.ctypes.data,
                                 X.ctypes.data, nrhs, restart, tol, max_outer, w, pre, post, {"V": 0, "W": 1, "K": 2}[cycle],
                                 {"Jac": 0, "Jac-GMRES": 1}[relax], int(gmres_from), it.ctypes.data,
                                 rr.ctypes.data, int(X0 is not None))
        if outer < 0:
            raise ValueError("Jac-GMRES takes at most 64 steps per smoothing")
        dt = time.perf_counter() - t0
        return CpuSolveResult(X=X, iters=it, relres=rr, outer=outer, setup_s=self.setup_s, solve_s=dt,
                              threads=lib().slmg_threads())

    def __del__(self):
        if getattr(self, "h", None):
            lib().slmg_destroy(self.h)
            self.h = None
