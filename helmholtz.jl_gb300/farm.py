"""Multi-frequency / multi-shot farming over solver handles.

The caller of solveLinearSystem in an inversion (jInv's forward-problem
farming) solves many shots at several frequencies.  Here each frequency gets
one solver whose operator and multigrid hierarchy are built once and reused
for every batch of shots; batches bound the device memory (the FGMRES
workspace scales with the columns of a batch); a frequency's device memory is
released (clear!) before the next one is set up unless ``keep`` is set.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import api


@dataclass
class FarmResult:
    X: list                      # one n x nshots array per frequency
    setup_time: list = field(default_factory=list)
    solve_time: list = field(default_factory=list)
    relres: list = field(default_factory=list)
    iters: list = field(default_factory=list)


def solve_frequencies(params, B, MG, shift=0.5, Krylov: str = "GMRES", inner: int = 10, batch: int = 32,
                      doTranspose: int = 0, keep: bool = False) -> FarmResult:
    """Solve H(omega_k) X_k = B_k for every frequency k.

    params: list of HelmholtzParam (one per frequency; omega, gamma may differ).
    B: one n x nshots array shared by all frequencies, or a list of them.
    batch: shots per solve call (columns of one hz_solve)."""
    if not params:
        raise ValueError("no frequencies")
    Bs = B if isinstance(B, (list, tuple)) else [B] * len(params)
    if len(Bs) != len(params):
        raise ValueError("one right-hand-side block per frequency expected")
    if batch < 1:
        raise ValueError("batch must be >= 1")
    out = FarmResult(X=[])
    for p, Bk in zip(params, Bs):
        Bk = np.asarray(Bk, dtype=np.complex128)
        Bk = Bk.reshape(Bk.shape[0], -1)
        S = api.getShiftedLaplacianMultigridSolver(p, MG, shift, Krylov, inner)
        X = np.zeros_like(Bk)
        rr = np.zeros(Bk.shape[1])
        it = np.zeros(Bk.shape[1], dtype=np.int64)
        for a in range(0, Bk.shape[1], batch):
            b = min(a + batch, Bk.shape[1])
            Xb, S = api.solveLinearSystem(None, Bk[:, a:b], S, doTranspose)
            X[:, a:b] = np.reshape(Xb, (Bk.shape[0], b - a))
            if S.last_relres is not None:
                rr[a:b] = S.last_relres
                it[a:b] = S.last_iters
        out.X.append(X)
        out.setup_time.append(S.setupTime)
        out.solve_time.append(S.solveTime)
        out.relres.append(rr)
        out.iters.append(it)
        if not keep:
            api.clear_(S)
            api._release(S)
    return out
