"""Right-hand-side sharding across GPUs (one process per GPU).

The columns of B are independent, so N ranks each solve a contiguous slice
of the columns with their own replica of the operator and hierarchy.  The
only communication is one status flag per solve (so that a failed rank stops
the others instead of leaving them in the gather) and the host-side gather of
X; no collective touches the data path.  Works with any torch.distributed
backend (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import numpy as np


def partition_columns(ncols: int, world: int) -> list[tuple[int, int]]:
    """Contiguous, balanced [start, stop) column ranges, one per rank (the
    first ncols % world ranks get one extra column)."""
    if ncols < 0 or world < 1:
        raise ValueError("ncols >= 0 and world >= 1 required")
    base, extra = divmod(ncols, world)
    out, start = [], 0
    for r in range(world):
        stop = start + base + (1 if r < extra else 0)
        out.append((start, stop))
        start = stop
    return out


def gather_columns(X_local: np.ndarray, ncols: int, dist, group=None) -> np.ndarray | None:
    """Gather every rank's solved columns into the full n x ncols block on
    rank 0 (None elsewhere).  X_local is n x (its slice width), complex128."""
    import torch
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = partition_columns(ncols, world)
    n = X_local.shape[0]
    width = max(b - a for a, b in parts)
    buf = np.zeros((n, width), dtype=np.complex128)
    buf[:, : X_local.shape[1]] = X_local
    t = torch.from_numpy(np.ascontiguousarray(buf).view(np.float64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    gathered = [torch.empty_like(t) for _ in range(world)] if rank == 0 else None
    dist.gather(t, gathered, dst=0, group=group)
    if rank != 0:
        return None
    X = np.zeros((n, ncols), dtype=np.complex128)
    for r, (a, b) in enumerate(parts):
        blk = gathered[r].cpu().numpy().view(np.complex128)
        X[:, a:b] = blk[:, : b - a]
    return X


class ShardFailed(RuntimeError):
    """Another rank's solve failed; this rank's slice was solved but not gathered."""


def solve_sharded(solve, B: np.ndarray, dist, group=None) -> np.ndarray | None:
    """Solve the columns of B across the ranks of `group`: each rank calls
    solve(B[:, its slice]) (normally solveLinearSystem on its own GPU) and
    rank 0 returns the gathered solution.

    Before the gather every rank reports whether its solve succeeded (one
    all-reduce of a status flag), so a failed rank does not leave the others
    waiting in the gather: it re-raises its own exception and every other rank
    raises ShardFailed."""
    import torch
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    a, b = partition_columns(B.shape[1], world)[rank]
    err = None
    try:
        X_local = solve(B[:, a:b]) if b > a else np.zeros((B.shape[0], 0), dtype=np.complex128)
        X_local = np.asarray(X_local, dtype=np.complex128).reshape(B.shape[0], b - a)
    except Exception as e:  # reported to every rank below, then re-raised here
        err = e
        X_local = None
    flag = torch.tensor([0.0 if err is None else 1.0], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        flag = flag.cuda()
    dist.all_reduce(flag, op=dist.ReduceOp.MAX, group=group)
    if err is not None:
        raise err
    if float(flag.item()) > 0.0:
        raise ShardFailed("column sharding: another rank's solve failed")
    return gather_columns(X_local, B.shape[1], dist, group)
