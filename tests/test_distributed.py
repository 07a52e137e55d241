"""Column sharding across ranks (world size 2, gloo on CPU): partitioning,
per-rank solve of its slice, gather of X on rank 0."""
import os
import socket

import numpy as np
import pytest


def test_partition_columns(hz):
    from helmholtz_jl_gb300.distributed import partition_columns
    assert partition_columns(64, 8) == [(8 * r, 8 * r + 8) for r in range(8)]
    p = partition_columns(10, 3)
    assert p == [(0, 4), (4, 7), (7, 10)]
    assert partition_columns(1, 2) == [(0, 1), (1, 1)]
    with pytest.raises(ValueError):
        partition_columns(4, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q, ncols=7):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    import torch.distributed as dist
    import __graft_entry__ as ge
    ge.load_package()
    from helmholtz_jl_gb300.distributed import solve_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(5)
    B = rng.standard_normal((50, ncols)) + 1j * rng.standard_normal((50, ncols))
    seen = []

    def fake_solve(Bs):  # stands in for the per-rank GPU solve; records its slice
        seen.append(Bs.shape[1])
        return (2.0 - 1.0j) * Bs

    X = solve_sharded(fake_solve, B, dist)
    if rank == 0:
        q.put(("x", np.abs(X - (2.0 - 1.0j) * B).max()))
    q.put(("cols", rank, seen[0] if seen else 0))
    dist.barrier()
    dist.destroy_process_group()


def _run_all(procs, timeout=120.0):
    """Start the rank processes and wait for them; a rank still alive after the
    timeout is terminated (then killed) before the test fails, so no hung rank
    keeps its port or outlives the test."""
    import time
    for p in procs:
        p.start()
    deadline = time.monotonic() + timeout
    for p in procs:
        p.join(max(0.0, deadline - time.monotonic()))
    hung = [p for p in procs if p.is_alive()]
    for p in hung:
        p.terminate()
    for p in hung:
        p.join(5)
        if p.is_alive():
            p.kill()
            p.join(5)
    assert not hung, f"{len(hung)} rank(s) did not finish within {timeout} s"
    assert [p.exitcode for p in procs] == [0] * len(procs)


def test_solve_sharded_gloo_world2(hz):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    _run_all(procs)
    msgs = [q.get(timeout=10) for _ in range(3)]
    xs = [m for m in msgs if m[0] == "x"]
    assert xs and xs[0][1] == 0.0
    cols = sorted((m[1], m[2]) for m in msgs if m[0] == "cols")
    assert cols == [(0, 4), (1, 3)]


def test_solve_sharded_gloo_world3_empty_slice(hz):
    """Fewer columns than ranks: the rank with an empty slice does not call the
    solve, sends nothing that lands in X, and rank 0 still assembles every column."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 3, port, q, 2)) for r in range(3)]
    _run_all(procs)
    msgs = [q.get(timeout=10) for _ in range(4)]
    xs = [m for m in msgs if m[0] == "x"]
    assert xs and xs[0][1] == 0.0
    cols = sorted((m[1], m[2]) for m in msgs if m[0] == "cols")
    assert cols == [(0, 1), (1, 1), (2, 0)]


def _failing_worker(rank, world, port, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    import torch.distributed as dist
    import __graft_entry__ as ge
    ge.load_package()
    from helmholtz_jl_gb300.distributed import ShardFailed, solve_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    B = np.ones((20, 4), dtype=np.complex128)

    def solve(Bs):  # rank 1's solve fails on the host (no GPU fault involved)
        if rank == 1:
            raise ValueError("injected failure")
        return Bs

    try:
        solve_sharded(solve, B, dist)
        q.put((rank, "returned"))
    except ShardFailed:
        q.put((rank, "ShardFailed"))
    except ValueError as e:
        q.put((rank, f"ValueError: {e}"))
    dist.destroy_process_group()


def test_failed_rank_does_not_hang_the_others(hz):
    """A rank whose solve raises re-raises it; the others learn of it through the
    status all-reduce before the gather and raise ShardFailed instead of waiting."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_failing_worker, args=(r, 2, port, q)) for r in range(2)]
    _run_all(procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, "ShardFailed"), (1, "ValueError: injected failure")]
