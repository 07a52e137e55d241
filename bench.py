"""Throughput benchmark: right-hand sides solved per second to relative
residual 1e-6 by the shifted-Laplacian multigrid FGMRES solve on one GB300.

One step = one hz_solve of the whole right-hand-side block of the workload
(every column to rel. residual <= tol).  The headline arm runs the
complex-FP32 V-cycle inside the FP64 FGMRES ("mixed"); the plain FP64 form of
the same solver is timed in the same process for the ratio the metric names.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c1|c2|c3|c4|c5]
  python bench.py --impl reference ...   # CPU reference path (C oracle, all host threads)

Under torchrun each rank solves its own seeded block of right-hand sides
(no data-path collective; weak scaling), timing is max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RHS solved/s to rel. residual 1e-6 on 1 GB300: learned+mixed vs plain FP64 SLMG"

# Synthetic seeded workloads (shapes, sizes and value distributions of the
# measured configurations; no external dataset is needed).
WORKLOADS = {
    # 2D 129 x 129 on [0,1]^2, v = 1.5 + 3 z with the v = 4.5 ellipse, one source
    # at (0.5, 2h), absorbing layer 16, 3 levels, FGMRES(10) to 1e-8
    "c1": dict(name="2D 129x129 gradient+ellipse, 1 source, 3 levels, FGMRES(10) tol 1e-8",
               cells=(128, 128), h=1.0 / 128, nrhs=1, levels=3, pad=16, ellipsoid=False, tol=1e-8,
               model="gradient_ellipse"),
    # 2D 1025 x 513 nodes, h = 10 m, 12 seeded layers in [1.5, 4.5] km/s,
    # absorbing layer 32 cells, 64 sources along the surface row, 5 levels
    "c2": dict(name="2D 1025x513 layered, 64 surface sources, 5 levels, FGMRES(10) tol 1e-6",
               cells=(1024, 512), h=0.010, nrhs=64, levels=5, pad=32, ellipsoid=False, tol=1e-6),
    # 3D 129^3 nodes layered + ellipsoid, absorbing layer 12, 4x4 surface sources, 4 levels
    "c3": dict(name="3D 129^3 layered+ellipsoid, 16 surface sources, 4 levels, FGMRES(10) tol 1e-6",
               cells=(128, 128, 128), h=0.010, nrhs=16, levels=4, pad=12, ellipsoid=True, tol=1e-6),
    # 2D 513 x 513 layered + inclusion models, learned coarse correction below level 2: trained on
    # pairs from seeded training models, evaluated on held-out seeds x 32 random-position sources
    "c4": dict(name="2D 513x513 layered+inclusion, learned coarse correction below level 2, 32 random sources, "
                    "5 levels, FGMRES(10) tol 1e-6",
               cells=(512, 512), h=0.010, nrhs=32, levels=5, pad=32, ellipsoid=True, tol=1e-6, learned=True,
               net_level=2),
    # 3D 257^3 nodes (16,974,593 unknowns per RHS), absorbing layer 16, 32 surface sources
    "c5": dict(name="3D 257^3 layered+ellipsoid, 32 surface sources, 5 levels, FGMRES(10) tol 1e-6",
               cells=(256, 256, 256), h=0.010, nrhs=32, levels=5, pad=16, ellipsoid=True, tol=1e-6),
}


def workload(args) -> dict:
    """The chosen workload with the command line's overrides (RHS count, level count)."""
    wl = dict(WORKLOADS[args.workload])
    if args.nrhs > 0:
        wl["nrhs"] = args.nrhs
    if args.levels > 0:
        wl["levels"] = args.levels
    return wl


def make_problem(wl: dict, seed: int):
    """Seeded layered (+ ellipsoid) velocity model, 10 points per wavelength,
    attenuation 0.01 w plus a quadratic absorbing layer of amplitude 0.95 w."""
    cells = wl["cells"]
    dim = len(cells)
    nodes = [c + 1 for c in cells]
    if wl.get("model") == "gradient_ellipse":
        h = np.full(dim, wl["h"])
        X, Z = np.meshgrid(h[0] * np.arange(nodes[0]), h[1] * np.arange(nodes[1]), indexing="ij")
        v = 1.5 + 3.0 * Z
        v[((X - 0.5) / 0.15) ** 2 + ((Z - 0.6) / 0.08) ** 2 <= 1.0] = 4.5
        m = (1.0 / v**2).ravel(order="F")
        w = (0.1 * 2 * np.pi) / (h.max() * np.sqrt(m.max()))
        return dict(dim=dim, cells=cells, nodes=nodes, h=h, m=m, w=w)
    rng = np.random.default_rng(seed)
    # layered model with depth along the last axis
    nl = 12
    wts = rng.uniform(0.5, 1.5, size=nl)
    bounds = np.concatenate([[0], np.cumsum(wts) / np.sum(wts) * nodes[-1]]).astype(np.int64)
    bounds[-1] = nodes[-1]
    vel = np.sort(rng.uniform(1.5, 4.5, size=nl))
    vz = np.empty(nodes[-1])
    for k in range(nl):
        vz[bounds[k]:bounds[k + 1]] = vel[k]
    v = np.broadcast_to(vz.reshape((1,) * (dim - 1) + (nodes[-1],)), nodes).copy()
    if wl["ellipsoid"]:
        c = rng.uniform(0.3, 0.7, size=dim)
        ax = rng.uniform(0.08, 0.2, size=dim)
        grids = np.ogrid[tuple(slice(0, n) for n in nodes)]
        r = sum(((g / (n - 1) - ci) / ai) ** 2 for g, n, ci, ai in zip(grids, nodes, c, ax))
        v[r <= 1.0] = 4.5
    m = (1.0 / v**2).ravel(order="F")
    h = np.full(dim, wl["h"])
    w = (0.1 * 2 * np.pi) / (h.max() * np.sqrt(m.max()))
    return dict(dim=dim, cells=cells, nodes=nodes, h=h, m=m, w=w)


def sources(P: dict, nrhs: int, seed: int) -> np.ndarray:
    """Delta sources q = 1/||h||^2 on the surface (depth index 1): evenly spaced
    along the surface row in 2D, on a square grid of the surface in 3D."""
    nodes = P["nodes"]
    N = int(np.prod(nodes))
    B = np.zeros((N, nrhs), dtype=np.complex128, order="F")
    amp = 1.0 / float(np.linalg.norm(P["h"])) ** 2
    if P["dim"] == 2 and nrhs == 1:
        B[(nodes[0] - 1) // 2 + nodes[0] * 2, 0] = amp  # (0.5, 2h)
    elif P["dim"] == 2:
        xs = np.linspace(nodes[0] * 0.05, nodes[0] * 0.95, nrhs).astype(np.int64)
        for c in range(nrhs):
            B[int(xs[c]) + nodes[0] * 1, c] = amp
    else:
        k = int(np.ceil(np.sqrt(nrhs)))
        g0 = np.linspace(nodes[0] * 0.2, nodes[0] * 0.8, k).astype(np.int64)
        g1 = np.linspace(nodes[1] * 0.2, nodes[1] * 0.8, k).astype(np.int64)
        shift = seed % 3
        for c in range(nrhs):
            i, j = int(g0[c % k]) + shift, int(g1[c // k])
            B[i + nodes[0] * (j + nodes[1] * 1), c] = amp
    return B


def gamma_of(P: dict, pad: int, lib, hz) -> np.ndarray:
    abl = hz.getABL(P["nodes"], True, [pad] * P["dim"], 0.95 * P["w"]).ravel(order="F")
    return abl + 0.01 * P["w"]


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, device: int = 0):
        self.samples = []
        self.proc = None
        self.device = device

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        return rank, ws, dist
    return 0, 1, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def kernel_table(lib, h):
    n = lib.hz_kernel_times(h, -1, None, 0, None, None, None, None)
    rows = []
    for i in range(n):
        name = C.create_string_buffer(64)
        la = C.c_int64()
        lt = C.c_int64()
        ms = C.c_double()
        by = C.c_double()
        lib.hz_kernel_times(h, i, name, 64, C.byref(la), C.byref(lt), C.byref(ms), C.byref(by))
        rows.append(dict(name=name.value.decode(), launches=la.value, timed=lt.value, ms=ms.value,
                         bytes=by.value))
    return rows


def traffic_ratio_from_profiles(kernel: str, workload: str):
    """DRAM bytes / algorithmic bytes of `kernel` from the committed ncu
    summary (a small case of the same workload; traffic scales with the
    columns processed), or None."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        e = d.get(workload, {}).get(kernel)
        return float(e["dram_over_algorithmic"]) if e else None
    except (ValueError, OSError, KeyError, TypeError):
        return None


def run_ours(args, rank, ws, dist):
    import torch
    import __graft_entry__ as ge
    ge._load_build_module().build()
    hz = ge.load_package()
    L = hz._lib
    lib = L.load()
    wl = workload(args)
    P = make_problem(wl, seed=1234)
    gam = gamma_of(P, wl["pad"], lib, hz)
    nrhs = wl["nrhs"]
    B = sources(P, nrhs, seed=rank)
    n = B.shape[0]

    def make_handle(precision):
        prob = L.hz_problem()
        prob.dim = P["dim"]
        for d in range(P["dim"]):
            prob.n[d] = P["cells"][d]
            prob.h[d] = P["h"][d]
        prob.omega_re, prob.omega_im = P["w"], 0.0
        keep = (np.ascontiguousarray(P["m"]), np.ascontiguousarray(gam))
        prob.m = keep[0].ctypes.data_as(C.POINTER(C.c_double))
        prob.gamma = keep[1].ctypes.data_as(C.POINTER(C.c_double))
        prob.neumann_on_top, prob.sommerfeld, prob.order_neumann_bc = 1, 1, 2
        o = L.hz_options()
        lib.hz_default_options(C.byref(o))
        o.levels, o.rel_tol, o.inner, o.max_outer = wl["levels"], wl["tol"], 10, args.max_outer
        o.cycle = ord(args.cycle)
        o.coarse_op = L.HZ_COARSE_REDISCRETIZE if args.coarse == "rediscretize" else L.HZ_COARSE_GALERKIN
        o.relax_type = L.HZ_RELAX_JAC_GMRES if args.relax == "jac-gmres" else L.HZ_RELAX_JAC
        o.relax_from = args.relax_from
        o.shift = args.shift
        o.cuda_graph = 0 if args.no_graph else 1
        o.autotune = 0 if args.no_tune else 1
        if args.krylov == "bicgstab":
            o.krylov, o.max_outer = L.HZ_KRYLOV_BICGSTAB, 2000
        o.precision = precision
        if precision == L.HZ_PREC_MIXED and args.outer == "emulated":
            o.outer_arith = L.HZ_OUTER_EMULATED
        o.device = torch.cuda.current_device()
        hh = C.c_void_p()
        L.check(lib.hz_create(C.byref(prob), C.byref(o), C.byref(hh)))
        return hh

    Bd = torch.from_numpy(np.ascontiguousarray(B.T)).to("cuda")  # (nrhs, n) row-major = column-major n x nrhs
    Xd = torch.empty_like(Bd)

    def solve_device(hh):
        st = L.hz_stats()
        code = lib.hz_solve(hh, Bd.data_ptr(), Xd.data_ptr(), n, nrhs, 0, L.HZ_MEM_DEVICE, C.byref(st))
        L.check(code, hh)
        return st, code

    def timed(hh, steps, fn):
        stream = torch.cuda.ExternalStream(lib.hz_stream(hh))
        barrier(dist)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        last = None
        for _ in range(steps):
            last = fn(hh)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier(dist)
        return e0.elapsed_time(e1) / 1000.0, last

    results = {}
    order = ["mixed", "fp64"] if args.precision == "both" else [args.precision]
    for prec in order:
        hh = make_handle(L.HZ_PREC_MIXED if prec == "mixed" else L.HZ_PREC_FP64)
        t_setup0 = time.perf_counter()
        for _ in range(args.warmup):
            solve_device(hh)
        setup_and_warm = time.perf_counter() - t_setup0
        steps = args.steps if prec == order[0] else max(1, args.plain_steps)
        lib.hz_reset_kernel_times(hh)
        lib.hz_set_profile(hh, 0)
        with ClockSampler(torch.cuda.current_device()) as clocks:
            t, (st, code) = timed(hh, steps, solve_device)
        t = max_over_ranks(dist, t)
        if prec == order[0]:
            # per-kernel CUDA events on the handle's stream over the same number of
            # solves right after (event records around every launch would slow the
            # timed solves themselves, most on small workloads)
            lib.hz_reset_kernel_times(hh)
            lib.hz_set_profile(hh, 1)
            timed(hh, steps, solve_device)
            lib.hz_set_profile(hh, 0)
        rr = np.zeros(nrhs)
        it = np.zeros(nrhs, dtype=np.int32)
        lib.hz_column_stats(hh, rr.ctypes.data_as(C.POINTER(C.c_double)), it.ctypes.data_as(C.POINTER(C.c_int32)),
                            nrhs)
        kt = kernel_table(lib, hh)
        res = dict(seconds=t, steps=steps, rhs_per_s=nrhs * ws * steps / t, ms_per_step=1000.0 * t / steps,
                   max_relres=float(rr.max()), mean_iters=float(it.mean()), max_iters=int(it.max()),
                   outer=int(st.outer), launches_per_step=int(st.kernel_launches), kernels=kt,
                   clocks=clocks.summary(), setup_warm_s=setup_and_warm, code=int(code))
        if prec == order[0]:
            # end to end through the public call with host buffers (pinned), copies inside the timed region
            Bh = torch.from_numpy(np.ascontiguousarray(B.T)).pin_memory()
            Xh = torch.empty_like(Bh).pin_memory()

            def solve_host(hh_):
                st_ = L.hz_stats()
                L.check(lib.hz_solve(hh_, Bh.data_ptr(), Xh.data_ptr(), n, nrhs, 0, L.HZ_MEM_HOST, C.byref(st_)),
                        hh_)
                return st_

            lib.hz_set_profile(hh, 0)
            solve_host(hh)
            t0 = time.perf_counter()
            barrier(dist)
            for _ in range(steps):
                st_h = solve_host(hh)
            barrier(dist)
            te = max_over_ranks(dist, time.perf_counter() - t0)
            res["e2e"] = dict(value=nrhs * ws * steps / te, unit="RHS/s", h2d_bytes_per_step=int(st_h.h2d_bytes),
                              d2h_bytes_per_step=int(st_h.d2h_bytes))
            # accuracy check of the last device solve against the FP64 operator
            Y = torch.empty_like(Xd)
            L.check(lib.hz_apply(hh, L.HZ_OP_H, 0, Xd.data_ptr(), Y.data_ptr(), n, nrhs, L.HZ_MEM_DEVICE), hh)
            rel = torch.linalg.vector_norm(Y - Bd, dim=1) / torch.linalg.vector_norm(Bd, dim=1)
            res["check_relres_max"] = float(rel.max())
        lib.hz_destroy(hh)
        results[prec] = res
        torch.cuda.empty_cache()
    return results, wl, P


def random_sources(P: dict, nrhs: int, seed: int, pad: int) -> np.ndarray:
    """Delta sources q = 1/||h||^2 at seeded random nodes outside the absorbing layer (2D)."""
    rng = np.random.default_rng(seed)
    nx, nz = P["nodes"]
    B = np.zeros((nx * nz, nrhs), dtype=np.complex128, order="F")
    amp = 1.0 / float(np.linalg.norm(P["h"])) ** 2
    for c in range(nrhs):
        i = int(rng.integers(pad, nx - pad))
        j = int(rng.integers(1, nz - pad))
        B[i + nx * j, c] = amp
    return B


def run_learned(args, rank, ws, dist):
    """Learned-correction workload: pairs from seeded training models (FP64
    solver), GPU training of the network, then per held-out model one step =
    solver setup + solve of its 32 right-hand sides (setup included in every arm)."""
    import torch
    import __graft_entry__ as ge
    ge._load_build_module().build()
    hz = ge.load_package()
    L = hz._lib
    lib = L.load()
    wl = workload(args)
    level = args.net_level if args.net_level > 0 else wl["net_level"]

    def solver(P, precision, outer="fp64", max_outer=60):
        M = hz.getRegularMesh(sum(([0.0, c * h] for c, h in zip(P["cells"], P["h"])), []), list(P["cells"]))
        gam = gamma_of(P, wl["pad"], lib, hz)
        param = hz.HelmholtzParam(M, gam, P["m"], P["w"], True, True)
        MG = hz.getMGparam(complex, int, wl["levels"], 1, max_outer, wl["tol"],
                           "Jac-GMRES" if args.relax == "jac-gmres" else "Jac", 0.8, 1, 1, args.cycle,
                           "Julia", 0.5, 0.0, precision=precision, outerArithmetic=outer,
                           coarseOperator="Rediscretize" if args.coarse == "rediscretize" else "Galerkin",
                           relaxFrom=args.relax_from)
        return hz.getShiftedLaplacianMultigridSolver(param, MG, args.shift, "GMRES", 10)

    # 1. training pairs from the FP64 solver on seeded training models
    t0 = time.perf_counter()
    xs, ts, pes = [], [], []
    for s in range(args.train_models):
        P = make_problem(wl, seed=10_000 + 97 * rank + s)
        S = solver(P, "fp64")
        B = random_sources(P, args.train_rhs, seed=20_000 + s, pad=wl["pad"])
        d = hz.learned.collect_pairs(S, B, level=level, sweeps=2, max_pairs=args.pairs_per_model)
        xs.append(d["x"].clone())
        ts.append(d["t"].clone())
        pes.append(d["plain_err"])
        del S, d
    x = torch.cat(xs).contiguous()
    t = torch.cat(ts).contiguous()
    del xs, ts
    collect_s = time.perf_counter() - t0
    # 2. training (the library's forward/backward/Adam kernels)
    net = hz.learned.CoarseNet(seed=1)
    t0 = time.perf_counter()
    hist = net.train(x, t, epochs=args.train_epochs, batch=32, lr=2e-3, seed=3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    train_err = float(np.median(hz.learned.pair_errors(net, x[:512], t[:512])))
    npairs = int(x.shape[0])
    del x, t
    torch.cuda.empty_cache()
    # held-out pairs: the network against one plain cycle from the same level
    P = make_problem(wl, seed=90_000 + rank)
    d = hz.learned.collect_pairs(solver(P, "fp64"), random_sources(P, 8, seed=90_001, pad=wl["pad"]), level=level,
                                 sweeps=2, max_pairs=400)
    held = dict(pairs=int(d["x"].shape[0]), net_median=float(np.median(hz.learned.pair_errors(net, d["x"], d["t"]))),
                plain_cycle_median=float(np.median(d["plain_err"])))
    del d
    # 3. timed arms on held-out models
    arms = [("learned_mixed", "mixed", True), ("mixed", "mixed", False), ("fp64", "fp64", False)]
    res = {}
    nrhs = wl["nrhs"]
    for name, prec, use_net in arms:
        nsteps = args.steps
        tot, iters, relres, fb, calls, launches, conv = 0.0, [], [], 0, 0, 0, 0
        clk = None
        for k in range(args.warmup + nsteps):
            P = make_problem(wl, seed=50_000 + 1000 * rank + k)
            B = random_sources(P, nrhs, seed=60_000 + k, pad=wl["pad"])
            Bd = torch.from_numpy(np.ascontiguousarray(B.T)).to("cuda")
            S = solver(P, prec, outer=args.outer if prec == "mixed" else "fp64")
            torch.cuda.synchronize()
            barrier(dist)
            sampler = ClockSampler(torch.cuda.current_device()) if k == args.warmup else None
            if sampler:
                sampler.__enter__()
            t0 = time.perf_counter()
            if use_net:
                hz.learned.attach(S, net, level=level, stag_ratio=args.stag_ratio)
            X, S = hz.solveLinearSystem(None, Bd.t(), S)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            if sampler:
                sampler.__exit__()
                clk = sampler.summary()
            if k >= args.warmup:
                tot += dt
                iters.append(float(np.mean(S.last_iters)))
                relres.append(float(np.max(S.last_relres)))
                conv += int(np.sum(S.last_relres <= wl["tol"]))
                launches += int(S.last_stats.kernel_launches)
                c_, f_ = hz.learned.learned_stats(S)
                calls += c_
                fb += f_
            del S, X, Bd
        tot = max_over_ranks(dist, tot)
        res[name] = dict(rhs_per_s=nrhs * ws * nsteps / tot, ms_per_step=1000.0 * tot / nsteps,
                         mean_iters=float(np.mean(iters)), max_relres=float(np.max(relres)), fallbacks=fb,
                         converged_cols=conv, cols=nrhs * nsteps, converged_rhs_per_s=conv * ws / tot,
                         net_calls=calls, launches_per_step=launches // nsteps, clocks=clk)
    info = dict(train_models=args.train_models, train_pairs=npairs, epochs=args.train_epochs,
                loss_first=float(hist[0]), loss_last=float(hist[-1]), collect_s=collect_s, train_s=train_s,
                train_pair_error_median=train_err, heldout=held)
    return res, info, wl


def run_cpu_sample(wl, P, gam_fn, budget_s: float, ncols_max: int = 4, cycle: str = "V",
                   coarse: str = "galerkin", relax: str = "jac", relax_from: int = 0, shift: float = 0.5):
    """C oracle (threaded CSR SLMG, plain FP64) on a bounded sample of the
    workload: the full grid and operator, a few of its right-hand sides, with
    the GPU arm's cycle, coarse operators (Galerkin or re-discretised) and
    smoother (damped Jacobi, or Jac-GMRES from level relax_from down)."""
    rkw = dict(relax="Jac-GMRES" if relax == "jac-gmres" else "Jac", gmres_from=relax_from)
    sys.path.insert(0, str(ROOT / "oracle"))
    import helmholtz_oracle as O
    import slmg_cpu
    M = O.getRegularMesh(sum(([0.0, c * h] for c, h in zip(P["cells"], P["h"])), []), list(P["cells"]))
    gam = gam_fn()
    H = O.GetHelmholtzOperator(M, P["m"], P["w"], gam, True, True)
    SH = (H + O.GetHelmholtzShiftOP(P["m"], P["w"], shift)).tocsr()
    hier = None
    if coarse == "rediscretize":
        hier = O.build_hierarchy_rediscretized(M, P["m"], gam, P["w"], shift, True, True, wl["levels"])
    cpu = slmg_cpu.CpuSLMG(H, SH, M, wl["levels"], hier=hier)
    B = sources(P, wl["nrhs"], seed=0)
    ncols = 1
    r = cpu.solve(B[:, :1], tol=wl["tol"], max_outer=200, cycle=cycle, **rkw)
    t1 = r.solve_s
    ncols = int(max(1, min(ncols_max, B.shape[1], budget_s // max(t1, 1e-3))))
    if ncols > 1:
        r = cpu.solve(B[:, :ncols], tol=wl["tol"], max_outer=200, cycle=cycle, **rkw)
    return dict(value=ncols / r.solve_s, unit="RHS/s", cores=r.threads, kind="port",
                sample=f"{ncols} of the {wl['nrhs']} right-hand sides of the same workload (full grid, "
                       f"same operator, plain FP64 SLMG ({cycle}-cycle, {coarse} coarse levels, {rkw['relax']} "
                       f"smoothing{f' from level {relax_from}' if relax == 'jac-gmres' else ''}) in threaded C, "
                       f"{int(r.iters.mean())} iterations per RHS)",
                seconds=r.solve_s, setup_s=r.setup_s, max_relres=float(r.relres.max()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("HZ_BENCH_WORKLOAD", "c2"), choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64"])
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nrhs", type=int, default=0, help="override the workload's RHS count (small profiling cases)")
    ap.add_argument("--krylov", default="fgmres", choices=["fgmres", "bicgstab"])
    ap.add_argument("--outer", default="emulated", choices=["fp64", "emulated"],
                    help="outer Krylov arithmetic of the mixed form: native FP64 or FP64 emulated with FP32 pairs")
    ap.add_argument("--no-graph", action="store_true", help="launch the cycles eagerly (no CUDA graphs)")
    ap.add_argument("--no-tune", action="store_true", help="default stencil launch shapes (no autotuning)")
    ap.add_argument("--max-outer", type=int, default=200,
                    help="FGMRES restart cycles (fewer: kernel-rate profiling runs, not a valid RHS/s)")
    ap.add_argument("--cycle", default="V", choices=["V", "W", "K"],
                    help="multigrid cycle (K: two FGMRES steps per coarse level)")
    ap.add_argument("--coarse", default="galerkin", choices=["galerkin", "rediscretize"],
                    help="coarse-level operators: Galerkin R A P, or the operator re-discretised on each coarse mesh")
    ap.add_argument("--levels", type=int, default=0, help="multigrid levels (0: the workload's)")
    ap.add_argument("--relax", default="jac", choices=["jac", "jac-gmres"],
                    help="smoother: damped Jacobi, or GMRES steps preconditioned by a Jacobi sweep (relaxType "
                         "'Jac-GMRES')")
    ap.add_argument("--relax-from", type=int, default=0, help="jac-gmres: first level smoothed by GMRES steps")
    ap.add_argument("--shift", type=float, default=0.5, help="s of the shifted operator SH = H + i s w^2 diag(m)")
    ap.add_argument("--train-models", type=int, default=48, help="learned workload: seeded training models")
    ap.add_argument("--train-rhs", type=int, default=4, help="learned workload: random sources per training model")
    ap.add_argument("--pairs-per-model", type=int, default=200)
    ap.add_argument("--train-epochs", type=int, default=20)
    ap.add_argument("--net-level", type=int, default=0, help="learned workload: multigrid level of the network "
                    "(0: the workload's)")
    ap.add_argument("--stag-ratio", type=float, default=0.95,
                    help="learned workload: a restart cycle reducing a residual by less than this hands over "
                         "to the plain cycle")
    args = ap.parse_args()
    peak, peak_kind = load_peaks()

    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        wl = workload(args)
        P = make_problem(wl, seed=1234)
        import __graft_entry__ as ge
        hz = ge.load_package()
        gam = gamma_of(P, wl["pad"], None, hz)
        vals = []
        cs = None
        for i in range(args.warmup + args.steps):
            cs = run_cpu_sample(wl, P, lambda: gam, args.cpu_budget / max(1, args.steps), cycle=args.cycle,
                                coarse=args.coarse, relax=args.relax, relax_from=args.relax_from,
                                shift=args.shift)
            if i >= args.warmup:
                vals.append(cs["value"])
        v = float(np.mean(vals))
        line = dict(metric=METRIC, value=v, unit="RHS/s", impl="reference", n_gpus=args.gpus, steps=args.steps,
                    warmup=args.warmup, higher_is_better=True, dtype="c128",
                    config=dict(workload=wl["name"], nrhs=wl["nrhs"], levels=wl["levels"], cycle=args.cycle,
                                coarse=args.coarse, relax=args.relax, relax_from=args.relax_from,
                                shift=args.shift),
                    cpu_baseline=dict(value=v, unit="RHS/s", cores=cs["cores"], kind="port", sample=cs["sample"]),
                    e2e=dict(value=v, unit="RHS/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                    note="reference path = the C oracle port of the Julia SLMG (Julia and Multigrid.jl are absent)")
        print(json.dumps(line))
        return

    rank, ws, dist = dist_setup()
    if WORKLOADS[args.workload].get("learned"):
        res, info, wl = run_learned(args, rank, ws, dist)
        if rank != 0:
            return
        head = res["learned_mixed"]
        # the metric counts right-hand sides solved to the tolerance: columns that
        # did not converge within the restart limit count as time spent, not as solved
        line = dict(metric=METRIC, value=head["converged_rhs_per_s"], unit="RHS/s", n_gpus=ws, steps=args.steps,
                    warmup=args.warmup, ms_per_step=head["ms_per_step"], higher_is_better=True, scaling="weak",
                    vs_baseline=None, dtype="c64 V-cycle + bf16 network / c128 outer",
                    data="synthetic (seeded layered+inclusion models, random source positions)",
                    config=dict(workload=wl["name"], nrhs=wl["nrhs"], levels=wl["levels"], tol=wl["tol"],
                                krylov="FGMRES(10)", cycle=args.cycle, coarse=args.coarse, relax=args.relax,
                                relax_from=args.relax_from, shift=args.shift, outer_arithmetic=args.outer,
                                learned=True,
                                net_level=args.net_level if args.net_level > 0 else wl["net_level"],
                                stag_ratio=args.stag_ratio,
                                step="solver setup + solve of one held-out model's right-hand sides",
                                l2="inputs larger than L2 (one step touches > 1 GB)"),
                    gpu_launches=head["launches_per_step"] * args.steps, clocks=head["clocks"],
                    learned_over_plain_fp64=(head["converged_rhs_per_s"] / res["fp64"]["converged_rhs_per_s"]
                                             if res["fp64"]["converged_rhs_per_s"] > 0 else None),
                    learned_over_mixed=(head["converged_rhs_per_s"] / res["mixed"]["converged_rhs_per_s"]
                                        if res["mixed"]["converged_rhs_per_s"] > 0 else None),
                    arms=res, training=info)
        print(json.dumps(line))
        return
    results, wl, P = run_ours(args, rank, ws, dist)
    if rank != 0:
        return
    head = results[args.precision if args.precision != "both" else "mixed"]
    # dominant kernel of the timed region (event-timed per launch on the handle's stream)
    kt = [k for k in head["kernels"] if k["timed"] > 0]
    # the graph entry aggregates the cycle's kernels: the roofline names a kernel
    kk = [k for k in kt if k["name"] != "vcycle_graph"]
    dom = max(kk, key=lambda k: k["ms"]) if kk else None
    roofline = None
    if dom:
        achieved = dom["bytes"] / (dom["ms"] / 1000.0) / 1e9
        ratio = traffic_ratio_from_profiles(dom["name"], args.workload) if args.nrhs == 0 else None
        tr = None if ratio is None else ratio * dom["bytes"] / dom["launches"]
        roofline = dict(bound="hbm", kernel=dom["name"], achieved=achieved, peak=peak, unit="GB/s",
                        frac=achieved / peak, peak_source=f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                        traffic=tr, avg_launch_ms=dom["ms"] / dom["timed"],
                        share=dom["ms"] / sum(k["ms"] for k in kt),
                        source="CUDA events around every launch on the handle's stream, over the same number of "
                               "solves right after the timed ones")
    # whole-solve roofline: the algorithmic bytes of every launched kernel of a
    # solve (from the profiled solves, same workload and iteration counts) over
    # the unprofiled time of a solve
    solve_bytes = sum(k["bytes"] for k in head["kernels"]) / max(1, head["steps"])
    solve_roof = dict(bound="hbm", achieved=solve_bytes / (head["ms_per_step"] / 1e3) / 1e9, peak=peak, unit="GB/s",
                      frac=solve_bytes / (head["ms_per_step"] / 1e3) / 1e9 / peak, bytes_per_solve=solve_bytes)
    cpu = None
    if not args.no_cpu:
        import __graft_entry__ as ge
        hz = ge.load_package()
        gam = gamma_of(P, wl["pad"], None, hz)
        cpu = run_cpu_sample(wl, P, lambda: gam, args.cpu_budget, cycle=args.cycle, coarse=args.coarse,
                             relax=args.relax, relax_from=args.relax_from, shift=args.shift)
    plain = results.get("fp64")
    line = dict(metric=METRIC, value=head["rhs_per_s"], unit="RHS/s", n_gpus=ws, steps=args.steps,
                warmup=args.warmup, ms_per_step=head["ms_per_step"], higher_is_better=True, scaling="weak",
                vs_baseline=None,
                dtype=("c64 V-cycle / c128 outer" + (" (emulated by FP32 pairs)" if args.outer == "emulated" else "")
                       if args.precision != "fp64" else "c128"),
                data="synthetic (seeded layered model)",
                config=dict(workload=wl["name"], nrhs=wl["nrhs"], levels=wl["levels"], tol=wl["tol"],
                            krylov="FGMRES(10)" if args.krylov == "fgmres" else "BiCGSTAB", cycle=args.cycle,
                            coarse=args.coarse, relax=args.relax, relax_from=args.relax_from, shift=args.shift,
                            cuda_graph=not args.no_graph, autotune=not args.no_tune,
                            outer_arithmetic=args.outer,
                            precision="mixed" if args.precision != "fp64" else "fp64", learned=False,
                            l2="inputs larger than L2 (RHS block %.2f GB)" % (P["m"].size * wl["nrhs"] * 16 / 1e9)),
                e2e=head.get("e2e"), gpu_launches=head["launches_per_step"] * args.steps,
                clocks=head["clocks"], roofline=roofline, solve_roofline=solve_roof,
                cpu_baseline=cpu,
                max_relres=head["max_relres"], check_relres_max=head.get("check_relres_max"),
                mean_iters=head["mean_iters"],
                plain_fp64=None if plain is None else dict(rhs_per_s=plain["rhs_per_s"],
                                                           ms_per_step=plain["ms_per_step"],
                                                           mean_iters=plain["mean_iters"],
                                                           max_relres=plain["max_relres"]),
                mixed_over_plain=None if plain is None else head["rhs_per_s"] / plain["rhs_per_s"],
                kernels=[dict(name=k["name"], launches=k["launches"], ms=round(k["ms"], 3),
                              gbs=(k["bytes"] / (k["ms"] / 1e3) / 1e9) if k["ms"] > 0 else None)
                         for k in sorted(kt, key=lambda k: -k["ms"])[:12]])
    print(json.dumps(line))


if __name__ == "__main__":
    main()
