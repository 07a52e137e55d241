"""Throughput benchmark: right-hand sides solved per second to relative
residual 1e-6 by the shifted-Laplacian multigrid FGMRES solve on one GB300.

One step = one hz_solve of the workload's whole right-hand-side block (every
column to rel. residual <= tol).  Default workload: 3D 257^3 nodes x 32
surface sources, five Galerkin levels, K-cycle with "Jac-GMRES" smoothing from
level 1 down, FGMRES(10) to 1e-6.  Three forms of the same solver run in one
process on the same GPU:

  mixed           complex-FP32 cycle, FP64 coarsest LU, native-FP64 outer FGMRES (headline)
  mixed_emulated  the same cycle, outer FGMRES in FP64 emulated by FP32 pairs (labelled arm)
  fp64            plain complex FP64 throughout (the metric's denominator)

Every arm states its relative residual and its error against an FP64 oracle
(2D: sparse direct solve of sampled columns; 3D: the C oracle's FP64 SLMG
solve of a sampled column to 1e-10).

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

# solver options a workload does not set
SOLVER_DEFAULTS = dict(cycle="V", relax="jac", relax_from=0, shift=0.5, coarse="galerkin")

# Synthetic seeded workloads (shapes, sizes and value distributions of the
# measured configurations; no external dataset is needed).
WORKLOADS = {
    # 2D 129 x 129 on [0,1]^2, v = 1.5 + 3 z with the v = 4.5 ellipse, one source
    # at (0.5, 2h), absorbing layer 16, 3 levels, FGMRES(10) to 1e-8
    "c1": dict(name="2D 129x129 gradient+ellipse, 1 source, 3 levels, FGMRES(10) tol 1e-8",
               cells=(128, 128), h=1.0 / 128, nrhs=1, levels=3, pad=16, ellipsoid=False, tol=1e-8,
               model="gradient_ellipse", err_cols=1),
    # 2D 1025 x 513 nodes, h = 10 m, 12 seeded layers in [1.5, 4.5] km/s,
    # absorbing layer 32 cells, 64 sources along the surface row, 5 levels
    "c2": dict(name="2D 1025x513 layered, 64 surface sources, 5 levels, FGMRES(10) tol 1e-6",
               cells=(1024, 512), h=0.010, nrhs=64, levels=5, pad=32, ellipsoid=False, tol=1e-6, err_cols=4),
    # 3D 129^3 nodes layered + ellipsoid, absorbing layer 12, 4x4 surface sources, 4 levels
    "c3": dict(name="3D 129^3 layered+ellipsoid, 16 surface sources, 4 levels, FGMRES(10) tol 1e-6",
               cells=(128, 128, 128), h=0.010, nrhs=16, levels=4, pad=12, ellipsoid=True, tol=1e-6, err_cols=1),
    # 2D 513 x 513 layered + inclusion models, learned coarse correction below level 2: trained on
    # pairs from seeded training models, evaluated on held-out seeds x 32 random-position sources
    "c4": dict(name="2D 513x513 layered+inclusion, learned coarse correction below level 2, 32 random sources, "
                    "5 levels, FGMRES(10) tol 1e-6",
               cells=(512, 512), h=0.010, nrhs=32, levels=5, pad=32, ellipsoid=True, tol=1e-6, learned=True,
               net_level=2),
    # 3D 257^3 nodes (16,974,593 unknowns per RHS), absorbing layer 16, 32 surface sources; the
    # five-level Galerkin hierarchy converges with the K-cycle and GMRES smoothing from level 1
    "c5": dict(name="3D 257^3 layered+ellipsoid, 32 surface sources, 5 levels, FGMRES(10) tol 1e-6",
               cells=(256, 256, 256), h=0.010, nrhs=32, levels=5, pad=16, ellipsoid=True, tol=1e-6, err_cols=1,
               cycle="K", relax="jac-gmres", relax_from=1, shift=0.3,
               # 3D learned correction: the network preconditions the K-cycle steps on level 3 (33^3) in
               # place of the level-3 cycle and the coarsest band LU; pairs from seeded training models
               learned3d=True, net_level=3, train_models=6, train_rhs=8, pairs_per_model=640, train_outer=2,
               pair_sweeps=30, train_epochs=30, train_batch=8),
}
DEFAULT_WORKLOAD = "c5"


def workload(args) -> dict:
    """The chosen workload with the command line's overrides (RHS count, level
    count, the learned correction's level and pairs per training model)."""
    wl = dict(WORKLOADS[args.workload])
    if args.nrhs > 0:
        wl["nrhs"] = args.nrhs
    if args.levels > 0:
        wl["levels"] = args.levels
    if getattr(args, "net_level", 0) > 0 and "net_level" in wl:
        wl["net_level"] = args.net_level
    if getattr(args, "pairs_per_model", None) and wl.get("learned3d"):
        wl["pairs_per_model"] = args.pairs_per_model
    return wl


def resolve_solver_args(args) -> None:
    """Fill the solver options the command line left unset from the workload."""
    wl = WORKLOADS[args.workload]
    for k, v in SOLVER_DEFAULTS.items():
        if getattr(args, k) is None:
            setattr(args, k, wl.get(k, v))


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
    """Total attenuation through the library's getABL (the GPU arms)."""
    abl = hz.getABL(P["nodes"], True, [pad] * P["dim"], 0.95 * P["w"]).ravel(order="F")
    return abl + 0.01 * P["w"]


def gamma_oracle(P: dict, pad: int) -> np.ndarray:
    """The same attenuation through the oracle's getABL (the CPU reference and
    checker legs, which use nothing of the product)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import helmholtz_oracle as O
    abl = O.getABL(np.array(P["nodes"]), True, [pad] * P["dim"], 0.95 * P["w"]).ravel(order="F")
    return abl + 0.01 * P["w"]


def run_config(args, wl: dict, P: dict) -> dict:
    """The `config` object both arms print (the same keys and values)."""
    return dict(workload=wl["name"], nrhs=wl["nrhs"], levels=wl["levels"], tol=wl["tol"],
                krylov="FGMRES(10)" if args.krylov == "fgmres" else "BiCGSTAB", cycle=args.cycle,
                coarse=args.coarse, relax=args.relax, relax_from=args.relax_from, shift=args.shift,
                seed=1234, learned=False,
                l2="inputs larger than L2 (RHS block %.2f GB)" % (P["m"].size * wl["nrhs"] * 16 / 1e9))


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


# GB300's FP64 rate: no measured figure exists for it, so the nominal one is used
FP64_PEAK_TFLOPS = 1.25
# the kernels of the outer Krylov method that compute in FP64 (the library counts
# their flops only when they do: the emulated form's kernels of these names count none)
FP64_KERNELS = ("krylov_dots", "krylov_update", "update_x", "outer_apply", "outer_resid")


def kernel_table(lib, h):
    n = lib.hz_kernel_times(h, -1, None, 0, None, None, None, None)
    rows = []
    for i in range(n):
        name = C.create_string_buffer(64)
        la = C.c_int64()
        lt = C.c_int64()
        ms = C.c_double()
        by = C.c_double()
        fl = C.c_double()
        lib.hz_kernel_times(h, i, name, 64, C.byref(la), C.byref(lt), C.byref(ms), C.byref(by))
        lib.hz_kernel_flops(h, i, C.byref(fl))
        rows.append(dict(name=name.value.decode(), launches=la.value, timed=lt.value, ms=ms.value,
                         bytes=by.value, flops=fl.value))
    return rows


def device_gb_in_use():
    """GB in use on the current CUDA device: every allocation on it, the library's
    own cudaMalloc buffers included (torch's allocator does not see those); None
    where the query fails."""
    try:
        import torch
        free, total = torch.cuda.mem_get_info()
        return (total - free) / 1e9
    except Exception:
        return None


def fp64_rate(k: dict):
    """FP64 TFLOP/s of a kernel-table row and its fraction of the nominal FP64
    peak, or None for a row that is not a native-FP64 kernel or was not timed."""
    if k["name"] not in FP64_KERNELS or not k.get("flops") or not k["ms"] > 0:
        return None
    t = k["flops"] / (k["ms"] / 1e3) / 1e12
    return dict(achieved=t, peak=FP64_PEAK_TFLOPS, unit="TFLOP/s", frac=t / FP64_PEAK_TFLOPS,
                peak_source="nominal GB300 FP64 rate (no measured FP64 peak)")


def kernel_rows(kt, peak: float, tot_ms: float, top: int = 24) -> list:
    """The bench line's per-kernel table: HBM rate and fraction of the measured
    copy bandwidth for every row, the tensor or FP64 rate where the library
    counts the kernel's flops."""
    out = []
    for k in sorted(kt, key=lambda k: -k["ms"])[:top]:
        r = dict(name=k["name"], launches=k["launches"], ms=round(k["ms"], 3),
                 gbs=(k["bytes"] / (k["ms"] / 1e3) / 1e9) if k["ms"] > 0 else None,
                 frac=(k["bytes"] / (k["ms"] / 1e3) / 1e9 / peak) if k["ms"] > 0 else None,
                 share=k["ms"] / tot_ms)
        f64 = fp64_rate(k)
        if f64 is not None:
            r["fp64_tflops"] = f64["achieved"]
            r["fp64_frac"] = f64["frac"]
        elif k.get("flops") and k["ms"] > 0:
            r["tflops"] = k["flops"] / (k["ms"] / 1e3) / 1e12
        out.append(r)
    return out


def profile_entry(kernel: str, workload: str) -> dict:
    """The committed ncu summary of `kernel` on a small case of the workload's
    path (profiles/traffic.json): DRAM / algorithmic bytes (traffic scales with
    the columns processed) and, for the FP64 kernels, the FP64 pipe's share of
    its peak; {} when there is none."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return {}
    try:
        e = json.loads(p.read_text()).get(workload, {}).get(kernel)
        return dict(e) if e else {}
    except (ValueError, OSError, TypeError):
        return {}


# ---------------------------------------------------------------------------
# GPU arms
# ---------------------------------------------------------------------------
ARMS = {
    # name: (precision, outer arithmetic, learned correction)
    "learned_mixed": ("mixed", "fp64", True),
    "mixed": ("mixed", "fp64", False),
    "mixed_emulated": ("mixed", "emulated", False),
    "learned_emulated": ("mixed", "emulated", True),
    "fp64": ("fp64", "fp64", False),
}
ARM_SETS = {"all": ["mixed", "mixed_emulated", "fp64"], "both": ["mixed", "fp64"], "mixed": ["mixed"],
            "emulated": ["mixed_emulated"], "fp64": ["fp64"]}
# with the learned correction the headline is the metric's own learned+mixed form
ARM_SETS_LEARNED = {"all": ["learned_mixed", "mixed", "mixed_emulated", "learned_emulated", "fp64"],
                    "both": ["learned_mixed", "fp64"], "mixed": ["learned_mixed"], "emulated": ["learned_emulated"],
                    "fp64": ["fp64"]}


def arm_names(args, wl) -> list:
    learned = wl.get("learned3d") and not args.no_learned
    return (ARM_SETS_LEARNED if learned else ARM_SETS)[args.precision]


def sources_random3(P: dict, nrhs: int, seed: int, pad: int) -> np.ndarray:
    """Delta sources q = 1/||h||^2 at seeded random nodes of a 3D grid outside the absorbing layer."""
    rng = np.random.default_rng(seed)
    nn = P["nodes"]
    B = np.zeros((int(np.prod(nn)), nrhs), dtype=np.complex128, order="F")
    amp = 1.0 / float(np.linalg.norm(P["h"])) ** 2
    for c in range(nrhs):
        i = int(rng.integers(pad, nn[0] - pad))
        j = int(rng.integers(pad, nn[1] - pad))
        k = int(rng.integers(1, nn[2] - pad))
        B[i + nn[0] * (j + nn[1] * k), c] = amp
    return B


def learned_cycle(args) -> str:
    """Cycle of the learned arms and of the solves that give their training pairs."""
    return args.learned_cycle or args.cycle


def train_network3d(args, wl, hz, lib):
    """Training pairs on the network's level from the FP64 solver on seeded
    training models (the first restart cycles of solves with random sources),
    then GPU training of the 3D network by the library's kernels."""
    import torch
    level = wl["net_level"]
    xs, ts, pes, worst = [], [], [], 0.0
    t0 = time.perf_counter()
    for s in range(wl["train_models"]):
        P = make_problem(wl, seed=10_000 + s)
        gam = gamma_of(P, wl["pad"], lib, hz)
        M = hz.getRegularMesh(sum(([0.0, c * h] for c, h in zip(P["cells"], P["h"])), []), list(P["cells"]))
        param = hz.HelmholtzParam(M, gam, P["m"], P["w"], True, True)
        MG = hz.getMGparam(complex, int, wl["levels"], 1, wl["train_outer"], wl["tol"],
                           "Jac-GMRES" if args.relax == "jac-gmres" else "Jac", 0.8, 1, 1, learned_cycle(args),
                           "Julia", args.shift, 0.0, precision="fp64", relaxFrom=args.relax_from)
        S = hz.getShiftedLaplacianMultigridSolver(param, MG, args.shift, "GMRES", 10)
        B = sources_random3(P, wl["train_rhs"], seed=20_000 + s, pad=wl["pad"])
        d = hz.learned.collect_pairs(S, B, level=level, sweeps=wl["pair_sweeps"], max_pairs=wl["pairs_per_model"])
        xs.append(d["x"].clone())
        ts.append(d["t"].clone())
        pes.append(d["plain_err"])
        worst = max(worst, float(d["target_relres"]))
        del S, d
        torch.cuda.empty_cache()
    x = torch.cat(xs).contiguous()
    t = torch.cat(ts).contiguous()
    del xs, ts
    collect_s = time.perf_counter() - t0
    net = hz.learned.CoarseNet3D(seed=1)
    t0 = time.perf_counter()
    hist = net.train(x, t, epochs=wl["train_epochs"], batch=wl["train_batch"], lr=2e-3, seed=3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    err = hz.learned.pair_errors(net, x[:256], t[:256], batch=8)
    pe = np.concatenate(pes)
    info = dict(train_models=wl["train_models"], train_pairs=int(x.shape[0]), grid=list(x.shape[1:4][::-1]),
                level=level, epochs=wl["train_epochs"], batch=wl["train_batch"], loss_first=float(hist[0]),
                loss_last=float(hist[-1]), collect_s=collect_s, train_s=train_s,
                target_relres_max=worst, pair_error_median_network=float(np.median(err)),
                pair_error_median_plain_correction=float(np.median(pe)),
                pairs="level-%d right-hand sides of the first %d restart cycles of FP64 solves of %d random sources "
                      "per training model; targets from %d restarted corrections on that level"
                      % (level, wl["train_outer"], wl["train_rhs"], wl["pair_sweeps"]))
    del x, t
    torch.cuda.empty_cache()
    return net, info


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
    err_cols = list(range(min(nrhs, wl.get("err_cols", 1))))

    def make_handle(precision, outer, cycle):
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
        o.cycle = ord(cycle)
        o.coarse_op = L.HZ_COARSE_REDISCRETIZE if args.coarse == "rediscretize" else L.HZ_COARSE_GALERKIN
        o.relax_type = L.HZ_RELAX_JAC_GMRES if args.relax == "jac-gmres" else L.HZ_RELAX_JAC
        o.relax_from = args.relax_from
        o.shift = args.shift
        o.cuda_graph = 0 if args.no_graph else 1
        o.autotune = 0 if args.no_tune else 1
        if args.krylov == "bicgstab":
            o.krylov, o.max_outer = L.HZ_KRYLOV_BICGSTAB, 2000
        o.precision = L.HZ_PREC_MIXED if precision == "mixed" else L.HZ_PREC_FP64
        o.outer_arith = L.HZ_OUTER_EMULATED if outer == "emulated" else L.HZ_OUTER_FP64
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
    names = arm_names(args, wl)
    net, train_info = None, None
    if any(ARMS[nm][2] for nm in names):
        net, train_info = train_network3d(args, wl, hz, lib)
    for ai, name in enumerate(names):
        prec, outer, use_net = ARMS[name]
        head = ai == 0
        cyc = learned_cycle(args) if use_net else args.cycle
        hh = make_handle(prec, outer, cyc)
        if use_net:
            L.check(lib.hz_attach_net(hh, net._h, wl["net_level"], args.stag_ratio), hh)
        warm = args.warmup if head else max(1, args.arm_warmup)
        steps = args.steps if head else max(1, args.plain_steps if name == "fp64" else args.arm_steps)
        t_setup0 = time.perf_counter()
        for _ in range(warm):
            solve_device(hh)
        setup_and_warm = time.perf_counter() - t_setup0
        lib.hz_reset_kernel_times(hh)
        lib.hz_set_profile(hh, 0)
        with ClockSampler(torch.cuda.current_device()) as clocks:
            t, (st, code) = timed(hh, steps, solve_device)
        t = max_over_ranks(dist, t)
        launches = int(st.kernel_launches)
        rr = np.zeros(nrhs)
        it = np.zeros(nrhs, dtype=np.int32)
        lib.hz_column_stats(hh, rr.ctypes.data_as(C.POINTER(C.c_double)), it.ctypes.data_as(C.POINTER(C.c_int32)),
                            nrhs)
        calls, fbs = C.c_int64(0), C.c_int32(0)
        if use_net:
            lib.hz_learned_stats(hh, C.byref(calls), C.byref(fbs))
        res = dict(precision=prec, outer_arithmetic=outer, learned=use_net, cycle=cyc, net_calls=int(calls.value),
                   net_fallbacks=int(fbs.value), seconds=t, steps=steps, warmup=warm,
                   rhs_per_s=nrhs * ws * steps / t, ms_per_step=1000.0 * t / steps, max_relres=float(rr.max()),
                   converged_cols=int(np.sum(rr <= wl["tol"])), mean_iters=float(it.mean()), max_iters=int(it.max()),
                   outer=int(st.outer), launches_per_step=launches, clocks=clocks.summary(),
                   setup_warm_s=setup_and_warm, code=int(code), device_gb=device_gb_in_use(),
                   x_err_cols=Xd[err_cols].cpu().numpy())
        if head:
            # per-kernel CUDA events on the handle's stream over one solve right after the timed
            # ones, with the cycle launched eagerly so that every kernel of it is timed by itself
            lib.hz_reset_kernel_times(hh)
            lib.hz_set_cuda_graph(hh, 0)
            lib.hz_set_profile(hh, 1)
            timed(hh, 1, solve_device)
            lib.hz_set_profile(hh, 0)
            lib.hz_set_cuda_graph(hh, 0 if args.no_graph else 1)
            res["kernels"] = kernel_table(lib, hh)
            # end to end through the public call with host buffers (pinned), copies inside the timed region
            Bh = torch.from_numpy(np.ascontiguousarray(B.T)).pin_memory()
            Xh = torch.empty_like(Bh).pin_memory()

            def solve_host(hh_):
                st_ = L.hz_stats()
                L.check(lib.hz_solve(hh_, Bh.data_ptr(), Xh.data_ptr(), n, nrhs, 0, L.HZ_MEM_HOST, C.byref(st_)),
                        hh_)
                return st_

            e2e_steps = max(1, min(steps, args.e2e_steps))
            solve_host(hh)
            barrier(dist)
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                st_h = solve_host(hh)
            barrier(dist)
            te = max_over_ranks(dist, time.perf_counter() - t0)
            res["e2e"] = dict(value=nrhs * ws * e2e_steps / te, unit="RHS/s", steps=e2e_steps,
                              h2d_bytes_per_step=int(st_h.h2d_bytes), d2h_bytes_per_step=int(st_h.d2h_bytes))
            # residual check of the last device solve with the FP64 operator
            Y = torch.empty_like(Xd)
            L.check(lib.hz_apply(hh, L.HZ_OP_H, 0, Xd.data_ptr(), Y.data_ptr(), n, nrhs, L.HZ_MEM_DEVICE), hh)
            rel = torch.linalg.vector_norm(Y - Bd, dim=1) / torch.linalg.vector_norm(Bd, dim=1)
            res["check_relres_max"] = float(rel.max())
            del Bh, Xh, Y
        lib.hz_destroy(hh)
        results[name] = res
        torch.cuda.empty_cache()
    del Bd, Xd
    torch.cuda.empty_cache()
    return results, wl, P, B, err_cols, train_info


# ---------------------------------------------------------------------------
# CPU legs (the oracle): checker and baseline
# ---------------------------------------------------------------------------
class OracleSolver:
    """The C oracle (threaded CSR SLMG, plain FP64) on the workload's full grid
    with the GPU arms' cycle, coarse operators and smoother."""

    def __init__(self, wl, P, args):
        sys.path.insert(0, str(ROOT / "oracle"))
        import helmholtz_oracle as O
        import slmg_cpu
        t0 = time.perf_counter()
        M = O.getRegularMesh(sum(([0.0, c * h] for c, h in zip(P["cells"], P["h"])), []), list(P["cells"]))
        gam = gamma_oracle(P, wl["pad"])
        H = O.GetHelmholtzOperator(M, P["m"], P["w"], gam, True, True)
        SH = (H + O.GetHelmholtzShiftOP(P["m"], P["w"], args.shift)).tocsr()
        hier = None
        if args.coarse == "rediscretize":
            hier = O.build_hierarchy_rediscretized(M, P["m"], gam, P["w"], args.shift, True, True, wl["levels"])
        self.cpu = slmg_cpu.CpuSLMG(H, SH, M, wl["levels"], hier=hier)
        self.kw = dict(cycle=args.cycle, relax="Jac-GMRES" if args.relax == "jac-gmres" else "Jac",
                       gmres_from=args.relax_from)
        self.desc = (f"plain FP64 SLMG ({args.cycle}-cycle, {args.coarse} coarse levels, {self.kw['relax']} smoothing"
                     f"{f' from level {args.relax_from}' if args.relax == 'jac-gmres' else ''}) in threaded C")
        self.setup_s = time.perf_counter() - t0

    def cycles(self, b, tol, max_cycles, X0=None):
        """Restart cycles of one column, one call per cycle, from X0 (default
        zero) until rel. residual <= tol: returns (X, iterations, seconds per
        cycle, relres, threads)."""
        X = np.zeros((b.shape[0], 1), dtype=np.complex128) if X0 is None else X0
        its, secs, rr, thr = 0, [], np.inf, 1
        for _ in range(max_cycles):
            r = self.cpu.solve(b, tol=tol, max_outer=1, X0=X, **self.kw)
            X = r.X
            its += int(r.iters.sum())
            secs.append(r.solve_s)
            rr = float(r.relres.max())
            thr = r.threads
            if rr <= tol:
                break
        return X, its, secs, rr, thr


def direct_errors(wl, P, B, err_cols, arms):
    """2D: relative error of each arm's sampled columns against a sparse direct
    solve (SuperLU) of the same operator, assembled by the oracle."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import helmholtz_oracle as O
    M = O.getRegularMesh(sum(([0.0, c * h] for c, h in zip(P["cells"], P["h"])), []), list(P["cells"]))
    H = O.GetHelmholtzOperator(M, P["m"], P["w"], gamma_oracle(P, wl["pad"]), True, True)
    Xref = O.direct_solve(H, B[:, err_cols])
    out = {}
    for name, res in arms.items():
        Xg = res["x_err_cols"].T
        out[name] = float(max(np.linalg.norm(Xg[:, k] - Xref[:, k]) / np.linalg.norm(Xref[:, k])
                              for k in range(len(err_cols))))
    return out, dict(kind="sparse direct solve (SciPy SuperLU) of the oracle's FP64 operator",
                     columns=list(err_cols))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("HZ_BENCH_WORKLOAD", DEFAULT_WORKLOAD),
                    choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="all", choices=sorted(ARM_SETS),
                    help="arms: all = mixed (headline) + mixed_emulated + fp64; both = mixed + fp64")
    ap.add_argument("--plain-steps", type=int, default=3, help="timed solves of the plain FP64 arm")
    ap.add_argument("--arm-steps", type=int, default=3, help="timed solves of the emulated-outer arm")
    ap.add_argument("--arm-warmup", type=int, default=1, help="untimed solves before the other arms' timed ones")
    ap.add_argument("--e2e-steps", type=int, default=3, help="end-to-end solves (host buffers), at most --steps")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and the 3D oracle error")
    ap.add_argument("--no-learned", action="store_true",
                    help="3D 257^3 workload: skip the learned correction (no training, no learned arms)")
    ap.add_argument("--learned-cycle", default=None, choices=["V", "K"],
                    help="cycle of the learned arms and their training pairs (default: the workload's cycle)")
    ap.add_argument("--nrhs", type=int, default=0, help="override the workload's RHS count (small profiling cases)")
    ap.add_argument("--krylov", default="fgmres", choices=["fgmres", "bicgstab"])
    ap.add_argument("--no-graph", action="store_true", help="launch the cycles eagerly (no CUDA graphs)")
    ap.add_argument("--no-tune", action="store_true", help="default stencil launch shapes (no autotuning)")
    ap.add_argument("--max-outer", type=int, default=200,
                    help="FGMRES restart cycles (fewer: kernel-rate profiling runs, not a valid RHS/s)")
    ap.add_argument("--cycle", default=None, choices=["V", "W", "K"],
                    help="multigrid cycle (K: two FGMRES steps per coarse level; default: the workload's)")
    ap.add_argument("--coarse", default=None, choices=["galerkin", "rediscretize"],
                    help="coarse-level operators: Galerkin R A P, or the operator re-discretised on each coarse mesh")
    ap.add_argument("--levels", type=int, default=0, help="multigrid levels (0: the workload's)")
    ap.add_argument("--relax", default=None, choices=["jac", "jac-gmres"],
                    help="smoother: damped Jacobi, or GMRES steps preconditioned by a Jacobi sweep (relaxType "
                         "'Jac-GMRES')")
    ap.add_argument("--relax-from", type=int, default=None, help="jac-gmres: first level smoothed by GMRES steps")
    ap.add_argument("--shift", type=float, default=None, help="s of the shifted operator SH = H + i s w^2 diag(m)")
    ap.add_argument("--outer", default="fp64", choices=["fp64", "emulated"],
                    help="learned workload: outer arithmetic of its mixed arms")
    ap.add_argument("--train-models", type=int, default=48, help="learned workload: seeded training models")
    ap.add_argument("--train-rhs", type=int, default=4, help="learned workload: random sources per training model")
    ap.add_argument("--pairs-per-model", type=int, default=None,
                    help="learned workloads: training pairs per seeded model (default: the workload's)")
    ap.add_argument("--train-epochs", type=int, default=20)
    ap.add_argument("--net-level", type=int, default=0, help="learned workload: multigrid level of the network "
                    "(0: the workload's)")
    ap.add_argument("--stag-ratio", type=float, default=0.95,
                    help="learned workload: a restart cycle reducing a residual by less than this hands over "
                         "to the plain cycle")
    args = ap.parse_args()
    resolve_solver_args(args)
    peak, peak_kind = load_peaks()

    if args.impl == "reference":
        run_reference(args)
        return

    rank, ws, dist = dist_setup()
    if WORKLOADS[args.workload].get("learned"):
        run_learned_main(args, rank, ws, dist)
        return
    results, wl, P, B, err_cols, train_info = run_ours(args, rank, ws, dist)
    if rank != 0:
        return
    names = arm_names(args, wl)
    head = results[names[0]]
    # per-kernel rates of the eager profiled solve; the dominant kernel names the roofline
    kt = [k for k in head["kernels"] if k["timed"] > 0]
    tot_ms = sum(k["ms"] for k in kt) or 1.0
    dom = max(kt, key=lambda k: k["ms"]) if kt else None
    roofline = None
    if dom:
        achieved = dom["bytes"] / (dom["ms"] / 1000.0) / 1e9
        prof = profile_entry(dom["name"], args.workload) if args.nrhs == 0 else {}
        ratio = prof.get("dram_over_algorithmic")
        tr = None if ratio is None else ratio * dom["bytes"] / dom["launches"]
        roofline = dict(bound="hbm", kernel=dom["name"], achieved=achieved, peak=peak, unit="GB/s",
                        frac=achieved / peak, peak_source=f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                        traffic=tr, avg_launch_ms=dom["ms"] / dom["timed"], share=dom["ms"] / tot_ms,
                        source="CUDA events around every launch on the handle's stream, over one eager solve "
                               "right after the timed ones")
        f64 = fp64_rate(dom)
        if f64 is not None:
            # the same kernel against GB300's FP64 rate: its algorithmic FP64 flops over the same events
            roofline["fp64"] = f64
        if "fp64_pipe_pct_of_peak" in prof:
            # native-FP64 kernels: GB300's FP64 pipe, not HBM, is the limit
            roofline["fp64_pipe_pct_of_peak_ncu"] = prof["fp64_pipe_pct_of_peak"]
            roofline["note"] = ("FP64 arithmetic: bound by the FP64 pipe (ncu, small case of the same path), "
                                "not by HBM; see profiles/fgmres_fp64_kernels_3d129_kcycle_8rhs.md")
    # whole-solve roofline: the algorithmic bytes of every launched kernel of a solve over
    # the unprofiled time of a solve
    solve_bytes = sum(k["bytes"] for k in head["kernels"])
    solve_roof = dict(bound="hbm", achieved=solve_bytes / (head["ms_per_step"] / 1e3) / 1e9, peak=peak, unit="GB/s",
                      frac=solve_bytes / (head["ms_per_step"] / 1e3) / 1e9 / peak, bytes_per_solve=solve_bytes)
    # error against an FP64 oracle, and the CPU baseline
    errs, err_info, cpu = {}, None, None
    if P["dim"] == 2:
        errs, err_info = direct_errors(wl, P, B, err_cols, results)
    if not args.no_cpu:
        orc = OracleSolver(wl, P, args)
        b0 = B[:, :1]
        X1, its, secs, rr1, thr = orc.cycles(b0, wl["tol"], 400)
        t1 = float(sum(secs))
        cpu = dict(value=1.0 / t1, unit="RHS/s", cores=thr, kind="port",
                   sample=f"column 0 of the {wl['nrhs']} right-hand sides of the same workload solved to "
                          f"{wl['tol']:g} ({its} iterations, {len(secs)} restart cycles timed one by one), full grid, "
                          f"same operator, {orc.desc}",
                   seconds=t1, setup_s=orc.setup_s, max_relres=rr1, iterations=its)
        if P["dim"] == 3:
            # continue column 0 to 1e-10: the FP64 oracle solution the arms' errors are taken against
            Xr, its2, secs2, rr2, _ = orc.cycles(b0, 1e-10, 400, X0=X1)
            xr = Xr[:, 0]
            for name, res in results.items():
                xg = res["x_err_cols"][0]
                errs[name] = float(np.linalg.norm(xg - xr) / np.linalg.norm(xr))
            err_info = dict(kind="C oracle FP64 FGMRES-SLMG solve (same cycle) to rel. residual 1e-10",
                            columns=[0], oracle_relres=rr2, oracle_iterations=its + its2)
    plain = results.get("fp64")
    emu = results.get("mixed_emulated")

    def arm_summary(r, name):
        return dict(precision=r["precision"], outer_arithmetic=r["outer_arithmetic"], learned=r["learned"],
                    cycle=r["cycle"], rhs_per_s=r["rhs_per_s"], ms_per_step=r["ms_per_step"], steps=r["steps"], warmup=r["warmup"],
                    mean_iters=r["mean_iters"], max_iters=r["max_iters"], max_relres=r["max_relres"],
                    converged_cols=r["converged_cols"], max_err_vs_oracle=errs.get(name),
                    net_calls=r["net_calls"], net_fallbacks=r["net_fallbacks"], clocks=r["clocks"],
                    device_gb_in_use=r.get("device_gb"))

    def over_plain(name):
        r = results.get(name)
        return None if (r is None or plain is None) else r["rhs_per_s"] / plain["rhs_per_s"]

    line = dict(metric=METRIC, value=head["rhs_per_s"], unit="RHS/s", n_gpus=ws, steps=args.steps,
                warmup=args.warmup, ms_per_step=head["ms_per_step"], higher_is_better=True, scaling="weak",
                vs_baseline=None,
                dtype=("c64 cycle" + (" + bf16 network" if head["learned"] else "") + " / c128 outer" +
                       (" (emulated by FP32 pairs)" if head["outer_arithmetic"] == "emulated" else "")
                       if head["precision"] == "mixed" else "c128"),
                data="synthetic (seeded layered+ellipsoid model)" if P["dim"] == 3 else "synthetic (seeded model)",
                config=dict(run_config(args, wl, P), precision=head["precision"],
                            outer_arithmetic=head["outer_arithmetic"], cuda_graph=not args.no_graph,
                            autotune=not args.no_tune, learned=bool(head["learned"]),
                            net_level=wl.get("net_level") if head["learned"] else None),
                e2e=head.get("e2e"), gpu_launches=head["launches_per_step"] * args.steps,
                clocks=head["clocks"], roofline=roofline, solve_roofline=solve_roof,
                cpu_baseline=cpu,
                max_relres=head["max_relres"], check_relres_max=head.get("check_relres_max"),
                converged_cols=head["converged_cols"], mean_iters=head["mean_iters"],
                max_err_vs_oracle=errs.get(names[0]), err_oracle=err_info,
                device_gb_in_use=head.get("device_gb"),
                arms={nm: arm_summary(r, nm) for nm, r in results.items()},
                plain_fp64=None if plain is None else arm_summary(plain, "fp64"),
                headline_over_plain=over_plain(names[0]),
                learned_over_plain_fp64=over_plain("learned_mixed"),
                mixed_over_plain=over_plain("mixed"),
                emulated_outer=None if emu is None else arm_summary(emu, "mixed_emulated"),
                emulated_over_plain=over_plain("mixed_emulated"),
                learned_emulated_over_plain=over_plain("learned_emulated"),
                training=train_info,
                kernels=kernel_rows(kt, peak, tot_ms),
                kernels_source="one eager solve (cycle kernels launched one by one) after the timed solves")
    print(json.dumps(line))


def run_reference(args):
    """The reference arm: the C oracle port of the reference's SLMG path (Julia
    and Multigrid.jl are absent), plain FP64 on all host threads, on the same
    workload and config.  One step = one restart cycle (10 FGMRES iterations)
    of the current column of the workload; a column that converges hands over
    to the next one.  RHS/s = (iterations per second over the timed cycles) /
    (iterations per right-hand side of the columns solved)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = workload(args)
    P = make_problem(wl, seed=1234)
    B = sources(P, wl["nrhs"], seed=0)
    orc = OracleSolver(wl, P, args)
    col, X = 0, None
    solved_iters, cur_iters = [], 0
    t_steps, it_steps = [], []
    thr = 1
    for step in range(args.warmup + args.steps):
        b = B[:, col:col + 1]
        X, its, secs, rr, thr = orc.cycles(b, wl["tol"], 1, X0=X)
        cur_iters += its
        if step >= args.warmup:
            t_steps.append(secs[0])
            it_steps.append(its)
        if rr <= wl["tol"]:
            solved_iters.append(cur_iters)
            col, X, cur_iters = (col + 1) % wl["nrhs"], None, 0
    if not solved_iters:
        # no column finished within the steps: finish the current one (untimed) for its iteration count
        b = B[:, col:col + 1]
        X, its, _, rr, _ = orc.cycles(b, wl["tol"], 400, X0=X)
        solved_iters.append(cur_iters + its)
    ips = sum(it_steps) / sum(t_steps)
    per_rhs = float(np.mean(solved_iters))
    v = ips / per_rhs
    line = dict(metric=METRIC, value=v, unit="RHS/s", impl="reference", n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=1000.0 * sum(t_steps) / len(t_steps), higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="c128",
                data="synthetic (seeded layered+ellipsoid model)" if P["dim"] == 3 else "synthetic (seeded model)",
                config=dict(run_config(args, wl, P), precision="fp64", outer_arithmetic="fp64", cuda_graph=False,
                            autotune=False, learned=False, net_level=None),
                cpu_baseline=dict(value=v, unit="RHS/s", cores=thr, kind="port",
                                  sample=f"one restart cycle (10 FGMRES iterations) of one column per step, full "
                                         f"grid, {orc.desc}; {per_rhs:.0f} iterations per right-hand side "
                                         f"({len(solved_iters)} column(s) solved to {wl['tol']:g})",
                                  setup_s=orc.setup_s),
                e2e=dict(value=v, unit="RHS/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                iterations_per_s=ips, iterations_per_rhs=per_rhs,
                note="reference path = the C oracle port of the Julia SLMG (Julia and Multigrid.jl are absent); "
                     "it imports nothing of the product")
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# Learned coarse correction workload (2D)
# ---------------------------------------------------------------------------
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
        d = hz.learned.collect_pairs(S, B, level=level, sweeps=2, max_pairs=args.pairs_per_model or 200)
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




def run_learned_main(args, rank, ws, dist):
    res, info, wl = run_learned(args, rank, ws, dist)
    if rank != 0:
        return
    head = res["learned_mixed"]
    # the metric counts right-hand sides solved to the tolerance: columns that
    # did not converge within the restart limit count as time spent, not as solved
    line = dict(metric=METRIC, value=head["converged_rhs_per_s"], unit="RHS/s", n_gpus=ws, steps=args.steps,
                warmup=args.warmup, ms_per_step=head["ms_per_step"], higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="c64 cycle + bf16 network / c128 outer",
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


if __name__ == "__main__":
    main()
