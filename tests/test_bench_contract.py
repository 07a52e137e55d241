"""The benchmark's reference arm (the CPU restatement of the reference's SLMG
solve on the host cores) prints one JSON line with the contract's keys, the
same config keys as the GPU arm, and loads nothing of the product; run on the
smallest workload so it finishes in seconds without a GPU."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

# run bench.py's reference arm in this interpreter, then report whether any
# module or shared library of the product was loaded
_PROBE = r"""
import runpy, sys, json
sys.argv = ["bench.py"] + sys.argv[1:]
runpy.run_path("bench.py", run_name="__main__")
mods = [m for m in sys.modules if m.startswith("helmholtz_jl_gb300")]
maps = open("/proc/self/maps").read()
print(json.dumps({"product_modules": mods, "libhelmgpu_loaded": "libhelmgpu" in maps}))
"""

CONFIG_KEYS = {"workload", "nrhs", "levels", "tol", "krylov", "cycle", "coarse", "relax", "relax_from", "shift",
               "seed", "learned", "l2", "precision", "outer_arithmetic", "cuda_graph", "autotune", "net_level"}


def _run(*extra):
    out = subprocess.run([sys.executable, "-c", _PROBE, "--impl", "reference", "--workload", "c1", "--steps", "2",
                          "--warmup", "1", *extra], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    return json.loads(lines[-2]), json.loads(lines[-1])


def test_reference_arm_json_line():
    line, probe = _run()
    for key in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "higher_is_better", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "RHS/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["sample"].startswith("one restart cycle")
    assert line["iterations_per_rhs"] > 0 and line["iterations_per_s"] > 0
    # the same config keys as the GPU arm's line
    assert set(line["config"]) == CONFIG_KEYS
    # the reference arm runs nothing of the product
    assert probe == {"product_modules": [], "libhelmgpu_loaded": False}


def test_reference_arm_follows_the_solver_options():
    """The reference arm runs the GPU arm's cycle, coarse operators, smoother and
    level count, and names them in its config and sample."""
    line, _ = _run("--cycle", "K", "--coarse", "rediscretize", "--relax", "jac-gmres", "--relax-from", "1",
                   "--levels", "2")
    cfg = line["config"]
    assert (cfg["cycle"], cfg["coarse"], cfg["relax"], cfg["relax_from"], cfg["levels"]) == \
        ("K", "rediscretize", "jac-gmres", 1, 2)
    assert "K-cycle, rediscretize coarse levels, Jac-GMRES smoothing from level 1" in line["cpu_baseline"]["sample"]
    assert line["value"] > 0


def test_workload_defaults_fill_the_solver_options():
    """The 3D 257^3 workload runs the K-cycle with GMRES smoothing from level 1 and
    shift 0.3 unless the command line says otherwise; the others keep the V-cycle."""
    sys.path.insert(0, str(ROOT))
    import argparse
    import bench
    a = argparse.Namespace(workload="c5", cycle=None, relax=None, relax_from=None, shift=None, coarse=None)
    bench.resolve_solver_args(a)
    assert (a.cycle, a.relax, a.relax_from, a.shift, a.coarse) == ("K", "jac-gmres", 1, 0.3, "galerkin")
    b = argparse.Namespace(workload="c2", cycle="W", relax=None, relax_from=None, shift=None, coarse=None)
    bench.resolve_solver_args(b)
    assert (b.cycle, b.relax, b.shift) == ("W", "jac", 0.5)
    assert bench.DEFAULT_WORKLOAD == "c5"


def test_kernel_rows_rate_the_fp64_and_tensor_kernels():
    """The per-kernel table gives every row its HBM rate; the native-FP64 outer
    kernels (flops counted by the library) also their FP64 rate against GB300's
    nominal FP64 peak, the tensor-core kernels their TFLOP/s; rows without flops
    (memory-bound kernels, the emulated form's kernels of the same names) neither."""
    sys.path.insert(0, str(ROOT))
    import bench
    kt = [dict(name="krylov_dots", launches=10, timed=10, ms=1000.0, bytes=2.0e12, flops=1.0e12),
          dict(name="net3_conv_fwd_tc", launches=4, timed=4, ms=10.0, bytes=1.0e9, flops=1.0e12),
          dict(name="fine_jacobi", launches=5, timed=5, ms=100.0, bytes=5.0e11, flops=0.0),
          dict(name="krylov_update", launches=5, timed=5, ms=500.0, bytes=3.0e12, flops=0.0)]
    rows = {r["name"]: r for r in bench.kernel_rows(kt, 6000.0, 1610.0)}
    assert [r["name"] for r in bench.kernel_rows(kt, 6000.0, 1610.0)] == \
        ["krylov_dots", "krylov_update", "fine_jacobi", "net3_conv_fwd_tc"]
    d = rows["krylov_dots"]
    assert abs(d["gbs"] - 2000.0) < 1e-9 and abs(d["frac"] - 2000.0 / 6000.0) < 1e-12
    assert abs(d["fp64_tflops"] - 1.0) < 1e-12 and abs(d["fp64_frac"] - 1.0 / bench.FP64_PEAK_TFLOPS) < 1e-12
    assert "tflops" not in d
    assert abs(rows["net3_conv_fwd_tc"]["tflops"] - 100.0) < 1e-9 and "fp64_frac" not in rows["net3_conv_fwd_tc"]
    for name in ("fine_jacobi", "krylov_update"):
        assert "tflops" not in rows[name] and "fp64_frac" not in rows[name]
    f = bench.fp64_rate(kt[0])
    assert f["unit"] == "TFLOP/s" and f["peak"] == bench.FP64_PEAK_TFLOPS and abs(f["frac"] - 0.8) < 1e-12
    assert bench.fp64_rate(kt[1]) is None and bench.fp64_rate(dict(kt[0], ms=0.0)) is None
