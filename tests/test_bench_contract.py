"""The benchmark's reference arm (the CPU restatement of the reference's SLMG
solve on the host cores) prints one JSON line with the contract's keys; run on
the smallest workload so it finishes in seconds without a GPU."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "c1",
                          "--steps", "1", "--warmup", "0", "--cpu-budget", "2"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "higher_is_better", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "RHS/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    # the sample never counts more columns than the workload has
    assert line["cpu_baseline"]["sample"].startswith("1 of the 1 ")


def test_reference_arm_follows_the_solver_options():
    """The reference arm runs the GPU arm's cycle, coarse operators, smoother and
    level count, and names them in its config and sample."""
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "c1",
                          "--steps", "1", "--warmup", "0", "--cpu-budget", "2", "--cycle", "K",
                          "--coarse", "rediscretize", "--relax", "jac-gmres", "--relax-from", "1", "--levels", "2"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    cfg = line["config"]
    assert (cfg["cycle"], cfg["coarse"], cfg["relax"], cfg["relax_from"], cfg["levels"]) == \
        ("K", "rediscretize", "jac-gmres", 1, 2)
    assert "K-cycle, rediscretize coarse levels, Jac-GMRES smoothing from level 1" in line["cpu_baseline"]["sample"]
    assert line["value"] > 0
