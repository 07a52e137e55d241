"""Compile the C oracle (oracle/slmg_cpu.c) into oracle/_build/libslmg_cpu.so.

TEST INFRASTRUCTURE ONLY: the C oracle is the checker and the CPU baseline;
the product never links it.  Portable C99 + OpenMP (no ISA-specific flags),
so it builds the same on x86_64 and aarch64.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "slmg_cpu.c"
OUT = HERE / "_build" / "libslmg_cpu.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if force or not OUT.exists() or OUT.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["gcc", "-std=c99", "-O3", "-fPIC", "-shared", "-fopenmp", "-o", str(OUT), str(SRC), "-lm"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"C oracle build failed:\n{r.stdout}")
    return OUT


if __name__ == "__main__":
    print(build(force=True))
