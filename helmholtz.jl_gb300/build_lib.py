"""Build the helmgpu CUDA library (libhelmgpu.so) in-tree for sm_103a.

Every translation unit is compiled in parallel with nvcc (host C++ with g++
through nvcc), then linked into ``helmholtz.jl_gb300/libhelmgpu.so``.  The
objects go to ``helmholtz.jl_gb300/_build/`` (git-ignored).  Rebuilds only
what changed (source or header newer than the object).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhelmgpu.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"]
SOURCES = ["hz_stencil.cu", "hz_krylov.cu", "hz_df64.cu", "hz_kcycle.cu", "hz_learn.cu", "hz_learn3d.cu",
           "hz_conv_tc.cu", "hz_solver.cu", "hz_host.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    procs = []
    objs = []
    for s in SOURCES:
        src = CSRC / s
        obj = BUILD / (s.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]
            if src.suffix == ".cpp":
                cmd = [nvcc] + NVCC_FLAGS + ["-x", "c++", "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((s, out))
        elif verbose and out.strip():
            print(out, file=sys.stderr)
    if failed:
        msg = "\n".join(f"--- {s} ---\n{o}" for s, o in failed)
        raise RuntimeError(f"helmgpu build failed:\n{msg}")
    if force or procs or not LIB.exists():
        cmd = [nvcc] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + \
              ["-Xcompiler", "-fopenmp", "-lgomp", "-lcudart"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"helmgpu link failed:\n{r.stdout}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
