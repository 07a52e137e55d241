"""The exact FP32 -> FP64 widening of the FP64 kernels (widen_f32_bits in
csrc/hz_common.cuh) against the host compiler's conversion, for every one of
the 2^32 FP32 bit patterns: the fast path must give the same bits wherever it
applies, and it must decline exactly the zero, subnormal, infinite and NaN
patterns.  Compiled with g++ from the library's own header (no GPU)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "helmholtz.jl_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <cstring>
#include "hz_common.cuh"
int main() {
  unsigned long long fast = 0, bad = 0;
  for (unsigned long long k = 0; k <= 0xffffffffull; ++k) {
    const uint32_t u = (uint32_t)k;
    float f;
    std::memcpy(&f, &u, 4);
    const uint32_t a = u & 0x7fffffffu;
    const bool special = a < 0x00800000u || a >= 0x7f800000u;
    uint32_t hi = 0, lo = 0;
    const bool ok = hz::widen_f32_bits(u, hi, lo);
    if (ok == special) { ++bad; continue; }
    if (!ok) continue;
    ++fast;
    const double d = (double)f;
    uint64_t bits;
    std::memcpy(&bits, &d, 8);
    if (bits != (((uint64_t)hi << 32) | lo)) ++bad;
  }
  std::printf("%llu %llu\n", fast, bad);
  return bad != 0;
}
"""


def test_widen_f32_bits_is_exact_for_every_pattern(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "widen.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "widen"
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run([gxx, "-O2", "-std=c++17", f"-I{CSRC}", f"-I{cuda_inc}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    fast, bad = map(int, out.stdout.split())
    assert bad == 0
    assert fast == 2 * (0x7f800000 - 0x00800000)  # every normal number of either sign
