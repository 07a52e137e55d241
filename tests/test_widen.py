"""The exact FP32 -> FP64 widening of the FP64 kernels (widen_f32_bits in
csrc/hz_common.cuh, integer operations only) against the host compiler's
conversion, for every one of the 2^32 FP32 bit patterns: normal, subnormal,
zero, infinite and NaN inputs must all give the host's bits (NaNs quiet, with
their payload).  Compiled with g++ from the library's own header (no GPU)."""
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
  unsigned long long checked = 0, bad = 0, sub = 0, nan = 0;
  for (unsigned long long k = 0; k <= 0xffffffffull; ++k) {
    const uint32_t u = (uint32_t)k;
    float f;
    std::memcpy(&f, &u, 4);
    const uint32_t a = u & 0x7fffffffu;
    sub += (a != 0 && a < 0x00800000u);
    nan += (a > 0x7f800000u);
    const volatile float fv = f;  // the host's conversion, not folded away
    const double d = (double)fv;
    uint64_t bits;
    std::memcpy(&bits, &d, 8);
    ++checked;
    if (bits != hz::widen_f32_bits(u)) {
      if (bad < 5) std::fprintf(stderr, "%08x: %016llx vs %016llx\n", u, (unsigned long long)bits,
                                (unsigned long long)hz::widen_f32_bits(u));
      ++bad;
    }
  }
  std::printf("%llu %llu %llu %llu\n", checked, bad, sub, nan);
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
    checked, bad, sub, nan = map(int, out.stdout.split())
    assert bad == 0, out.stderr
    assert checked == 2**32
    assert sub == 2 * (0x00800000 - 1) and nan == 2 * (0x7fffffff - 0x7f800000)
