"""The staged-tile Galerkin stencil (k_rap_tile, csrc/hz_rap_tile.cuh) emulated
on the host: every thread of every CTA runs the kernel's own load and compute
steps in the order its barriers impose, with every shared-memory index checked.
Its outputs must equal, bit for bit, k_rap's formula (the 27 clamped neighbours
summed in k_rap's order) restated here, for every mode, both right-hand-side
precisions, grids with partial tiles and z-ranges, and a permuted, partial
column list.  Compiled with g++ from the library's own headers (no GPU)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "helmholtz.jl_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include "hz_rap_tile.cuh"
using namespace hz;

// k_rap's value for node p of column offset off (csrc/hz_stencil.cu), restated
template <typename T, typename TB, int MODE>
cplx<T> rap_ref(const Grid& g, long long p, const cplx<T>* coef, long long cld, const cplx<T>* dinv,
                const cplx<T>* x, const cplx<TB>* b, long long off, T w) {
  const int i = (int)(p % g.nx);
  const long long t = p / g.nx;
  const int j = (int)(t % g.ny), k = (int)(t / g.ny);
  const long long sy = g.nx, sz = (long long)g.nx * g.ny;
  const long long dxo[3] = {i > 0 ? -1LL : 0LL, 0LL, i < g.nx - 1 ? 1LL : 0LL};
  const long long dyo[3] = {j > 0 ? -sy : 0LL, 0LL, j < g.ny - 1 ? sy : 0LL};
  const long long dzo[3] = {k > 0 ? -sz : 0LL, 0LL, k < g.nz - 1 ? sz : 0LL};
  cplx<T> ax = mk<T>(0, 0), xp = mk<T>(0, 0);
  for (int s = 0; s < 27; ++s) {
    const cplx<T> v = x[off + p + dxo[s % 3] + dyo[(s / 3) % 3] + dzo[s / 9]];
    if (s == 13) xp = v;
    ax = cfma<T>(coef[s * cld + p], v, ax);
  }
  if (MODE == MODE_APPLY) return ax;
  const cplx<TB> bb = b[off + p];
  const cplx<T> r = mk<T>((T)bb.x - ax.x, (T)bb.y - ax.y);
  if (MODE == MODE_RESID) return r;
  const cplx<T> dr = cmul<T>(dinv[p], r);
  return mk<T>(xp.x + w * dr.x, xp.y + w * dr.y);
}

template <typename TB, int MODE>
long long run(int nx, int ny, int nz, unsigned seed) {
  typedef float T;
  const Grid g{nx, ny, nz, (long long)nx * ny * nz};
  const int ntot = 13;                                   // columns of the block
  const int cols_h[11] = {12, 0, 5, 3, 9, 1, 11, 7, 2, 10, 6};  // the active ones, permuted
  const int ncols = 11;
  const long long ld = g.N + 7, cld = g.N + 3;
  std::mt19937 rng(seed);
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  std::vector<cplx<T>> coef(27 * cld), dinv(g.N), x(ntot * ld), yref(ntot * ld), yt(ntot * ld);
  std::vector<cplx<TB>> b(ntot * ld);
  for (auto& v : coef) v = mk<T>(u(rng), u(rng));
  for (auto& v : dinv) v = mk<T>(u(rng), u(rng));
  for (auto& v : x) v = mk<T>(u(rng), u(rng));
  for (auto& v : b) { v.x = u(rng); v.y = u(rng); }
  for (long long e = 0; e < ntot * ld; ++e) yref[e] = yt[e] = mk<T>(12345.f, -54321.f);  // untouched marker
  const T w = 0.8f;
  for (int c = 0; c < ncols; ++c)
    for (long long p = 0; p < g.N; ++p)
      yref[(long long)cols_h[c] * ld + p] =
          rap_ref<T, TB, MODE>(g, p, coef.data(), cld, dinv.data(), x.data(), b.data(), (long long)cols_h[c] * ld, w);
  int bx, by, bz;
  rap_tile_grid(g, ncols, bx, by, bz);
  std::vector<cplx<T>> sm(kRtSmemElems);
  for (int k = 0; k < bz; ++k)
    for (int j = 0; j < by; ++j)
      for (int i = 0; i < bx; ++i) {
        const RapTileCta t = rap_tile_cta(g, i, j, k, ncols);
        rap_tile_emulate_cta<T, TB, MODE>(t, coef.data(), cld, dinv.data(), x.data(), b.data(), yt.data(), ld,
                                          cols_h, sm.data(), w);
      }
  long long bad = 0;
  for (long long e = 0; e < ntot * ld; ++e)
    if (std::memcmp(&yref[e], &yt[e], sizeof(cplx<T>)) != 0) ++bad;
  return bad;
}

int main() {
  const int grids[][3] = {{17, 17, 17}, {33, 9, 40}, {9, 5, 3}, {65, 7, 33}, {3, 3, 3}, {40, 6, 17}, {5, 13, 1}};
  long long bad = 0;
  int cases = 0;
  for (const auto& gd : grids) {
    const unsigned s = 1000u * gd[0] + 10u * gd[1] + gd[2];
    bad += run<float, MODE_APPLY>(gd[0], gd[1], gd[2], s);
    bad += run<float, MODE_RESID>(gd[0], gd[1], gd[2], s + 1);
    bad += run<float, MODE_JACOBI>(gd[0], gd[1], gd[2], s + 2);
    bad += run<double, MODE_RESID>(gd[0], gd[1], gd[2], s + 3);
    bad += run<double, MODE_JACOBI>(gd[0], gd[1], gd[2], s + 4);
    cases += 5;
  }
  std::printf("%d %lld\n", cases, bad);
  return bad != 0;
}
"""


def test_staged_tile_stencil_matches_k_rap_bit_for_bit(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "rap_tile.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "rap_tile"
    r = subprocess.run([gxx, "-O1", "-std=c++17", f"-I{CSRC}", f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include",
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, (out.stdout, out.stderr[-2000:])
    cases, bad = map(int, out.stdout.split())
    assert cases == 35 and bad == 0
