// Galerkin (stored-coefficient) 27-point stencil of a 3D coarse level with the
// right-hand sides' values staged in shared memory (complex-FP32 cycle).
//
// The unstaged kernel (k_rap) reads the 27 neighbours of a node from global
// memory for every column, so each value crosses L1/L2 27 times.  Here a CTA
// owns a tile of 32 x 4 nodes of the x-y plane, a range of up to 16 z-planes and
// up to 8 columns.  It keeps the planes z - 1, z and z + 1 of its tile plus a
// one-node halo for each column in a ring of three shared-memory planes.  It
// marches along z, loading one new plane per step, and holds a node's 27
// coefficients in registers across the columns.  Neighbours outside the grid
// are clamped to the node itself exactly as k_rap clamps them, and the 27 terms
// are summed in k_rap's order, so both kernels give the same bits.
//
// The per-thread steps are __host__ __device__ functions: the kernel runs them
// with a barrier between the load and compute steps, and a host emulation runs
// them for every thread of every CTA in the same order, checking every
// shared-memory index.
#pragma once

#include <assert.h>

#include "hz_common.cuh"
#include "hz_kernels.cuh"

namespace hz {

constexpr int kRtX = 32, kRtY = 4;       // nodes of a tile in x and y: one per thread
constexpr int kRtThreads = kRtX * kRtY;  // 128
constexpr int kRtZ = 16;                 // z-planes per CTA
constexpr int kRtC = 8;                  // columns per CTA
constexpr int kRtHX = kRtX + 2, kRtHY = kRtY + 2;
constexpr int kRtPlane = kRtHX * kRtHY;  // staged nodes of one plane of one column (204)
constexpr int kRtRing = 3;               // planes z - 1, z, z + 1
constexpr int kRtSmemElems = kRtC * kRtRing * kRtPlane;

#ifdef __CUDA_ARCH__
#define HZ_RT_CHECK(cond) ((void)0)
#else
#define HZ_RT_CHECK(cond) assert(cond)
#endif

// streaming loads and stores on the device (b read once, y written once), plain ones on the host
template <typename V> __host__ __device__ __forceinline__ V rt_ld_stream(const V* p) {
#ifdef __CUDA_ARCH__
  return __ldcs(p);
#else
  return *p;
#endif
}
template <typename V> __host__ __device__ __forceinline__ void rt_st_stream(V* p, V v) {
#ifdef __CUDA_ARCH__
  __stcs(p, v);
#else
  *p = v;
#endif
}

// the work of one CTA
struct RapTileCta {
  Grid g;
  int x0, y0;  // tile origin
  int z0, z1;  // z-planes [z0, z1)
  int c0, nc;  // first entry of the column list and the number of columns (<= kRtC)
};

__host__ __device__ __forceinline__ int rt_min(int a, int b) { return a < b ? a : b; }

// grid: x = tiles of the x-y plane, y = z-ranges, z = column groups
__host__ __device__ inline void rap_tile_grid(const Grid& g, int ncols, int& bx, int& by, int& bz) {
  bx = ((g.nx + kRtX - 1) / kRtX) * ((g.ny + kRtY - 1) / kRtY);
  by = (g.nz + kRtZ - 1) / kRtZ;
  bz = (ncols + kRtC - 1) / kRtC;
}

__host__ __device__ inline RapTileCta rap_tile_cta(const Grid& g, int bx, int by, int bz, int ncols) {
  const int tiles_x = (g.nx + kRtX - 1) / kRtX;
  RapTileCta t;
  t.g = g;
  t.x0 = (bx % tiles_x) * kRtX;
  t.y0 = (bx / tiles_x) * kRtY;
  t.z0 = by * kRtZ;
  t.z1 = rt_min(g.nz, t.z0 + kRtZ);
  t.c0 = bz * kRtC;
  t.nc = rt_min(kRtC, ncols - t.c0);
  return t;
}

// ring slot of plane z (z >= -1)
__host__ __device__ __forceinline__ int rap_tile_slot(int z) { return (z + 3) % kRtRing; }

// Thread tid's share of staging plane zp of every column of the CTA: the tile
// plus its halo, zeros outside the grid (never read: neighbours are clamped).
template <typename T>
__host__ __device__ inline void rap_tile_load(const RapTileCta& t, int tid, int zp, const cplx<T>* __restrict__ x,
                                              long long ld, const int* __restrict__ cols, cplx<T>* sm) {
  const int slot = rap_tile_slot(zp);
  const bool zin = zp >= 0 && zp < t.g.nz;
  for (int e = tid; e < t.nc * kRtPlane; e += kRtThreads) {
    const int c = e / kRtPlane, r = e - c * kRtPlane;
    const int hy = r / kRtHX, hx = r - hy * kRtHX;
    const int gx = t.x0 - 1 + hx, gy = t.y0 - 1 + hy;
    cplx<T> v = mk<T>(0, 0);
    if (zin && gx >= 0 && gx < t.g.nx && gy >= 0 && gy < t.g.ny)
      v = x[(long long)cols[t.c0 + c] * ld + ((long long)zp * t.g.ny + gy) * t.g.nx + gx];
    const int k = (c * kRtRing + slot) * kRtPlane + r;
    HZ_RT_CHECK(k >= 0 && k < kRtSmemElems);
    sm[k] = v;
  }
}

// Thread tid's node of plane z for every column of the CTA: the 27-point sum in
// k_rap's order with k_rap's clamped neighbours, then the mode's output.
template <typename T, typename TB, int MODE>
__host__ __device__ inline void rap_tile_node(const RapTileCta& t, int tid, int z, const cplx<T>* __restrict__ coef,
                                              long long cld, const cplx<T>* __restrict__ dinv,
                                              const cplx<TB>* __restrict__ b, cplx<T>* __restrict__ y, long long ld,
                                              const int* __restrict__ cols, const cplx<T>* sm, T w) {
  const int tx = tid % kRtX, ty = tid / kRtX;
  const int i = t.x0 + tx, j = t.y0 + ty;
  if (i >= t.g.nx || j >= t.g.ny) return;
  const long long p = ((long long)z * t.g.ny + j) * t.g.nx + i;
  // staged offsets of the (dx, dy, dz) = (-1, 0, +1) neighbours; a missing one is the node itself
  const int hx[3] = {tx + (i > 0 ? 0 : 1), tx + 1, tx + (i < t.g.nx - 1 ? 2 : 1)};
  const int hy[3] = {(ty + (j > 0 ? 0 : 1)) * kRtHX, (ty + 1) * kRtHX, (ty + (j < t.g.ny - 1 ? 2 : 1)) * kRtHX};
  const int pz[3] = {rap_tile_slot(z > 0 ? z - 1 : z) * kRtPlane, rap_tile_slot(z) * kRtPlane,
                     rap_tile_slot(z < t.g.nz - 1 ? z + 1 : z) * kRtPlane};
  cplx<T> c[27];
#pragma unroll
  for (int s = 0; s < 27; ++s) c[s] = coef[s * cld + p];
  cplx<T> di = mk<T>(0, 0);
  if (MODE == MODE_JACOBI) di = dinv[p];
  for (int ci = 0; ci < t.nc; ++ci) {
    const cplx<T>* sc = sm + ci * kRtRing * kRtPlane;
    const long long off = (long long)cols[t.c0 + ci] * ld;
    cplx<T> ax = mk<T>(0, 0);
    cplx<T> xp = mk<T>(0, 0);
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int k = pz[s / 9] + hy[(s / 3) % 3] + hx[s % 3];
      HZ_RT_CHECK(k >= 0 && k < kRtRing * kRtPlane);
      const cplx<T> v = sc[k];
      if (s == 13) xp = v;
      ax = cfma<T>(c[s], v, ax);
    }
    if (MODE == MODE_APPLY) {
      rt_st_stream(&y[off + p], ax);
    } else {
      const cplx<TB> bb = rt_ld_stream(&b[off + p]);
      const cplx<T> r = mk<T>((T)bb.x - ax.x, (T)bb.y - ax.y);
      if (MODE == MODE_RESID) {
        rt_st_stream(&y[off + p], r);
      } else {
        const cplx<T> dr = cmul<T>(di, r);
        rt_st_stream(&y[off + p], mk<T>(xp.x + w * dr.x, xp.y + w * dr.y));
      }
    }
  }
}

// One CTA's whole sequence for thread tid on the host: every step for every
// thread before the next step, which is what the kernel's barriers give.
template <typename T, typename TB, int MODE>
inline void rap_tile_emulate_cta(const RapTileCta& t, const cplx<T>* coef, long long cld, const cplx<T>* dinv,
                                 const cplx<T>* x, const cplx<TB>* b, cplx<T>* y, long long ld, const int* cols,
                                 cplx<T>* sm, T w) {
  for (int tid = 0; tid < kRtThreads; ++tid) rap_tile_load<T>(t, tid, t.z0 - 1, x, ld, cols, sm);
  for (int tid = 0; tid < kRtThreads; ++tid) rap_tile_load<T>(t, tid, t.z0, x, ld, cols, sm);
  for (int z = t.z0; z < t.z1; ++z) {
    for (int tid = 0; tid < kRtThreads; ++tid) rap_tile_load<T>(t, tid, z + 1, x, ld, cols, sm);
    for (int tid = 0; tid < kRtThreads; ++tid)
      rap_tile_node<T, TB, MODE>(t, tid, z, coef, cld, dinv, b, y, ld, cols, sm, w);
  }
}

}  // namespace hz
