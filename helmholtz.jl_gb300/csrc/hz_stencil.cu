// Multigrid kernels: matrix-free fine-level Helmholtz stencil, Galerkin
// coarse-level stencils, damped Jacobi, full-weighting restriction,
// bi/trilinear prolongation, the banded coarsest solve and the setup kernels.
//
// Replaces the sparse assembly + ParSpMatVec SpMV of the reference
// (src/GetHelmholtz.jl:33-50, 85-95; src/PlainNodalLaplacian.jl:18-46) and
// the Multigrid.jl relaxation / transfer / coarse-solve steps called from
// src/ShiftedLaplacianMultigridSolver.jl:89.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>

#include <cooperative_groups.h>

#include "hz_launch.cuh"
#include "hz_rap_tile.cuh"

namespace cg = cooperative_groups;

namespace hz {

// ---------------------------------------------------------------------------
// Launch bookkeeping
// ---------------------------------------------------------------------------
int Ctx::name_id(const char* name) {
  for (size_t i = 0; i < names.size(); ++i)
    if (names[i] == name) return (int)i;
  names.emplace_back(name);
  counts.push_back(0);
  timed.push_back(0);
  total_ms.push_back(0.0);
  alg_bytes.push_back(0.0);
  alg_flops.push_back(0.0);
  return (int)names.size() - 1;
}

void Ctx::before(int id, cudaEvent_t* a) {
  (void)id;
  if (!profile) return;
  if (pool.empty()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    pool.push_back(e);
  }
  *a = pool.back();
  pool.pop_back();
  cudaEventRecord(*a, stream);
}

void Ctx::after(int id, cudaEvent_t a, double bytes) {
  ++launches;
  counts[id] += 1;
  alg_bytes[id] += bytes;
  if (!profile) return;
  cudaEvent_t b;
  if (pool.empty()) {
    cudaEventCreate(&b);
  } else {
    b = pool.back();
    pool.pop_back();
  }
  cudaEventRecord(b, stream);
  pending.push_back({id, a, b});
}

void Ctx::resolve() {
  for (auto& p : pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      timed[p.id] += 1;
      total_ms[p.id] += ms;
    }
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  pending.clear();
}

void Ctx::release() {
  resolve();
  for (auto e : pool) cudaEventDestroy(e);
  pool.clear();
}


// ---------------------------------------------------------------------------
// Fine-level stencil
// ---------------------------------------------------------------------------
template <typename T> struct FineOpT {
  int nx, ny, nz;
  long long N;
  T o[3], b[3];
  int adj;
};

// Off-diagonal magnitudes of the two neighbours of node i on an axis of n
// nodes.  Row i of the 1D operator is (2u_i - u_{i-1} - u_{i+1})/h^2 inside and
// (BC u_0 - BC u_1)/h^2, (BC u_{n-1} - BC u_{n-2})/h^2 on the boundary rows
// (src/PlainNodalLaplacian.jl:18-30).  The adjoint takes entry (j, i).
template <typename T>
__device__ __forceinline__ void axis_coef(int i, int n, T o, T bb, int adj, T& cl, T& cr) {
  if (!adj) {
    cl = (i > 0) ? ((i == n - 1) ? bb : o) : T(0);
    cr = (i < n - 1) ? ((i == 0) ? bb : o) : T(0);
  } else {
    cl = (i > 0) ? ((i - 1 == 0) ? bb : o) : T(0);
    cr = (i < n - 1) ? ((i + 1 == n - 1) ? bb : o) : T(0);
  }
}

template <typename T, typename TX, typename TB, int MODE, bool IS3D>
__global__ void __launch_bounds__(256) k_fine(FineOpT<T> op, const cplx<T>* __restrict__ diag,
                                              const cplx<T>* __restrict__ dinv, const cplx<TX>* __restrict__ x,
                                              const cplx<TB>* __restrict__ b, cplx<T>* __restrict__ y, long long ld,
                                              const int* __restrict__ cols, int ncols, int cpb, T w) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= op.N) return;
  const int nx = op.nx, ny = op.ny;
  const int i = (int)(p % nx);
  const long long t = p / nx;
  const int j = (int)(t % ny);
  const int k = (int)(t / ny);
  T cxl, cxr, cyl, cyr, czl = 0, czr = 0;
  axis_coef<T>(i, nx, op.o[0], op.b[0], op.adj, cxl, cxr);
  axis_coef<T>(j, ny, op.o[1], op.b[1], op.adj, cyl, cyr);
  if (IS3D) axis_coef<T>(k, op.nz, op.o[2], op.b[2], op.adj, czl, czr);
  // clamped neighbour offsets: a missing neighbour has a zero coefficient
  const long long sx = 1, sy = nx, sz = (long long)nx * ny;
  const long long oxl = (i > 0) ? -sx : 0, oxr = (i < nx - 1) ? sx : 0;
  const long long oyl = (j > 0) ? -sy : 0, oyr = (j < ny - 1) ? sy : 0;
  long long ozl = 0, ozr = 0;
  if (IS3D) {
    ozl = (k > 0) ? -sz : 0;
    ozr = (k < op.nz - 1) ? sz : 0;
  }
  cplx<T> d = diag[p];
  if (op.adj) d.y = -d.y;
  cplx<T> di = mk<T>(0, 0);
  if (MODE == MODE_JACOBI) {
    di = dinv[p];
    if (op.adj) di.y = -di.y;
  }
  const int c0 = blockIdx.y * cpb;
  const int c1 = min(ncols, c0 + cpb);
  // columns are independent: unrolled so that several columns' loads are in flight
#pragma unroll 4
  for (int ci = c0; ci < c1; ++ci) {
    const long long off = (long long)cols[ci] * ld;
    const cplx<TX>* xc = x + off + p;
    const cplx<T> xp = ccast<T, TX>(xc[0]);
    const cplx<T> a = ccast<T, TX>(xc[oxl]), bq = ccast<T, TX>(xc[oxr]);
    const cplx<T> c = ccast<T, TX>(xc[oyl]), e = ccast<T, TX>(xc[oyr]);
    T sr = cxl * a.x + cxr * bq.x + cyl * c.x + cyr * e.x;
    T si = cxl * a.y + cxr * bq.y + cyl * c.y + cyr * e.y;
    if (IS3D) {
      const cplx<T> f = ccast<T, TX>(xc[ozl]), g = ccast<T, TX>(xc[ozr]);
      sr += czl * f.x + czr * g.x;
      si += czl * f.y + czr * g.y;
    }
    cplx<T> ax = mk<T>(-sr, -si);
    ax = cfma<T>(d, xp, ax);
    // b is read once and y written once: streaming hints keep the cache for the
    // x planes whose neighbours are read again
    if (MODE == MODE_APPLY) {
      __stcs(&y[off + p], ax);
    } else {
      const cplx<TB> bb = __ldcs(&b[off + p]);
      const cplx<T> r = mk<T>((T)bb.x - ax.x, (T)bb.y - ax.y);
      if (MODE == MODE_RESID) {
        __stcs(&y[off + p], r);
      } else {
        const cplx<T> dr = cmul<T>(di, r);
        __stcs(&y[off + p], mk<T>(xp.x + w * dr.x, xp.y + w * dr.y));
      }
    }
  }
}

template <typename T, typename TX, typename TB>
void launch_fine(Ctx& ctx, int mode, const FineOp& op, const cplx<T>* diag, const cplx<T>* dinv, const cplx<TX>* x,
                 const cplx<TB>* b, cplx<T>* y, long long ld, const int* cols, int ncols, double w) {
  if (ncols <= 0) return;
  FineOpT<T> o;
  o.nx = op.g.nx;
  o.ny = op.g.ny;
  o.nz = op.g.nz;
  o.N = op.g.N;
  for (int d = 0; d < 3; ++d) {
    o.o[d] = (T)op.o[d];
    o.b[d] = (T)op.b[d];
  }
  o.adj = op.adj;
  const int TPB = 256;
  long long nbx = (op.g.N + TPB - 1) / TPB;
  int ch = ctx.tune_fine > 0 ? chunks_for(nbx, ncols, ctx.tune_fine) : chunks_for(nbx, ncols);
  int cpb = (ncols + ch - 1) / ch;
  dim3 grid((unsigned)nbx, (unsigned)ch);
  const bool is3d = op.g.nz > 1;
  // x (and b) read and y written once per active column, the diagonal (and
  // its inverse) once per node
  double fbytes = (double)op.g.N * ncols * (sizeof(cplx<TX>) + sizeof(cplx<T>)) + (double)op.g.N * sizeof(cplx<T>);
  if (mode != MODE_APPLY) fbytes += (double)op.g.N * ncols * sizeof(cplx<TB>);
  if (mode == MODE_JACOBI) fbytes += (double)op.g.N * sizeof(cplx<T>);
#define HZ_FINE_CASE(M, D, NAME) \
  HZ_LAUNCH(ctx, NAME, fbytes, (k_fine<T, TX, TB, M, D>), grid, TPB, 0, o, diag, dinv, x, b, y, ld, cols, ncols, cpb, (T)w)
  const char* nm_apply = op.outer ? "outer_apply" : "fine_apply";
  const char* nm_resid = op.outer ? "outer_resid" : "fine_resid";
  // FP64 arithmetic of the Krylov method's operator, per node and column: a multiply
  // and an add per component of each real-coefficient neighbour, 8 flops for the
  // complex diagonal, 2 for b - H x
  if (op.outer && std::is_same<T, double>::value && mode != MODE_JACOBI)
    ctx.add_flops(mode == MODE_APPLY ? nm_apply : nm_resid,
                  (8.0 * (is3d ? 3 : 2) + 8.0 + (mode == MODE_RESID ? 2.0 : 0.0)) * (double)op.g.N * ncols);
  if (mode == MODE_APPLY) {
    if (is3d) HZ_FINE_CASE(MODE_APPLY, true, nm_apply);
    else HZ_FINE_CASE(MODE_APPLY, false, nm_apply);
  } else if (mode == MODE_RESID) {
    if (is3d) HZ_FINE_CASE(MODE_RESID, true, nm_resid);
    else HZ_FINE_CASE(MODE_RESID, false, nm_resid);
  } else {
    if (is3d) HZ_FINE_CASE(MODE_JACOBI, true, "fine_jacobi");
    else HZ_FINE_CASE(MODE_JACOBI, false, "fine_jacobi");
  }
#undef HZ_FINE_CASE
}

// ---------------------------------------------------------------------------
// Galerkin (stored-coefficient) stencil
// ---------------------------------------------------------------------------
template <typename T, typename TB, int MODE, bool IS3D>
__global__ void __launch_bounds__(128) k_rap(Grid g, const cplx<T>* __restrict__ coef, long long cld,
                                             const cplx<T>* __restrict__ dinv, const cplx<T>* __restrict__ x,
                                             const cplx<TB>* __restrict__ b, cplx<T>* __restrict__ y, long long ld,
                                             const int* __restrict__ cols, int ncols, int cpb, T w) {
  constexpr int NS = IS3D ? 27 : 9;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.N) return;
  const int nx = g.nx, ny = g.ny;
  const int i = (int)(p % nx);
  const long long t = p / nx;
  const int j = (int)(t % ny);
  const int k = (int)(t / ny);
  const long long sy = nx, sz = (long long)nx * ny;
  const long long dxo[3] = {(i > 0) ? -1LL : 0LL, 0LL, (i < nx - 1) ? 1LL : 0LL};
  const long long dyo[3] = {(j > 0) ? -sy : 0LL, 0LL, (j < ny - 1) ? sy : 0LL};
  long long dzo[3] = {0, 0, 0};
  if (IS3D) {
    dzo[0] = (k > 0) ? -sz : 0;
    dzo[2] = (k < g.nz - 1) ? sz : 0;
  }
  cplx<T> c[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    c[s] = coef[s * cld + p];
  }
  cplx<T> di = mk<T>(0, 0);
  if (MODE == MODE_JACOBI) di = dinv[p];
  const int c0 = blockIdx.y * cpb;
  const int c1 = min(ncols, c0 + cpb);
  // columns are independent: unrolled so that several columns' loads are in flight
#pragma unroll 2
  for (int ci = c0; ci < c1; ++ci) {
    const long long off = (long long)cols[ci] * ld;
    const cplx<T>* xc = x + off + p;
    cplx<T> ax = mk<T>(0, 0);
    cplx<T> xp = mk<T>(0, 0);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const long long o = dxo[s % 3] + dyo[(s / 3) % 3] + (IS3D ? dzo[s / 9] : 0LL);
      const cplx<T> v = xc[o];
      if (s == NS / 2) xp = v;
      ax = cfma<T>(c[s], v, ax);
    }
    // b read once, y written once: streaming hints, as in k_fine
    if (MODE == MODE_APPLY) {
      __stcs(&y[off + p], ax);
    } else {
      const cplx<TB> bb = __ldcs(&b[off + p]);
      const cplx<T> r = mk<T>((T)bb.x - ax.x, (T)bb.y - ax.y);
      if (MODE == MODE_RESID) {
        __stcs(&y[off + p], r);
      } else {
        const cplx<T> dr = cmul<T>(di, r);
        __stcs(&y[off + p], mk<T>(xp.x + w * dr.x, xp.y + w * dr.y));
      }
    }
  }
}

// The 3D Galerkin stencil of the complex-FP32 cycle on staged tiles (the steps
// and the layout are in hz_rap_tile.cuh); the same outputs, bit for bit, as k_rap.
template <typename TB, int MODE>
__global__ void __launch_bounds__(kRtThreads) k_rap_tile(Grid g, const float2* __restrict__ coef, long long cld,
                                                         const float2* __restrict__ dinv,
                                                         const float2* __restrict__ x, const cplx<TB>* __restrict__ b,
                                                         float2* __restrict__ y, long long ld,
                                                         const int* __restrict__ cols, int ncols, float w) {
  __shared__ float2 sm[kRtSmemElems];
  const RapTileCta t = rap_tile_cta(g, blockIdx.x, blockIdx.y, blockIdx.z, ncols);
  const int tid = threadIdx.x;
  rap_tile_load<float>(t, tid, t.z0 - 1, x, ld, cols, sm);
  rap_tile_load<float>(t, tid, t.z0, x, ld, cols, sm);
  for (int z = t.z0; z < t.z1; ++z) {
    // plane z + 1 takes the slot of plane z - 2, free since the barrier closing the last step
    rap_tile_load<float>(t, tid, z + 1, x, ld, cols, sm);
    __syncthreads();
    rap_tile_node<float, TB, MODE>(t, tid, z, coef, cld, dinv, b, y, ld, cols, sm, w);
    __syncthreads();
  }
}

template <typename TB>
void launch_rap_tile(Ctx& ctx, int mode, const Grid& g, const float2* coef, long long cld, const float2* dinv,
                     const float2* x, const cplx<TB>* b, float2* y, long long ld, const int* cols, int ncols, double w,
                     double bytes) {
  int bx, by, bz;
  rap_tile_grid(g, ncols, bx, by, bz);
  const dim3 grid((unsigned)bx, (unsigned)by, (unsigned)bz);
  if (mode == MODE_APPLY)
    HZ_LAUNCH(ctx, "rap_tile_apply", bytes, (k_rap_tile<TB, MODE_APPLY>), grid, kRtThreads, 0, g, coef, cld, dinv, x,
              b, y, ld, cols, ncols, (float)w);
  else if (mode == MODE_RESID)
    HZ_LAUNCH(ctx, "rap_tile_resid", bytes, (k_rap_tile<TB, MODE_RESID>), grid, kRtThreads, 0, g, coef, cld, dinv, x,
              b, y, ld, cols, ncols, (float)w);
  else
    HZ_LAUNCH(ctx, "rap_tile_jacobi", bytes, (k_rap_tile<TB, MODE_JACOBI>), grid, kRtThreads, 0, g, coef, cld, dinv,
              x, b, y, ld, cols, ncols, (float)w);
}

template <typename T, typename TB>
void launch_rap(Ctx& ctx, int mode, const Grid& g, const cplx<T>* coef, long long cld, const cplx<T>* dinv,
                const cplx<T>* x, const cplx<TB>* b, cplx<T>* y, long long ld, const int* cols, int ncols, double w) {
  if (ncols <= 0) return;
  const int TPB = 128;
  long long nbx = (g.N + TPB - 1) / TPB;
  int ch = ctx.tune_rap > 0 ? chunks_for(nbx, ncols, ctx.tune_rap) : chunks_for(nbx, ncols);
  int cpb = (ncols + ch - 1) / ch;
  dim3 grid((unsigned)nbx, (unsigned)ch);
  const bool is3d = g.nz > 1;
  const int ns = is3d ? 27 : 9;
  double rbytes = (double)g.N * ncols * 2 * sizeof(cplx<T>) + (double)g.N * ns * sizeof(cplx<T>);
  if (mode != MODE_APPLY) rbytes += (double)g.N * ncols * sizeof(cplx<TB>);
  if (mode == MODE_JACOBI) rbytes += (double)g.N * sizeof(cplx<T>);
  if constexpr (std::is_same<T, float>::value) {
    if (is3d && ctx.rap_tiled) {
      launch_rap_tile<TB>(ctx, mode, g, coef, cld, dinv, x, b, y, ld, cols, ncols, w, rbytes);
      return;
    }
  }
#define HZ_RAP_CASE(M, D, NAME) \
  HZ_LAUNCH(ctx, NAME, rbytes, (k_rap<T, TB, M, D>), grid, TPB, 0, g, coef, cld, dinv, x, b, y, ld, cols, ncols, cpb, (T)w)
  if (mode == MODE_APPLY) {
    if (is3d) HZ_RAP_CASE(MODE_APPLY, true, "rap_apply");
    else HZ_RAP_CASE(MODE_APPLY, false, "rap_apply");
  } else if (mode == MODE_RESID) {
    if (is3d) HZ_RAP_CASE(MODE_RESID, true, "rap_resid");
    else HZ_RAP_CASE(MODE_RESID, false, "rap_resid");
  } else {
    if (is3d) HZ_RAP_CASE(MODE_JACOBI, true, "rap_jacobi");
    else HZ_RAP_CASE(MODE_JACOBI, false, "rap_jacobi");
  }
#undef HZ_RAP_CASE
}

// ---------------------------------------------------------------------------
// First Jacobi sweep from a zero guess: y = w dinv b
// ---------------------------------------------------------------------------
template <typename T, typename TB>
__global__ void __launch_bounds__(256) k_jacobi0(long long N, const cplx<T>* __restrict__ dinv, int adj,
                                                 const cplx<TB>* __restrict__ b, cplx<T>* __restrict__ y, long long ld,
                                                 const int* __restrict__ cols, int ncols, int cpb, T w) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  cplx<T> di = dinv[p];
  if (adj) di.y = -di.y;
  di.x *= w;
  di.y *= w;
  const int c0 = blockIdx.y * cpb;
  const int c1 = min(ncols, c0 + cpb);
  // columns are independent: unrolled so that several columns' loads are in flight
#pragma unroll 4
  for (int ci = c0; ci < c1; ++ci) {
    const long long off = (long long)cols[ci] * ld;
    const cplx<TB> bb = b[off + p];
    y[off + p] = cmul<T>(di, mk<T>((T)bb.x, (T)bb.y));
  }
}

template <typename T, typename TB>
void launch_jacobi0(Ctx& ctx, const Grid& g, const cplx<T>* dinv, int adj, const cplx<TB>* b, cplx<T>* y, long long ld,
                    const int* cols, int ncols, double w) {
  if (ncols <= 0) return;
  const int TPB = 256;
  long long nbx = (g.N + TPB - 1) / TPB;
  int ch = chunks_for(nbx, ncols);
  int cpb = (ncols + ch - 1) / ch;
  dim3 grid((unsigned)nbx, (unsigned)ch);
  const double jbytes = (double)g.N * ncols * (sizeof(cplx<TB>) + sizeof(cplx<T>)) + (double)g.N * sizeof(cplx<T>);
  HZ_LAUNCH(ctx, "jacobi0", jbytes, (k_jacobi0<T, TB>), grid, TPB, 0, g.N, dinv, adj, b, y, ld, cols, ncols, cpb, (T)w);
}

// ---------------------------------------------------------------------------
// Transfers
// ---------------------------------------------------------------------------
template <typename T, bool IS3D>
__global__ void __launch_bounds__(256) k_restrict(Grid gf, Grid gc, const cplx<T>* __restrict__ rf, long long ldf,
                                                  cplx<T>* __restrict__ rc, long long ldc, const int* __restrict__ cols,
                                                  int ncols, int cpb) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= gc.N) return;
  const int I = (int)(q % gc.nx);
  const long long t = q / gc.nx;
  const int J = (int)(t % gc.ny);
  const int K = (int)(t / gc.ny);
  const int fi = 2 * I, fj = 2 * J, fk = 2 * K;
  const long long sy = gf.nx, sz = (long long)gf.nx * gf.ny;
  const long long pc = fi + fj * sy + (IS3D ? fk * sz : 0);
  // weights of the three fine nodes per axis; a missing node has weight 0
  const T wx[3] = {(fi > 0) ? T(0.5) : T(0), T(1), (fi < gf.nx - 1) ? T(0.5) : T(0)};
  const T wy[3] = {(fj > 0) ? T(0.5) : T(0), T(1), (fj < gf.ny - 1) ? T(0.5) : T(0)};
  T wz[3] = {T(0), T(1), T(0)};
  if (IS3D) {
    wz[0] = (fk > 0) ? T(0.5) : T(0);
    wz[2] = (fk < gf.nz - 1) ? T(0.5) : T(0);
  }
  const long long ox[3] = {(fi > 0) ? -1LL : 0LL, 0LL, (fi < gf.nx - 1) ? 1LL : 0LL};
  const long long oy[3] = {(fj > 0) ? -sy : 0LL, 0LL, (fj < gf.ny - 1) ? sy : 0LL};
  long long oz[3] = {0, 0, 0};
  if (IS3D) {
    oz[0] = (fk > 0) ? -sz : 0;
    oz[2] = (fk < gf.nz - 1) ? sz : 0;
  }
  const T scale = IS3D ? T(0.125) : T(0.25);
  const int c0 = blockIdx.y * cpb;
  const int c1 = min(ncols, c0 + cpb);
  // columns are independent: unrolled so that several columns' loads are in flight
#pragma unroll 4
  for (int ci = c0; ci < c1; ++ci) {
    const int col = cols[ci];
    const cplx<T>* r = rf + (long long)col * ldf + pc;
    T ar = 0, ai = 0;
#pragma unroll
    for (int c = 0; c < (IS3D ? 3 : 1); ++c) {
#pragma unroll
      for (int bq = 0; bq < 3; ++bq) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const T wgt = wx[a] * wy[bq] * (IS3D ? wz[c] : T(1));
          const cplx<T> v = r[ox[a] + oy[bq] + (IS3D ? oz[c] : 0LL)];
          ar += wgt * v.x;
          ai += wgt * v.y;
        }
      }
    }
    rc[(long long)col * ldc + q] = mk<T>(scale * ar, scale * ai);
  }
}

template <typename T>
void launch_restrict(Ctx& ctx, const Grid& gf, const Grid& gc, const cplx<T>* rf, long long ldf, cplx<T>* rc,
                     long long ldc, const int* cols, int ncols) {
  if (ncols <= 0) return;
  const int TPB = 256;
  long long nbx = (gc.N + TPB - 1) / TPB;
  int ch = chunks_for(nbx, ncols);
  int cpb = (ncols + ch - 1) / ch;
  dim3 grid((unsigned)nbx, (unsigned)ch);
  const double tbytes = (double)ncols * (gf.N + gc.N) * sizeof(cplx<T>);
  if (gf.nz > 1)
    HZ_LAUNCH(ctx, "restrict", tbytes, (k_restrict<T, true>), grid, TPB, 0, gf, gc, rf, ldf, rc, ldc, cols, ncols, cpb);
  else
    HZ_LAUNCH(ctx, "restrict", tbytes, (k_restrict<T, false>), grid, TPB, 0, gf, gc, rf, ldf, rc, ldc, cols, ncols, cpb);
}

template <typename T, bool IS3D>
__global__ void __launch_bounds__(256) k_prolong(Grid gf, Grid gc, const cplx<T>* __restrict__ ec, long long ldc,
                                                 const cplx<T>* xin, cplx<T>* xout, long long ldf,
                                                 const int* __restrict__ cols, int ncols, int cpb) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= gf.N) return;
  const int i = (int)(p % gf.nx);
  const long long t = p / gf.nx;
  const int j = (int)(t % gf.ny);
  const int k = (int)(t / gf.ny);
  // Parent pair per axis: (i>>1, (i+1)>>1).  An even fine index has both
  // entries equal to its single parent, an odd one has its two neighbours, so
  // a uniform weight of 1/2 per axis is exact linear interpolation.
  const long long sy = gc.nx, sz = (long long)gc.nx * gc.ny;
  const long long a0 = i >> 1, a1 = (i + 1) >> 1;
  const long long b0 = (long long)(j >> 1) * sy, b1 = (long long)((j + 1) >> 1) * sy;
  const long long z0 = IS3D ? (long long)(k >> 1) * sz : 0, z1 = IS3D ? (long long)((k + 1) >> 1) * sz : 0;
  const T wgt = IS3D ? T(0.125) : T(0.25);
  const int c0 = blockIdx.y * cpb;
  const int c1 = min(ncols, c0 + cpb);
  // columns are independent: unrolled so that several columns' loads are in flight
#pragma unroll 4
  for (int ci = c0; ci < c1; ++ci) {
    const int col = cols[ci];
    const cplx<T>* e = ec + (long long)col * ldc;
    cplx<T> v0 = e[z0 + b0 + a0], v1 = e[z0 + b0 + a1], v2 = e[z0 + b1 + a0], v3 = e[z0 + b1 + a1];
    T ar = (v0.x + v1.x) + (v2.x + v3.x);
    T ai = (v0.y + v1.y) + (v2.y + v3.y);
    if (IS3D) {
      cplx<T> u0 = e[z1 + b0 + a0], u1 = e[z1 + b0 + a1], u2 = e[z1 + b1 + a0], u3 = e[z1 + b1 + a1];
      ar += (u0.x + u1.x) + (u2.x + u3.x);
      ai += (u0.y + u1.y) + (u2.y + u3.y);
    }
    const long long o = (long long)col * ldf + p;
    // the fine vector is read and written once (streaming); the coarse one stays cached
    const cplx<T> base = xin ? __ldcs(&xin[o]) : mk<T>(0, 0);
    __stcs(&xout[o], mk<T>(base.x + wgt * ar, base.y + wgt * ai));
  }
}

template <typename T>
void launch_prolong(Ctx& ctx, const Grid& gf, const Grid& gc, const cplx<T>* ec, long long ldc, const cplx<T>* xin,
                    cplx<T>* xout, long long ldf, const int* cols, int ncols) {
  if (ncols <= 0) return;
  const int TPB = 256;
  long long nbx = (gf.N + TPB - 1) / TPB;
  int ch = chunks_for(nbx, ncols);
  int cpb = (ncols + ch - 1) / ch;
  dim3 grid((unsigned)nbx, (unsigned)ch);
  const double pbytes = (double)ncols * (gc.N + (xin ? 2 : 1) * gf.N) * sizeof(cplx<T>);
  if (gf.nz > 1)
    HZ_LAUNCH(ctx, "prolong", pbytes, (k_prolong<T, true>), grid, TPB, 0, gf, gc, ec, ldc, xin, xout, ldf, cols, ncols, cpb);
  else
    HZ_LAUNCH(ctx, "prolong", pbytes, (k_prolong<T, false>), grid, TPB, 0, gf, gc, ec, ldc, xin, xout, ldf, cols, ncols, cpb);
}

// ---------------------------------------------------------------------------
// Coarsest level: blocked banded LU solve, FP64 arithmetic.
//
// The host folds each block of kl elimination steps of the band LU (row
// interchanges included) into a dense window operator T_I, and each block of
// the back substitution into G_I = [U_II^{-1} | -U_II^{-1} U_right]; a solve is
// then N/kl sequential window mat-vecs per direction, each spread over the
// whole GPU: one warp per (output row, column), lanes split the window sum.
// ---------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_band_block(long long N, long long s, int Win, int split,
                                                    const double2* __restrict__ M, const double2* __restrict__ src0,
                                                    const cplx<T>* __restrict__ b, long long ldb,
                                                    const int* __restrict__ cols, const double2* __restrict__ src1,
                                                    double2* __restrict__ dst, cplx<T>* __restrict__ xout,
                                                    long long ldx, int ncols) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x;
  const int ci = blockIdx.y * 8 + warp;
  if (ci >= ncols) return;
  const double2* Mr = M + (long long)i * Win;
  const long long base = (long long)ci * N + s;
  double ar = 0.0, ai = 0.0;
  for (int k = lane; k < Win; k += 32) {
    const double2 m = Mr[k];
    double2 v;
    if (k < split) {
      v = src0[base + k];
    } else if (MODE == 0) {
      const cplx<T> bb = b[(long long)cols[ci] * ldb + s + k];
      v = mk<double>((double)bb.x, (double)bb.y);
    } else {
      v = src1[base + k];
    }
    ar = fma(m.x, v.x, ar);
    ar = fma(-m.y, v.y, ar);
    ai = fma(m.x, v.y, ai);
    ai = fma(m.y, v.x, ai);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    ai += __shfl_xor_sync(0xffffffffu, ai, o);
  }
  if (lane == 0) {
    dst[base + i] = mk<double>(ar, ai);
    if (MODE == 1) xout[(long long)cols[ci] * ldx + s + i] = mk<T>((T)ar, (T)ai);
  }
}

// All block steps of the solve in one cooperative launch.  A warp item is one
// row of the current window operator for BCW columns: the row entries are
// loaded once and feed BCW independent accumulators (more loads in flight per
// warp than one column per item).  The grid synchronises between block steps;
// the launch is sized to the co-resident capacity (cudaLaunchCooperativeKernel
// refuses a larger grid rather than deadlocking).
static constexpr int BCW = 1;  // one column per item: more items in flight per step

template <typename T>
__global__ void __launch_bounds__(256) k_band_coop(long long N, int nbk, const BandBlock* __restrict__ blocks,
                                                   const double2* __restrict__ Tops, const double2* __restrict__ Gops,
                                                   const cplx<T>* __restrict__ b, long long ldb,
                                                   const int* __restrict__ cols, int ncols, double2* __restrict__ work,
                                                   cplx<T>* __restrict__ x, long long ldx) {
  cg::grid_group grid = cg::this_grid();
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  double2* const Y0 = work;
  double2* const Y1 = work + (long long)ncols * N;
  double2* const X64 = work + 2LL * ncols * N;
  const int ngrp = (ncols + BCW - 1) / BCW;
  long long prev_end = 0;
  for (int I = 0; I < nbk; ++I) {
    const BandBlock B = blocks[I];
    const int split = (I == 0) ? 0 : (int)(prev_end - B.s);
    const double2* src0 = (I & 1) ? Y0 : Y1;  // output of block I-1
    double2* dst = (I & 1) ? Y1 : Y0;
    const long long items = (long long)B.W * ngrp;
    for (long long it = gw; it < items; it += nw) {
      const int i = (int)(it % B.W), c0 = (int)(it / B.W) * BCW;
      const double2* Mr = Tops + B.toff + (long long)i * B.W;
      double ar[BCW], ai[BCW];
#pragma unroll
      for (int c = 0; c < BCW; ++c) ar[c] = ai[c] = 0.0;
      for (int k = lane; k < B.W; k += 32) {
        const double2 m = Mr[k];
#pragma unroll
        for (int c = 0; c < BCW; ++c) {
          const int ci = c0 + c;
          if (ci < ncols) {
            double2 v;
            if (k < split) {
              v = src0[(long long)ci * N + B.s + k];
            } else {
              const cplx<T> bb = b[(long long)cols[ci] * ldb + B.s + k];
              v = mk<double>((double)bb.x, (double)bb.y);
            }
            ar[c] = fma(m.x, v.x, ar[c]);
            ar[c] = fma(-m.y, v.y, ar[c]);
            ai[c] = fma(m.x, v.y, ai[c]);
            ai[c] = fma(m.y, v.x, ai[c]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < BCW; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          ar[c] += __shfl_xor_sync(0xffffffffu, ar[c], o);
          ai[c] += __shfl_xor_sync(0xffffffffu, ai[c], o);
        }
        if (lane == 0 && c0 + c < ncols) dst[(long long)(c0 + c) * N + B.s + i] = mk<double>(ar[c], ai[c]);
      }
    }
    prev_end = B.s + B.W;
    grid.sync();
  }
  for (int I = nbk - 1; I >= 0; --I) {
    const BandBlock B = blocks[I];
    const double2* yb = (I & 1) ? Y1 : Y0;
    const long long items = (long long)B.nb * ngrp;
    for (long long it = gw; it < items; it += nw) {
      const int i = (int)(it % B.nb), c0 = (int)(it / B.nb) * BCW;
      const double2* Mr = Gops + B.goff + (long long)i * B.Wb;
      double ar[BCW], ai[BCW];
#pragma unroll
      for (int c = 0; c < BCW; ++c) ar[c] = ai[c] = 0.0;
      for (int k = lane; k < B.Wb; k += 32) {
        const double2 m = Mr[k];
#pragma unroll
        for (int c = 0; c < BCW; ++c) {
          const int ci = c0 + c;
          if (ci < ncols) {
            const long long q = (long long)ci * N + B.s + k;
            const double2 v = (k < B.nb) ? yb[q] : X64[q];
            ar[c] = fma(m.x, v.x, ar[c]);
            ar[c] = fma(-m.y, v.y, ar[c]);
            ai[c] = fma(m.x, v.y, ai[c]);
            ai[c] = fma(m.y, v.x, ai[c]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < BCW; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          ar[c] += __shfl_xor_sync(0xffffffffu, ar[c], o);
          ai[c] += __shfl_xor_sync(0xffffffffu, ai[c], o);
        }
        const int ci = c0 + c;
        if (lane == 0 && ci < ncols) {
          X64[(long long)ci * N + B.s + i] = mk<double>(ar[c], ai[c]);
          x[(long long)cols[ci] * ldx + B.s + i] = mk<T>((T)ar[c], (T)ai[c]);
        }
      }
    }
    grid.sync();
  }
}

template <typename T>
void launch_band_solve(Ctx& ctx, const BandSolveOps& op, const cplx<T>* b, cplx<T>* x, long long ld, const int* cols,
                       int ncols, double2* work) {
  if (ncols <= 0) return;
  const long long N = op.N;
  const int nbk = (int)op.blocks.size();
  double bytes = 0.0;
  for (const BandBlock& B : op.blocks)
    bytes += ((double)B.W * B.W + (double)B.nb * B.Wb) * sizeof(double2) +
             ncols * (2.0 * B.W + B.Wb + 2.0 * B.nb) * sizeof(double2);
  if (op.dblocks) {
    // one cooperative launch, grid = co-resident capacity
    static int capacity[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < kMaxDevices && capacity[dev] == 0) {
      int per_sm = 0, sms = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_band_coop<T>, 256, 0);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      capacity[dev] = std::max(1, std::min(per_sm, 4)) * std::max(1, sms);
    }
    const int grid = (dev >= 0 && dev < kMaxDevices) ? capacity[dev] : kSMs;
    static thread_local int id = -1;
    if (id < 0 || (size_t)id >= ctx.names.size() || ctx.names[id] != "band_solve") id = ctx.name_id("band_solve");
    cudaEvent_t ev = nullptr;
    ctx.before(id, &ev);
    const BandBlock* blk = op.dblocks;
    const double2* Tp = op.T;
    const double2* Gp = op.G;
    long long ldb = ld, ldx = ld;
    void* args[] = {(void*)&N,    (void*)&nbk,  (void*)&blk,   (void*)&Tp,   (void*)&Gp, (void*)&b,
                    (void*)&ldb,  (void*)&cols, (void*)&ncols, (void*)&work, (void*)&x,  (void*)&ldx};
    const cudaError_t e =
        cudaLaunchCooperativeKernel((const void*)k_band_coop<T>, dim3(grid), dim3(256), args, 0, ctx.stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw std::runtime_error(std::string("band_solve cooperative launch failed: ") + cudaGetErrorString(e));
    }
    ctx.after(id, ev, bytes);
    return;
  }
  double2* Y[2] = {work, work + (long long)ncols * N};
  double2* X64 = work + 2LL * ncols * N;
  const unsigned gy = (unsigned)((ncols + 7) / 8);
  long long prev_end = 0;
  for (int I = 0; I < nbk; ++I) {
    const BandBlock& B = op.blocks[(size_t)I];
    const int split = (I == 0) ? 0 : (int)(prev_end - B.s);
    const double fb = (double)B.W * B.W * sizeof(double2) + 2.0 * ncols * B.W * sizeof(double2);
    HZ_LAUNCH(ctx, "band_forward", fb, (k_band_block<T, 0>), dim3((unsigned)B.W, gy), 256, 0, N, B.s, B.W, split,
              op.T + B.toff, Y[(I + 1) % 2], b, ld, cols, (const double2*)nullptr, Y[I % 2], (cplx<T>*)nullptr,
              0LL, ncols);
    prev_end = B.s + B.W;
  }
  for (int I = nbk - 1; I >= 0; --I) {
    const BandBlock& B = op.blocks[(size_t)I];
    const double bb = (double)B.nb * B.Wb * sizeof(double2) + ncols * (B.Wb + 2.0 * B.nb) * sizeof(double2);
    HZ_LAUNCH(ctx, "band_backward", bb, (k_band_block<T, 1>), dim3((unsigned)B.nb, gy), 256, 0, N, B.s, B.Wb,
              B.nb, op.G + B.goff, Y[I % 2], (const cplx<T>*)nullptr, 0LL, cols, X64, X64, x, ld, ncols);
  }
}

// ---------------------------------------------------------------------------
// Allocation-free operator apply (hz_apply_noalloc).  The column-index list
// the stencil kernel reads is kept in a file-scope device array instead of a
// per-call allocation.  Host code must not pass the symbol itself to a kernel
// (in host code it is only a host-side stand-in); its device address is looked
// up with cudaGetSymbolAddress once per device, with that device current.
// ---------------------------------------------------------------------------
static __device__ __align__(256) int g_noalloc_cols[kNoAllocMaxCols];

__global__ void k_iota(int* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}

static int* noalloc_cols_address(int dev, std::string* err) {
  static std::mutex mu;
  static int* addr[kNoAllocMaxDevices] = {};
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    *err = "device ordinal out of range for the allocation-free entry point";
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    int* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_cols);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      *err = std::string("cudaGetSymbolAddress of the column-list scratch failed: ") + cudaGetErrorString(e);
      return nullptr;
    }
    addr[dev] = p;
  }
  return addr[dev];
}

int launch_fine_apply_noalloc(cudaStream_t stream, int dev, const FineOp& op, const double2* diag, const double2* x,
                              double2* y, long long ld, int nrhs, std::string* err) {
  if (nrhs < 1 || nrhs > kNoAllocMaxCols) {
    *err = "nrhs must be in [1, " + std::to_string(kNoAllocMaxCols) + "] for the allocation-free apply";
    return -1;
  }
  int* cols = noalloc_cols_address(dev, err);
  if (!cols) return -2;
  // every call rewrites the entries it reads: the array keeps the previous call's contents
  k_iota<<<(nrhs + 255) / 256, 256, 0, stream>>>(cols, nrhs);
  FineOpT<double> o;
  o.nx = op.g.nx;
  o.ny = op.g.ny;
  o.nz = op.g.nz;
  o.N = op.g.N;
  for (int d = 0; d < 3; ++d) {
    o.o[d] = op.o[d];
    o.b[d] = op.b[d];
  }
  o.adj = op.adj;
  const int TPB = 256;
  const long long nbx = (op.g.N + TPB - 1) / TPB;
  const int ch = chunks_for(nbx, nrhs);
  const int cpb = (nrhs + ch - 1) / ch;
  const dim3 grid((unsigned)nbx, (unsigned)ch);
  if (op.g.nz > 1)
    k_fine<double, double, double, MODE_APPLY, true><<<grid, TPB, 0, stream>>>(
        o, diag, nullptr, x, (const double2*)nullptr, y, ld, cols, nrhs, cpb, 0.0);
  else
    k_fine<double, double, double, MODE_APPLY, false><<<grid, TPB, 0, stream>>>(
        o, diag, nullptr, x, (const double2*)nullptr, y, ld, cols, nrhs, cpb, 0.0);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *err = std::string("allocation-free apply launch failed: ") + cudaGetErrorString(e);
    return -2;
  }
  return 0;
}

// explicit instantiations
#define HZ_INST_T_TB(T, TB)                                                                                        \
  template void launch_fine<T, T, TB>(Ctx&, int, const FineOp&, const cplx<T>*, const cplx<T>*, const cplx<T>*,     \
                                      const cplx<TB>*, cplx<T>*, long long, const int*, int, double);               \
  template void launch_rap<T, TB>(Ctx&, int, const Grid&, const cplx<T>*, long long, const cplx<T>*,                \
                                  const cplx<T>*, const cplx<TB>*, cplx<T>*, long long, const int*, int, double);   \
  template void launch_jacobi0<T, TB>(Ctx&, const Grid&, const cplx<T>*, int, const cplx<TB>*, cplx<T>*, long long, \
                                      const int*, int, double);
HZ_INST_T_TB(double, double)
HZ_INST_T_TB(float, float)
HZ_INST_T_TB(float, double)
HZ_INST_T_TB(float, df64_tag)
template void launch_fine<double, float, double>(Ctx&, int, const FineOp&, const double2*, const double2*,
                                                 const float2*, const double2*, double2*, long long, const int*, int,
                                                 double);
#undef HZ_INST_T_TB
template void launch_restrict<double>(Ctx&, const Grid&, const Grid&, const double2*, long long, double2*, long long,
                                      const int*, int);
template void launch_restrict<float>(Ctx&, const Grid&, const Grid&, const float2*, long long, float2*, long long,
                                     const int*, int);
template void launch_prolong<double>(Ctx&, const Grid&, const Grid&, const double2*, long long, const double2*,
                                     double2*, long long, const int*, int);
template void launch_prolong<float>(Ctx&, const Grid&, const Grid&, const float2*, long long, const float2*, float2*,
                                    long long, const int*, int);
template void launch_band_solve<double>(Ctx&, const BandSolveOps&, const double2*, double2*, long long, const int*, int,
                                        double2*);
template void launch_band_solve<float>(Ctx&, const BandSolveOps&, const float2*, float2*, long long, const int*, int,
                                       double2*);

}  // namespace hz
