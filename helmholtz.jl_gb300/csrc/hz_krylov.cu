// FP64 FGMRES kernels (Arnoldi with classical Gram-Schmidt, Givens rotations,
// least squares, solution update) batched over the active right-hand-side
// columns, plus the multigrid setup kernels (Galerkin probing, coefficient
// transpose, casts).
//
// Replaces solveGMRES_MG of Multigrid.jl / KrylovMethods.jl called at
// src/ShiftedLaplacianMultigridSolver.jl:89 and the RAP products of MGsetup
// (src/ShiftedLaplacianMultigridSolver.jl:64-65).
#include <algorithm>

#include "hz_launch.cuh"

namespace hz {

static constexpr int KG = 16;  // dot products carried per pass in registers

// sqrt of a reduced sum of squares: rounding can leave it a hair below zero;
// NaN and Inf pass through so the host sees a corrupted column.
__device__ __forceinline__ double safe_sqrt(double v) { return (v > 0.0 || v != v) ? sqrt(v) : 0.0; }
static constexpr int RT = 256; // threads per reduction CTA

int krylov_nblk(long long N, int ncols) {
  long long target = 4LL * kSMs * 2;  // ~8 CTAs of 256 threads per SM in total
  long long nb = (target + ncols - 1) / std::max(ncols, 1);
  long long maxb = (N + RT - 1) / RT;
  nb = std::max(1LL, std::min(nb, maxb));
  return (int)nb;
}

// Block-wide sums of nv complex values (v[0..nv)) and, when want_norm, one
// real value; thread s writes slot s of this block's partials:
// part[s*nblk + blockIdx.x] (the norm goes to slot nv).
template <int NV>
__device__ __forceinline__ void block_reduce_store(const double2 (&v)[NV], int nv, double nrm, int want_norm,
                                                   double2* part, int nblk) {
  __shared__ double2 red[RT / 32][NV + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < NV; ++s) {
    if (s < nv) {
      double a = v[s].x, b = v[s].y;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
      }
      if (lane == 0) red[warp][s] = mk<double>(a, b);
    }
  }
  if (want_norm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
    if (lane == 0) red[warp][NV] = mk<double>(nrm, 0.0);
  }
  __syncthreads();
  const int tot = nv + want_norm;
  if (threadIdx.x < tot) {
    const int src = (threadIdx.x < nv) ? threadIdx.x : NV;
    double a = 0, b = 0;
    for (int w = 0; w < RT / 32; ++w) {
      a += red[w][src].x;
      b += red[w][src].y;
    }
    part[(long long)threadIdx.x * nblk + blockIdx.x] = mk<double>(a, b);
  }
}

// Zero partials of a masked-off column (the reduce then yields zeros).
__device__ __forceinline__ void store_zero_partials(int K1, double2* part, int nblk) {
  if (threadIdx.x < K1) part[(long long)threadIdx.x * nblk + blockIdx.x] = mk<double>(0, 0);
}

template <int KT>
__global__ void __launch_bounds__(RT, 2) k_dots(long long N, const double2* __restrict__ V, long long vstride,
                                                long long ld, int i0, const double2* __restrict__ w, long long wld,
                                                const int* __restrict__ cols, const int* __restrict__ mask, int nblk,
                                                int want_norm, double2* __restrict__ part) {
  const int pos = blockIdx.y;
  const int c = cols[pos];
  const int K1 = KT + want_norm;
  double2* pp = part + (long long)pos * K1 * nblk;
  if (mask && !mask[c]) {
    store_zero_partials(K1, pp, nblk);
    return;
  }
  const double2* wc = w + (long long)c * wld;
  const double2* vb = V + ((long long)i0 * vstride + c) * ld;
  const long long vs = vstride * ld;  // distance between consecutive basis vectors
  constexpr int KA = KT > 0 ? KT : 1;  // KT = 0: the norm alone
  double2 acc[KA];
#pragma unroll
  for (int s = 0; s < KA; ++s) acc[s] = mk<double>(0, 0);
  double nrm = 0.0;
  const long long stride = (long long)nblk * RT;
  for (long long p = (long long)blockIdx.x * RT + threadIdx.x; p < N; p += stride) {
    const double2 wv = wc[p];
#pragma unroll
    for (int s = 0; s < KT; ++s) acc[s] = cfma_conj<double>(vb[s * vs + p], wv, acc[s]);
    if (want_norm) nrm = fma(wv.x, wv.x, fma(wv.y, wv.y, nrm));
  }
  block_reduce_store<KA>(acc, KT, nrm, want_norm, pp, nblk);
}

template <int KT>
__global__ void __launch_bounds__(RT, 2) k_update(long long N, const double2* __restrict__ V, long long vstride,
                                                  long long ld, int i0, const double2* __restrict__ h, int hstride,
                                                  double2* __restrict__ w, long long wld,
                                                  const int* __restrict__ cols, const int* __restrict__ mask,
                                                  int nblk, int want_norm, double2* __restrict__ part) {
  const int pos = blockIdx.y;
  const int c = cols[pos];
  double2* pp = part + (long long)pos * want_norm * nblk;
  if (mask && !mask[c]) {
    store_zero_partials(want_norm, pp, nblk);
    return;
  }
  double2 hv[KT];
#pragma unroll
  for (int s = 0; s < KT; ++s) hv[s] = h[(long long)c * hstride + i0 + s];
  const double2* vb = V + ((long long)i0 * vstride + c) * ld;
  const long long vs = vstride * ld;
  double nrm = 0.0;
  double2* wc = w + (long long)c * wld;
  const long long stride = (long long)nblk * RT;
  for (long long p = (long long)blockIdx.x * RT + threadIdx.x; p < N; p += stride) {
    double2 wv = wc[p];
#pragma unroll
    for (int s = 0; s < KT; ++s) wv = cfms<double>(hv[s], vb[s * vs + p], wv);
    wc[p] = wv;
    if (want_norm) nrm = fma(wv.x, wv.x, fma(wv.y, wv.y, nrm));
  }
  if (want_norm) {
    const double2 none[1] = {mk<double>(0, 0)};
    block_reduce_store<1>(none, 0, nrm, 1, pp, nblk);
  }
}

#define HZ_K_CASES(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16)

void launch_dots(Ctx& ctx, long long N, const double2* V, long long vstride, long long ld, int i0, int K,
                 const double2* w, long long wld, const int* cols, int ncols, int nblk, int want_norm, double2* part,
                 const int* mask) {
  if (ncols <= 0) return;
  dim3 grid(nblk, ncols);
  // a masked pass is charged by the host once it knows which columns took it
  const double bytes = mask ? 0.0 : (double)N * ncols * (K + 1) * sizeof(double2);
  // FP64 arithmetic: a complex multiply-add (8 flops) per vector and node, 4 for ||w||^2
  if (!mask) ctx.add_flops("krylov_dots", (double)N * ncols * (8.0 * K + (want_norm ? 4.0 : 0.0)));
  switch (K) {
#define HZ_DOTS_CASE(k)                                                                                     \
  case k:                                                                                                   \
    HZ_LAUNCH(ctx, "krylov_dots", bytes, k_dots<k>, grid, RT, 0, N, V, vstride, ld, i0, w, wld, cols, mask, \
              nblk, want_norm, part);                                                                       \
    break;
    HZ_DOTS_CASE(0)
    HZ_K_CASES(HZ_DOTS_CASE)
#undef HZ_DOTS_CASE
    default:
      throw std::runtime_error("launch_dots: 1..16 vectors per pass");
  }
}

void launch_update(Ctx& ctx, long long N, const double2* V, long long vstride, long long ld, int i0, int K,
                   const double2* h, int hstride, double2* w, long long wld, const int* cols, int ncols, int nblk,
                   int want_norm, double2* part, const int* mask) {
  if (ncols <= 0) return;
  dim3 grid(nblk, ncols);
  const double bytes = mask ? 0.0 : (double)N * ncols * (K + 2) * sizeof(double2);
  if (!mask) ctx.add_flops("krylov_update", (double)N * ncols * (8.0 * K + (want_norm ? 4.0 : 0.0)));
  switch (K) {
#define HZ_UPD_CASE(k)                                                                                           \
  case k:                                                                                                        \
    HZ_LAUNCH(ctx, "krylov_update", bytes, k_update<k>, grid, RT, 0, N, V, vstride, ld, i0, h, hstride, w, wld, \
              cols, mask, nblk, want_norm, part);                                                                \
    break;
    HZ_K_CASES(HZ_UPD_CASE)
#undef HZ_UPD_CASE
    default:
      throw std::runtime_error("launch_update: 1..16 vectors per pass");
  }
}

// DGKS test per column: a second Gram-Schmidt pass is needed when the first
// one removed more than half of the squared norm (||w'||^2 < ||w||^2 / 2).
__global__ void k_dgks(const int* __restrict__ cols, int ncols, const double2* __restrict__ before, int bstride,
                       int bslot, const double2* __restrict__ after, int astride, int* __restrict__ flag) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  const double b = before[(long long)c * bstride + bslot].x;
  const double a = after[(long long)c * astride].x;
  flag[c] = (a < 0.5 * b) ? 1 : 0;
}

void launch_dgks(Ctx& ctx, const int* cols, int ncols, const double2* before, int bstride, int bslot,
                 const double2* after, int astride, int* flag) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "dgks", 0.0, k_dgks, (ncols + 127) / 128, 128, 0, cols, ncols, before, bstride, bslot, after, astride,
            flag);
}

// One warp per (column, slot): fixed-order sum over the nblk partials.
__global__ void k_reduce(const double2* __restrict__ part, const int* __restrict__ cols, int ncols, int K1, int nblk,
                         double2* __restrict__ out, int ostride, int accum) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= ncols * K1) return;
  const int pos = gw / K1, slot = gw % K1;
  const double2* pp = part + ((long long)pos * K1 + slot) * nblk;
  double a = 0, b = 0;
  for (int i = lane; i < nblk; i += 32) {
    a += pp[i].x;
    b += pp[i].y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    double2* dst = out + (long long)cols[pos] * ostride + slot;
    if (accum) {
      a += dst->x;
      b += dst->y;
    }
    *dst = mk<double>(a, b);
  }
}

void launch_reduce(Ctx& ctx, const double2* part, const int* cols, int ncols, int K1, int nblk, double2* out,
                   int ostride, int accum) {
  if (ncols <= 0 || K1 <= 0) return;
  long long warps = (long long)ncols * K1;
  int blocks = (int)((warps * 32 + 255) / 256);
  HZ_LAUNCH(ctx, "krylov_reduce", (double)ncols * K1 * (nblk + 1) * sizeof(double2), k_reduce, blocks, 256, 0, part, cols, ncols, K1, nblk, out, ostride, accum);
}

// ---- deferred normalisation of the FGMRES basis --------------------------------
// The stored basis vector v_i of column c stands for V_i = sig_i v_i with
// sig_i = sig[c*sstride + i] > 0, so no pass over the vector is spent on
// normalising it.  From the stored dots d_i = conj(v_i) . w' of the stored
// candidate w' (= H Z'_j, Z'_j the cycle applied to v_j): the update uses the
// coefficients sig_i^2 d_i, the Hessenberg entries are sig_i sig_j d_i and
// h_{j+1,j} = sig_j ||w''||.
__global__ void k_sig_init(const int* __restrict__ cols, int ncols, double* __restrict__ sig, int sstride) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncols) sig[(long long)cols[i] * sstride] = 1.0;
}

__global__ void k_sig_coef(const int* __restrict__ cols, int ncols, int K, const double* __restrict__ sig, int sstride,
                           const double2* __restrict__ d, int hstride, double2* __restrict__ coef) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncols * K) return;
  const int c = cols[t / K], i = t % K;
  const double s = sig[(long long)c * sstride + i];
  const double2 v = d[(long long)c * hstride + i];
  coef[(long long)c * hstride + i] = mk<double>(s * s * v.x, s * s * v.y);
}

__global__ void k_sig_true(int j, const int* __restrict__ cols, int ncols, const double* __restrict__ sig, int sstride,
                           double2* __restrict__ hA, double2* __restrict__ hB, double2* __restrict__ nr,
                           double2* __restrict__ nr2, int hstride) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  const double* sc = sig + (long long)c * sstride;
  const double sj = sc[j];
  for (int i = 0; i <= j; ++i) {
    const double f = sc[i] * sj;
    double2& a = hA[(long long)c * hstride + i];
    double2& b = hB[(long long)c * hstride + i];
    a = mk<double>(f * a.x, f * a.y);
    b = mk<double>(f * b.x, f * b.y);
  }
  nr[(long long)c * hstride].x *= sj * sj;
  nr2[(long long)c * hstride].x *= sj * sj;
}

__global__ void k_sig_next(int j, const int* __restrict__ cols, int ncols, double* __restrict__ sig, int sstride,
                           const double* __restrict__ invhn) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  sig[(long long)c * sstride + j + 1] = sig[(long long)c * sstride + j] * invhn[c];
}

__global__ void k_sig_y(const int* __restrict__ cols, int ncols, const int* __restrict__ kcol,
                        const double* __restrict__ sig, int sstride, double2* __restrict__ y, int ystride) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  for (int i = 0; i < kcol[c]; ++i) {
    const double s = sig[(long long)c * sstride + i];
    double2& v = y[(long long)c * ystride + i];
    v = mk<double>(s * v.x, s * v.y);
  }
}

void launch_sig_init(Ctx& ctx, const int* cols, int ncols, double* sig, int sstride) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "basis_scale", 0.0, k_sig_init, (ncols + 127) / 128, 128, 0, cols, ncols, sig, sstride);
}
void launch_sig_coef(Ctx& ctx, const int* cols, int ncols, int K, const double* sig, int sstride, const double2* d,
                     int hstride, double2* coef) {
  if (ncols <= 0 || K <= 0) return;
  HZ_LAUNCH(ctx, "basis_scale", 0.0, k_sig_coef, (ncols * K + 127) / 128, 128, 0, cols, ncols, K, sig, sstride, d,
            hstride, coef);
}
void launch_sig_true(Ctx& ctx, int j, const int* cols, int ncols, const double* sig, int sstride, double2* hA,
                     double2* hB, double2* nr, double2* nr2, int hstride) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "basis_scale", 0.0, k_sig_true, (ncols + 127) / 128, 128, 0, j, cols, ncols, sig, sstride, hA, hB, nr,
            nr2, hstride);
}
void launch_sig_next(Ctx& ctx, int j, const int* cols, int ncols, double* sig, int sstride, const double* invhn) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "basis_scale", 0.0, k_sig_next, (ncols + 127) / 128, 128, 0, j, cols, ncols, sig, sstride, invhn);
}
void launch_sig_y(Ctx& ctx, const int* cols, int ncols, const int* kcol, const double* sig, int sstride, double2* y,
                  int ystride) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "basis_scale", 0.0, k_sig_y, (ncols + 127) / 128, 128, 0, cols, ncols, kcol, sig, sstride, y,
            ystride);
}

__global__ void __launch_bounds__(256) k_scale_cols(long long N, const double2* __restrict__ x, long long xld,
                                                    double2* __restrict__ y, long long yld,
                                                    const double* __restrict__ s, const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const double sc = s[c];
  const double2* xc = x + (long long)c * xld;
  double2* yc = y + (long long)c * yld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
    const double2 v = __ldcs(&xc[p]);  // streamed once
    __stcs(&yc[p], mk<double>(sc * v.x, sc * v.y));
  }
}

void launch_scale_cols(Ctx& ctx, long long N, const double2* x, long long xld, double2* y, long long yld,
                       const double* s, const int* cols, int ncols) {
  if (ncols <= 0) return;
  int nb = krylov_nblk(N, ncols);
  dim3 grid(nb, ncols);
  HZ_LAUNCH(ctx, "scale_cols", (double)N * ncols * 2 * sizeof(double2), k_scale_cols, grid, 256, 0, N, x, xld, y, yld, s, cols);
}

template <typename TZ>
__global__ void __launch_bounds__(256) k_update_x(long long N, const cplx<TZ>* __restrict__ Z, long long zstride,
                                                  long long ld, const int* __restrict__ kcol,
                                                  const double2* __restrict__ y, int ystride, double2* __restrict__ x,
                                                  long long xld, const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const int k = kcol[c];
  double2 yv[KG];
#pragma unroll
  for (int s = 0; s < KG; ++s) yv[s] = (s < k) ? y[(long long)c * ystride + s] : mk<double>(0, 0);
  double2* xc = x + (long long)c * xld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
    double2 acc = xc[p];
#pragma unroll
    for (int s = 0; s < KG; ++s) {
      if (s < k) {
        const cplx<TZ> z = Z[((long long)s * zstride + c) * ld + p];
        acc = cfma<double>(yv[s], ccast<double, TZ>(z), acc);
      }
    }
    for (int s = KG; s < k; ++s) {  // restart lengths above KG
      const cplx<TZ> z = Z[((long long)s * zstride + c) * ld + p];
      acc = cfma<double>(y[(long long)c * ystride + s], ccast<double, TZ>(z), acc);
    }
    xc[p] = acc;
  }
}

template <typename TZ>
void launch_update_x(Ctx& ctx, long long N, const cplx<TZ>* Z, long long zstride, long long ld, const int* kcol,
                     const double2* y, int ystride, double2* x, long long xld, const int* cols, int ncols,
                     long long zcols) {
  if (ncols <= 0) return;
  int nb = krylov_nblk(N, ncols);
  dim3 grid(nb, ncols);
  const double bytes = (double)N * (ncols * 2.0 * sizeof(double2) + zcols * sizeof(cplx<TZ>));
  ctx.add_flops("update_x", 8.0 * N * zcols);  // FP64: a complex multiply-add per stored Z vector and node
  HZ_LAUNCH(ctx, "update_x", bytes, k_update_x<TZ>, grid, 256, 0, N, Z, zstride, ld, kcol, y, ystride, x, xld, cols);
}

__global__ void k_norms(const double2* __restrict__ red, int stride, int slot, const int* __restrict__ cols, int ncols,
                        double* __restrict__ nrm, double* __restrict__ inv) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  const double v = safe_sqrt(red[(long long)c * stride + slot].x);
  nrm[c] = v;
  if (inv) inv[c] = (v > 0) ? 1.0 / v : 0.0;
}

void launch_norms(Ctx& ctx, const double2* red, int stride, int slot, const int* cols, int ncols, double* nrm,
                  double* inv) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "krylov_norms", 0.0, k_norms, (ncols + 127) / 128, 128, 0, red, stride, slot, cols, ncols, nrm, inv);
}

__global__ void k_cycle_init(int m, const int* __restrict__ cols, int ncols, const double* __restrict__ beta,
                             double2* __restrict__ g) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  for (int i = 0; i <= m; ++i) g[(long long)c * (m + 1) + i] = mk<double>(i == 0 ? beta[c] : 0.0, 0.0);
}

void launch_cycle_init(Ctx& ctx, int m, const int* cols, int ncols, const double* beta, double2* g) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "cycle_init", 0.0, k_cycle_init, (ncols + 127) / 128, 128, 0, m, cols, ncols, beta, g);
}

// Complex Givens rotation convention: (u, v) -> (conj(c) u + conj(s) v, -s u + c v).
__global__ void k_arnoldi_step(int j, int m, const int* __restrict__ cols, int ncols, const double2* __restrict__ hA,
                               const double2* __restrict__ hB, const double2* __restrict__ nrm,
                               const double2* __restrict__ nrm2, const int* __restrict__ flag, int hstride,
                               double2* __restrict__ Hh, double2* __restrict__ cs, double2* __restrict__ sn,
                               double2* __restrict__ g, double* __restrict__ est, double* __restrict__ inv_hn) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  double2* H = Hh + (long long)c * (m + 1) * m + (long long)j * (m + 1);
  const double2* csc = cs + (long long)c * m;
  const double2* snc = sn + (long long)c * m;
  for (int i = 0; i <= j; ++i) {
    double2 v = hA[(long long)c * hstride + i];
    if (hB) v = cadd<double>(v, hB[(long long)c * hstride + i]);
    H[i] = v;
  }
  const bool second = flag && flag[c];
  const double hn = safe_sqrt((second ? nrm2 : nrm)[(long long)c * hstride].x);
  H[j + 1] = mk<double>(hn, 0.0);
  for (int i = 0; i < j; ++i) {
    const double2 u = H[i], v = H[i + 1];
    const double2 ci = csc[i], si = snc[i];
    H[i] = cadd<double>(cmul<double>(cconj<double>(ci), u), cmul<double>(cconj<double>(si), v));
    H[i + 1] = csub<double>(cmul<double>(ci, v), cmul<double>(si, u));
  }
  const double2 a = H[j], b = H[j + 1];
  double den = sqrt(a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y);
  double2 cj, sj;
  if (den > 0) {
    cj = mk<double>(a.x / den, a.y / den);
    sj = mk<double>(b.x / den, b.y / den);
  } else {
    cj = mk<double>(1.0, 0.0);
    sj = mk<double>(0.0, 0.0);
    den = 0.0;
  }
  cs[(long long)c * m + j] = cj;
  sn[(long long)c * m + j] = sj;
  H[j] = mk<double>(den, 0.0);
  H[j + 1] = mk<double>(0.0, 0.0);
  double2* gc = g + (long long)c * (m + 1);
  const double2 gj = gc[j];
  gc[j] = cmul<double>(cconj<double>(cj), gj);
  const double2 gn = cmul<double>(sj, gj);
  gc[j + 1] = mk<double>(-gn.x, -gn.y);
  est[c] = sqrt(gn.x * gn.x + gn.y * gn.y);
  inv_hn[c] = (hn > 0) ? 1.0 / hn : 0.0;
}

void launch_arnoldi_step(Ctx& ctx, int j, int m, const int* cols, int ncols, const double2* hA, const double2* hB,
                         const double2* nrm, const double2* nrm2, const int* flag, int hstride, double2* Hh,
                         double2* cs, double2* sn, double2* g, double* est, double* inv_hn) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "arnoldi_step", 0.0, k_arnoldi_step, (ncols + 63) / 64, 64, 0, j, m, cols, ncols, hA, hB, nrm, nrm2,
            flag, hstride, Hh, cs, sn, g, est, inv_hn);
}

__global__ void k_lsq(int m, const int* __restrict__ cols, int ncols, const int* __restrict__ kcol,
                      const double2* __restrict__ Hh, const double2* __restrict__ g, double2* __restrict__ y) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  const int k = kcol[c];
  const double2* H = Hh + (long long)c * (m + 1) * m;
  const double2* gc = g + (long long)c * (m + 1);
  double2* yc = y + (long long)c * m;
  for (int i = k - 1; i >= 0; --i) {
    double2 s = gc[i];
    for (int l = i + 1; l < k; ++l) s = cfms<double>(H[(long long)l * (m + 1) + i], yc[l], s);
    const double2 d = H[(long long)i * (m + 1) + i];
    const double den = d.x * d.x + d.y * d.y;
    yc[i] = (den > 0) ? mk<double>((s.x * d.x + s.y * d.y) / den, (s.y * d.x - s.x * d.y) / den) : mk<double>(0, 0);
  }
}

void launch_lsq(Ctx& ctx, int m, const int* cols, int ncols, const int* kcol, const double2* Hh, const double2* g,
                double2* y) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "lsq", 0.0, k_lsq, (ncols + 63) / 64, 64, 0, m, cols, ncols, kcol, Hh, g, y);
}

// ---------------------------------------------------------------------------
// BiCGSTAB (right preconditioned) per-column vector updates and scalars
// ---------------------------------------------------------------------------
// Scalars per column c (complex, sc[c*8 + k]): 0 rho, 1 rho_prev, 2 alpha,
// 3 omega, 4 beta.  red[c*rstride + slot] hold the reduced dot products.
__global__ void k_bicg_scalars(int stage, const int* __restrict__ cols, int ncols, const double2* __restrict__ red,
                               int rstride, double2* __restrict__ sc) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ncols) return;
  const int c = cols[pos];
  double2* q = sc + (long long)c * 8;
  const double2* d = red + (long long)c * rstride;
  auto cdiv = [](double2 a, double2 b) {
    const double den = b.x * b.x + b.y * b.y;
    return mk<double>((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
  };
  if (stage == -1) {  // start: rho_prev = alpha = omega = 1
    q[1] = mk<double>(1, 0);
    q[2] = mk<double>(1, 0);
    q[3] = mk<double>(1, 0);
  } else if (stage == 0) {  // d[0] = <rh, r>: beta = (rho/rho_prev)(alpha/omega)
    const double2 rho = d[0];
    q[4] = cmul<double>(cdiv(rho, q[1]), cdiv(q[2], q[3]));
    q[0] = rho;
    q[1] = rho;
  } else if (stage == 1) {  // d[0] = <rh, v>: alpha = rho / <rh, v>
    q[2] = cdiv(q[0], d[0]);
  } else {  // d[0] = sum conj(s) t = conj(<t, s>), d[1] = ||t||^2: omega = <t, s> / ||t||^2
    q[3] = mk<double>(d[0].x / d[1].x, -d[0].y / d[1].x);
  }
}

void launch_bicg_scalars(Ctx& ctx, int stage, const int* cols, int ncols, const double2* red, int rstride,
                         double2* sc) {
  if (ncols <= 0) return;
  HZ_LAUNCH(ctx, "bicg_scalars", 0.0, k_bicg_scalars, (ncols + 127) / 128, 128, 0, stage, cols, ncols, red, rstride,
            sc);
}

// mode 0: p = r + beta (p - omega v);  mode 1: s = r - alpha v (into out)
__global__ void __launch_bounds__(256) k_bicg_vec(int mode, long long N, const double2* __restrict__ r,
                                                  double2* __restrict__ p, const double2* __restrict__ v,
                                                  double2* __restrict__ out, const double2* __restrict__ sc,
                                                  const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const double2* q = sc + (long long)c * 8;
  const long long off = (long long)c * N;
  const double2 beta = q[4], omega = q[3], alpha = q[2];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const double2 ri = r[off + i], vi = v[off + i];
    if (mode == 0) {
      const double2 t = cfms<double>(omega, vi, p[off + i]);  // p - omega v
      p[off + i] = cfma<double>(beta, t, ri);
    } else {
      out[off + i] = cfms<double>(alpha, vi, ri);
    }
  }
}

void launch_bicg_vec(Ctx& ctx, int mode, long long N, const double2* r, double2* p, const double2* v, double2* out,
                     const double2* sc, const int* cols, int ncols) {
  if (ncols <= 0) return;
  const int nb = krylov_nblk(N, ncols);
  const double bytes = (double)N * ncols * (mode == 0 ? 4 : 3) * sizeof(double2);
  HZ_LAUNCH(ctx, mode == 0 ? "bicg_p" : "bicg_s", bytes, k_bicg_vec, dim3(nb, ncols), 256, 0, mode, N, r, p, v, out,
            sc, cols);
}

// x += alpha ph + omega sh ;  r = s - omega t   (ph, sh in the cycle precision)
template <typename TZ>
__global__ void __launch_bounds__(256) k_bicg_xr(long long N, double2* __restrict__ x, const cplx<TZ>* __restrict__ ph,
                                                 const cplx<TZ>* __restrict__ sh, const double2* __restrict__ s,
                                                 const double2* __restrict__ t, double2* __restrict__ r,
                                                 const double2* __restrict__ sc, const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const double2* q = sc + (long long)c * 8;
  const long long off = (long long)c * N;
  const double2 alpha = q[2], omega = q[3];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const cplx<TZ> a = ph[off + i], b = sh[off + i];
    double2 xi = x[off + i];
    xi = cfma<double>(alpha, mk<double>((double)a.x, (double)a.y), xi);
    xi = cfma<double>(omega, mk<double>((double)b.x, (double)b.y), xi);
    x[off + i] = xi;
    r[off + i] = cfms<double>(omega, t[off + i], s[off + i]);
  }
}

template <typename TZ>
void launch_bicg_xr(Ctx& ctx, long long N, double2* x, const cplx<TZ>* ph, const cplx<TZ>* sh, const double2* s,
                    const double2* t, double2* r, const double2* sc, const int* cols, int ncols) {
  if (ncols <= 0) return;
  const int nb = krylov_nblk(N, ncols);
  const double bytes = (double)N * ncols * (5 * sizeof(double2) + 2 * sizeof(cplx<TZ>));
  HZ_LAUNCH(ctx, "bicg_xr", bytes, k_bicg_xr<TZ>, dim3(nb, ncols), 256, 0, N, x, ph, sh, s, t, r, sc, cols);
}
template void launch_bicg_xr<double>(Ctx&, long long, double2*, const double2*, const double2*, const double2*,
                                     const double2*, double2*, const double2*, const int*, int);
template void launch_bicg_xr<float>(Ctx&, long long, double2*, const float2*, const float2*, const double2*,
                                    const double2*, double2*, const double2*, const int*, int);

// ---------------------------------------------------------------------------
// Operator setup on the device (src/GetHelmholtz.jl:33-50, 81-83, 222-247)
// ---------------------------------------------------------------------------
// Per node: Sommerfeld term summed over the boundary faces the node lies on
// (top face skipped when NeumannOnTop; same face order as the host helper),
// mass = -w^2 m (1 - i gamma / Re w) - Somm, diag(H) = Laplacian diagonal + mass,
// diag(SH) = diag(H) + i s (Re w)^2 m, and 1/diag(SH).  BC is the Laplacian's
// boundary-row factor (orderNeumannBC); the Sommerfeld term always takes the
// factor 2, because src/GetHelmholtz.jl:45 calls getSommerfeldBC without the
// order and its default is 2 (:222).
__global__ void k_fine_setup(Grid g, int dim, double h0, double h1, double h2, double wr, double wi, double s,
                             double BC, int neumann_on_top, int sommerfeld, const double* __restrict__ m,
                             const double* __restrict__ gamma, double2* __restrict__ dH, double2* __restrict__ dSH,
                             double2* __restrict__ iSH) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.N) return;
  const int i = (int)(p % g.nx);
  const long long t = p / g.nx;
  const int j = (int)(t % g.ny);
  const int k = (int)(t / g.ny);
  const double mp = m[p], gp = gamma[p];
  // -w^2 m (1 - i gamma / Re w), w complex
  const double w2r = wr * wr - wi * wi, w2i = 2.0 * wr * wi;
  const double a = 1.0, b = -gp / wr;  // (1 + i b)
  double mr = -(w2r * a - w2i * b) * mp;
  double mi = -(w2r * b + w2i * a) * mp;
  if (sommerfeld) {
    // Somm += -i w (SB/h_d) sqrt(m) on each face, SB = 2; host order: 2D top, bottom,
    // x-high, x-low; 3D top, bottom, y-low, y-high, x-low, x-high
    const double SB = 2.0;
    const double sq = sqrt(mp);
    double si = 0.0;
    if (dim == 2) {
      if (!neumann_on_top && j == 0) si += -wr * (SB / h1) * sq;
      if (j == g.ny - 1) si += -wr * (SB / h1) * sq;
      if (i == g.nx - 1) si += -wr * (SB / h0) * sq;
      if (i == 0) si += -wr * (SB / h0) * sq;
    } else {
      if (!neumann_on_top && k == 0) si += -wr * (SB / h2) * sq;
      if (k == g.nz - 1) si += -wr * (SB / h2) * sq;
      if (j == 0) si += -wr * (SB / h1) * sq;
      if (j == g.ny - 1) si += -wr * (SB / h1) * sq;
      if (i == 0) si += -wr * (SB / h0) * sq;
      if (i == g.nx - 1) si += -wr * (SB / h0) * sq;
    }
    mi -= si;
  }
  double lap = ((i == 0 || i == g.nx - 1) ? BC : 2.0) / (h0 * h0) + ((j == 0 || j == g.ny - 1) ? BC : 2.0) / (h1 * h1);
  if (dim == 3) lap += ((k == 0 || k == g.nz - 1) ? BC : 2.0) / (h2 * h2);
  const double hr = lap + mr, hi = mi;
  dH[p] = mk<double>(hr, hi);
  const double sr = hr, shi = hi + s * wr * wr * mp;
  dSH[p] = mk<double>(sr, shi);
  const double den = sr * sr + shi * shi;
  iSH[p] = mk<double>(sr / den, -shi / den);
}

void launch_fine_setup(Ctx& ctx, const Grid& g, int dim, const double* h, double wr, double wi, double shift, double BC,
                       int neumann_on_top, int sommerfeld, const double* m, const double* gamma, double2* dH,
                       double2* dSH, double2* iSH) {
  const long long nb = (g.N + 255) / 256;
  HZ_LAUNCH(ctx, "fine_setup", (double)g.N * (2 * 8 + 3 * 16), k_fine_setup, (unsigned)nb, 256, 0, g, dim, h[0], h[1],
            dim == 3 ? h[2] : 1.0, wr, wi, shift, BC, neumann_on_top, sommerfeld, m, gamma, dH, dSH, iSH);
}

// ---------------------------------------------------------------------------
// Setup kernels
// ---------------------------------------------------------------------------
// Galerkin probing: column k of the probe block is the indicator of the
// coarse nodes whose subscripts are congruent to pattern(k) modulo 3.  Within
// a 3^d neighbourhood exactly one node of each class exists, so R A P applied
// to probe k yields, at node I, the entry A_c(I, J) for that unique J.
__global__ void k_probe_init(Grid g, int dim, double2* out, long long ld) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.N) return;
  const int i = (int)(p % g.nx);
  const long long t = p / g.nx;
  const int j = (int)(t % g.ny);
  const int k = (int)(t / g.ny);
  const int cls = (i % 3) + 3 * (j % 3) + (dim == 3 ? 9 * (k % 3) : 0);
  const int ns = dim == 3 ? 27 : 9;
  for (int s = 0; s < ns; ++s) out[(long long)s * ld + p] = mk<double>(s == cls ? 1.0 : 0.0, 0.0);
}

void launch_probe_init(Ctx& ctx, const Grid& gc, int dim, double2* out, long long ld) {
  long long nb = (gc.N + 255) / 256;
  HZ_LAUNCH(ctx, "probe_init", (double)gc.N * (dim == 3 ? 27 : 9) * sizeof(double2), k_probe_init, (unsigned)nb, 256, 0, gc, dim, out, ld);
}

__device__ __forceinline__ int off3(int cls_d, int I) {
  // offset o in {-1,0,1} with (I + o) = cls_d (mod 3)
  int o = ((cls_d - I) % 3 + 3) % 3;
  return o == 2 ? -1 : o;
}

__global__ void k_probe_scatter(Grid g, int dim, const double2* __restrict__ y, long long ld, double2* coef,
                                long long cld) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.N) return;
  const int i = (int)(p % g.nx);
  const long long t = p / g.nx;
  const int j = (int)(t % g.ny);
  const int k = (int)(t / g.ny);
  const int ns = dim == 3 ? 27 : 9;
  for (int s = 0; s < ns; ++s) {
    const int ox = off3(s % 3, i), oy = off3((s / 3) % 3, j), oz = dim == 3 ? off3(s / 9, k) : 0;
    const int slot = (ox + 1) + 3 * (oy + 1) + (dim == 3 ? 9 * (oz + 1) : 0);
    coef[(long long)slot * cld + p] = y[(long long)s * ld + p];
  }
}

void launch_probe_scatter(Ctx& ctx, const Grid& gc, int dim, const double2* y, long long ld, double2* coef,
                          long long cld) {
  long long nb = (gc.N + 255) / 256;
  HZ_LAUNCH(ctx, "probe_scatter", 2.0 * gc.N * (dim == 3 ? 27 : 9) * sizeof(double2), k_probe_scatter, (unsigned)nb, 256, 0, gc, dim, y, ld, coef, cld);
}

// coefT[o][I] = conj(coef[-o][I + o]) (zero where I + o is outside the grid).
__global__ void k_coef_transpose(Grid g, int dim, const double2* __restrict__ coef, double2* __restrict__ coefT,
                                 long long cld) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.N) return;
  const int i = (int)(p % g.nx);
  const long long t = p / g.nx;
  const int j = (int)(t % g.ny);
  const int k = (int)(t / g.ny);
  const int ns = dim == 3 ? 27 : 9;
  for (int s = 0; s < ns; ++s) {
    const int ox = s % 3 - 1, oy = (s / 3) % 3 - 1, oz = dim == 3 ? s / 9 - 1 : 0;
    const int ii = i + ox, jj = j + oy, kk = k + oz;
    double2 v = mk<double>(0, 0);
    if (ii >= 0 && ii < g.nx && jj >= 0 && jj < g.ny && kk >= 0 && kk < g.nz) {
      const long long q = ii + (long long)g.nx * (jj + (long long)g.ny * kk);
      const int ms = (1 - ox) + 3 * (1 - oy) + (dim == 3 ? 9 * (1 - oz) : 0);
      v = coef[(long long)ms * cld + q];
      v.y = -v.y;
    }
    coefT[(long long)s * cld + p] = v;
  }
}

void launch_coef_transpose(Ctx& ctx, const Grid& g, int dim, const double2* coef, double2* coefT, long long cld) {
  long long nb = (g.N + 255) / 256;
  HZ_LAUNCH(ctx, "coef_transpose", 2.0 * g.N * (dim == 3 ? 27 : 9) * sizeof(double2), k_coef_transpose, (unsigned)nb, 256, 0, g, dim, coef, coefT, cld);
}

template <typename T>
__global__ void k_center_inverse(long long N, int center, const double2* __restrict__ coef, long long cld,
                                 cplx<T>* __restrict__ dinv) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  const double2 d = coef[(long long)center * cld + p];
  const double den = d.x * d.x + d.y * d.y;
  dinv[p] = mk<T>((T)(d.x / den), (T)(-d.y / den));
}

template <typename T>
void launch_center_inverse(Ctx& ctx, const Grid& g, int dim, const double2* coef, long long cld, cplx<T>* dinv) {
  long long nb = (g.N + 255) / 256;
  HZ_LAUNCH(ctx, "center_inverse", (double)g.N * (sizeof(double2) + sizeof(cplx<T>)), k_center_inverse<T>, (unsigned)nb, 256, 0, g.N, dim == 3 ? 13 : 4, coef, cld,
            dinv);
}

template <typename To, typename From>
__global__ void k_cast(const cplx<From>* __restrict__ in, cplx<To>* __restrict__ out, long long n) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
    out[p] = mk<To>((To)in[p].x, (To)in[p].y);
}

template <typename To, typename From>
void launch_cast(Ctx& ctx, const cplx<From>* in, cplx<To>* out, long long n) {
  if (n <= 0) return;
  long long nb = std::min<long long>((n + 255) / 256, 16LL * kSMs);
  HZ_LAUNCH(ctx, "cast", (double)n * (sizeof(cplx<To>) + sizeof(cplx<From>)), (k_cast<To, From>), (unsigned)nb, 256, 0, in, out, n);
}

template <typename To, typename From>
__global__ void k_cast_cols(long long N, const cplx<From>* __restrict__ in, long long ldi, cplx<To>* __restrict__ out,
                            long long ldo, const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const cplx<From>* ic = in + (long long)c * ldi;
  cplx<To>* oc = out + (long long)c * ldo;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
    oc[p] = mk<To>((To)ic[p].x, (To)ic[p].y);
}

template <typename To, typename From>
void launch_cast_cols(Ctx& ctx, long long N, const cplx<From>* in, long long ldi, cplx<To>* out, long long ldo,
                      const int* cols, int ncols) {
  if (ncols <= 0) return;
  int nb = krylov_nblk(N, ncols);
  dim3 grid(nb, ncols);
  HZ_LAUNCH(ctx, "cast_cols", (double)N * ncols * (sizeof(cplx<To>) + sizeof(cplx<From>)), (k_cast_cols<To, From>), grid, 256, 0, N, in, ldi, out, ldo, cols);
}

template <typename T>
__global__ void k_zero_cols(long long N, cplx<T>* __restrict__ x, long long ld, const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  cplx<T>* xc = x + (long long)c * ld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
    xc[p] = mk<T>(0, 0);
}

template <typename T>
void launch_zero_cols(Ctx& ctx, long long N, cplx<T>* x, long long ld, const int* cols, int ncols) {
  if (ncols <= 0) return;
  int nb = krylov_nblk(N, ncols);
  dim3 grid(nb, ncols);
  HZ_LAUNCH(ctx, "zero_cols", (double)N * ncols * sizeof(cplx<T>), k_zero_cols<T>, grid, 256, 0, N, x, ld, cols);
}

// explicit instantiations
template void launch_update_x<double>(Ctx&, long long, const double2*, long long, long long, const int*,
                                      const double2*, int, double2*, long long, const int*, int, long long);
template void launch_update_x<float>(Ctx&, long long, const float2*, long long, long long, const int*, const double2*,
                                     int, double2*, long long, const int*, int, long long);
template void launch_center_inverse<double>(Ctx&, const Grid&, int, const double2*, long long, double2*);
template void launch_center_inverse<float>(Ctx&, const Grid&, int, const double2*, long long, float2*);
template void launch_cast<float, double>(Ctx&, const double2*, float2*, long long);
template void launch_cast<double, float>(Ctx&, const float2*, double2*, long long);
template void launch_cast_cols<float, double>(Ctx&, long long, const double2*, long long, float2*, long long,
                                              const int*, int);
template void launch_cast_cols<double, float>(Ctx&, long long, const float2*, long long, double2*, long long,
                                              const int*, int);
template void launch_cast_cols<double, double>(Ctx&, long long, const double2*, long long, double2*, long long,
                                               const int*, int);
template void launch_cast_cols<float, df64_tag>(Ctx&, long long, const float4*, long long, float2*, long long,
                                                const int*, int);
template void launch_zero_cols<double>(Ctx&, long long, double2*, long long, const int*, int);
template void launch_zero_cols<float>(Ctx&, long long, float2*, long long, const int*, int);

}  // namespace hz
