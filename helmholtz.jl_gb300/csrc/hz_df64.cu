// Emulated-FP64 ("df64") outer FGMRES kernels: a complex value is stored as
// float4 (re_hi, im_hi, re_lo, im_lo) with x = hi + lo exactly representable to
// about 2^-48 relative, and arithmetic uses error-free FP32 transformations
// (TwoSum: Knuth; TwoProd via fused multiply-add), which run on the FP32 pipe
// (64x the FP64 rate of GB300).  Used for the Krylov basis, H z, Gram-Schmidt
// and the basis scaling of the mixed-precision form; the true residual at
// every restart is still computed in native FP64.
//
// The (re_hi, im_hi) pair is the float2 a complex-FP32 kernel reads, so the
// V-cycle takes a df64 basis vector directly as its right-hand side.
#include <algorithm>

#include <cooperative_groups.h>

#include "hz_launch.cuh"

namespace cg = cooperative_groups;

namespace hz {

// ---- error-free transformations (no contraction, no reassociation) ---------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void quick_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Accumulator: hi + lo, lo collects rounding errors and cross terms and is
// folded back by renorm().
struct DAcc {
  float hi, lo;
  __device__ __forceinline__ void init(float h, float l) {
    hi = h;
    lo = l;
  }
  // += (ah + al) * (bh + bl)
  __device__ __forceinline__ void mac(float ah, float al, float bh, float bl) {
    float p, e, s, t;
    two_prod(ah, bh, p, e);
    two_sum(hi, p, s, t);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(t, e));
    lo = __fmaf_rn(ah, bl, lo);
    lo = __fmaf_rn(al, bh, lo);
  }
  // -= (ah + al) * (bh + bl)
  __device__ __forceinline__ void msub(float ah, float al, float bh, float bl) { mac(-ah, -al, bh, bl); }
  // += (ah + al) * b   (b exact float)
  __device__ __forceinline__ void mac1(float ah, float al, float b) {
    float p, e, s, t;
    two_prod(ah, b, p, e);
    two_sum(hi, p, s, t);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(t, e));
    lo = __fmaf_rn(al, b, lo);
  }
  // += x (an FP32 value) with the rounding error of the sum kept in lo
  __device__ __forceinline__ void add(float x) {
    float s, t;
    two_sum(hi, x, s, t);
    hi = s;
    lo = __fadd_rn(lo, t);
  }
  __device__ __forceinline__ void renorm() { quick_two_sum(hi, lo, hi, lo); }
  __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ void split(double x, float& hi, float& lo) {
  hi = __double2float_rn(x);
  lo = __double2float_rn(x - (double)hi);
}

// ---- H z (z complex FP32) into a df64 basis vector ---------------------------
// dHd: diag(H) as float4 (re_hi, im_hi, re_lo, im_lo); c[6] = (hi, lo) of the
// interior / boundary-row magnitudes per axis.
struct DFOp {
  int nx, ny, nz;
  long long N;
  float oh[3], ol[3], bh[3], bl[3];
  int adj;
};

__device__ __forceinline__ void axis_df(int i, int n, const DFOp& op, int a, float& clh, float& cll, float& crh,
                                        float& crl) {
  // same rule as the FP32/FP64 stencil: boundary rows use BC/h^2, the adjoint takes entry (j, i)
  bool lb, rb;  // left / right coefficient is the boundary one
  if (!op.adj) {
    lb = (i == n - 1);
    rb = (i == 0);
  } else {
    lb = (i - 1 == 0);
    rb = (i + 1 == n - 1);
  }
  if (i > 0) {
    clh = lb ? op.bh[a] : op.oh[a];
    cll = lb ? op.bl[a] : op.ol[a];
  } else {
    clh = cll = 0.f;
  }
  if (i < n - 1) {
    crh = rb ? op.bh[a] : op.oh[a];
    crl = rb ? op.bl[a] : op.ol[a];
  } else {
    crh = crl = 0.f;
  }
}

__device__ __forceinline__ void store_out(float4* y, long long i, const DAcc& re, const DAcc& im) {
  y[i] = make_float4(re.hi, im.hi, re.lo, im.lo);
}
__device__ __forceinline__ void store_out(double2* y, long long i, const DAcc& re, const DAcc& im) {
  y[i] = mk<double>(re.to_double(), im.to_double());
}

// TO = float4: df64 result (basis vector); TO = double2: rounded to FP64
template <bool IS3D, typename TO>
__global__ void __launch_bounds__(256) k_fine_df64(DFOp op, const float4* __restrict__ dHd,
                                                   const float2* __restrict__ z, TO* __restrict__ y, long long ld,
                                                   const int* __restrict__ cols, int ncols, int cpb) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= op.N) return;
  const int nx = op.nx, ny = op.ny;
  const int i = (int)(p % nx);
  const long long t = p / nx;
  const int j = (int)(t % ny);
  const int k = (int)(t / ny);
  float c[12];  // (hi, lo) of left/right per axis
  axis_df(i, nx, op, 0, c[0], c[1], c[2], c[3]);
  axis_df(j, ny, op, 1, c[4], c[5], c[6], c[7]);
  if (IS3D) axis_df(k, op.nz, op, 2, c[8], c[9], c[10], c[11]);
  const long long sy = nx, sz = (long long)nx * ny;
  const long long o[6] = {(i > 0) ? -1LL : 0LL, (i < nx - 1) ? 1LL : 0LL, (j > 0) ? -sy : 0LL,
                          (j < ny - 1) ? sy : 0LL, (IS3D && k > 0) ? -sz : 0LL, (IS3D && k < op.nz - 1) ? sz : 0LL};
  float4 d = dHd[p];
  if (op.adj) {
    d.y = -d.y;
    d.w = -d.w;
  }
  const int c0 = blockIdx.y * cpb;
  const int c1 = min(ncols, c0 + cpb);
  for (int ci = c0; ci < c1; ++ci) {
    const long long off = (long long)cols[ci] * ld;
    const float2* zc = z + off + p;
    const float2 zp = zc[0];
    DAcc re, im;
    re.init(0.f, 0.f);
    im.init(0.f, 0.f);
    // diagonal: (dr + i di)(zr + i zi)
    re.mac1(d.x, d.z, zp.x);
    re.mac1(-d.y, -d.w, zp.y);
    im.mac1(d.x, d.z, zp.y);
    im.mac1(d.y, d.w, zp.x);
#pragma unroll
    for (int q = 0; q < (IS3D ? 6 : 4); ++q) {
      const float2 zn = zc[o[q]];
      re.mac1(-c[2 * q], -c[2 * q + 1], zn.x);
      im.mac1(-c[2 * q], -c[2 * q + 1], zn.y);
    }
    re.renorm();
    im.renorm();
    store_out(y, off + p, re, im);
  }
}

template <typename TO>
void launch_fine_df64(Ctx& ctx, const FineOp& op, const float4* dHd, const float2* z, TO* y, long long ld,
                      const int* cols, int ncols) {
  if (ncols <= 0) return;
  DFOp d;
  d.nx = op.g.nx;
  d.ny = op.g.ny;
  d.nz = op.g.nz;
  d.N = op.g.N;
  for (int a = 0; a < 3; ++a) {
    d.oh[a] = (float)op.o[a];
    d.ol[a] = (float)(op.o[a] - (double)d.oh[a]);
    d.bh[a] = (float)op.b[a];
    d.bl[a] = (float)(op.b[a] - (double)d.bh[a]);
  }
  d.adj = op.adj;
  const int TPB = 256;
  const long long nbx = (op.g.N + TPB - 1) / TPB;
  const int ch = chunks_for(nbx, ncols);
  const int cpb = (ncols + ch - 1) / ch;
  const double bytes = (double)op.g.N * ncols * (8 + 16) + (double)op.g.N * 16;
  if (op.g.nz > 1)
    HZ_LAUNCH(ctx, "outer_apply_df64", bytes, (k_fine_df64<true, TO>), dim3((unsigned)nbx, (unsigned)ch), TPB, 0, d, dHd,
              z, y, ld, cols, ncols, cpb);
  else
    HZ_LAUNCH(ctx, "outer_apply_df64", bytes, (k_fine_df64<false, TO>), dim3((unsigned)nbx, (unsigned)ch), TPB, 0, d, dHd,
              z, y, ld, cols, ncols, cpb);
}
template void launch_fine_df64<float4>(Ctx&, const FineOp&, const float4*, const float2*, float4*, long long,
                                       const int*, int);
template void launch_fine_df64<double2>(Ctx&, const FineOp&, const float4*, const float2*, double2*, long long,
                                        const int*, int);

// ---- Gram-Schmidt: dots and update on df64 vectors ---------------------------
static constexpr int RT = 256;
static constexpr int KG = 16;

template <int NV>
__device__ __forceinline__ void block_reduce_df(const double2 (&v)[NV], int nv, double nrm, int want_norm,
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

__device__ __forceinline__ void zero_partials(int K1, double2* part, int nblk) {
  if (threadIdx.x < K1) part[(long long)threadIdx.x * nblk + blockIdx.x] = mk<double>(0, 0);
}

// slots s < KT: sum conj(V_{i0+s}) w, slot KT (want_norm): ||w||^2
template <int KT>
__global__ void __launch_bounds__(RT, 2) k_dots_df(long long N, const float4* __restrict__ V, long long vstride,
                                                   long long ld, int i0, const float4* __restrict__ w, long long wld,
                                                   const int* __restrict__ cols, const int* __restrict__ mask,
                                                   int nblk, int want_norm, double2* __restrict__ part) {
  constexpr int KA = KT > 0 ? KT : 1;
  const int pos = blockIdx.y;
  const int c = cols[pos];
  const int K1 = KT + want_norm;
  double2* pp = part + (long long)pos * K1 * nblk;
  if (mask && !mask[c]) {
    zero_partials(K1, pp, nblk);
    return;
  }
  const float4* wc = w + (long long)c * wld;
  const float4* vb = V + ((long long)i0 * vstride + c) * ld;
  const long long vs = vstride * ld;
  DAcc ar[KA], ai[KA], nn;
#pragma unroll
  for (int s = 0; s < KA; ++s) {
    ar[s].init(0.f, 0.f);
    ai[s].init(0.f, 0.f);
  }
  nn.init(0.f, 0.f);
  const long long stride = (long long)nblk * RT;
  for (long long p = (long long)blockIdx.x * RT + threadIdx.x; p < N; p += stride) {
    const float4 wv = wc[p];
#pragma unroll
    for (int s = 0; s < KT; ++s) {
      const float4 v = vb[s * vs + p];
      // conj(v) w = (vr wr + vi wi) + i (vr wi - vi wr)
      ar[s].mac(v.x, v.z, wv.x, wv.z);
      ar[s].mac(v.y, v.w, wv.y, wv.w);
      ai[s].mac(v.x, v.z, wv.y, wv.w);
      ai[s].msub(v.y, v.w, wv.x, wv.z);
    }
    if (want_norm) {
      nn.mac(wv.x, wv.z, wv.x, wv.z);
      nn.mac(wv.y, wv.w, wv.y, wv.w);
    }
  }
  double2 acc[KA];
#pragma unroll
  for (int s = 0; s < KA; ++s) acc[s] = mk<double>(ar[s].to_double(), ai[s].to_double());
  block_reduce_df<KA>(acc, KT, nn.to_double(), want_norm, pp, nblk);
}

// w -= sum_s h[c*hstride + i0 + s] V_{i0+s}; slot 0 (want_norm): ||w_new||^2
template <int KT>
__global__ void __launch_bounds__(RT, 2) k_update_df(long long N, const float4* __restrict__ V, long long vstride,
                                                     long long ld, int i0, const double2* __restrict__ h,
                                                     int hstride, float4* __restrict__ w, long long wld,
                                                     const int* __restrict__ cols, const int* __restrict__ mask,
                                                     int nblk, int want_norm, double2* __restrict__ part) {
  const int pos = blockIdx.y;
  const int c = cols[pos];
  double2* pp = part + (long long)pos * want_norm * nblk;
  if (mask && !mask[c]) {
    zero_partials(want_norm, pp, nblk);
    return;
  }
  float hrh[KT], hrl[KT], hih[KT], hil[KT];
#pragma unroll
  for (int s = 0; s < KT; ++s) {
    const double2 hv = h[(long long)c * hstride + i0 + s];
    split(hv.x, hrh[s], hrl[s]);
    split(hv.y, hih[s], hil[s]);
  }
  const float4* vb = V + ((long long)i0 * vstride + c) * ld;
  const long long vs = vstride * ld;
  float4* wc = w + (long long)c * wld;
  DAcc nn;
  nn.init(0.f, 0.f);
  const long long stride = (long long)nblk * RT;
  for (long long p = (long long)blockIdx.x * RT + threadIdx.x; p < N; p += stride) {
    const float4 wv = wc[p];
    DAcc re, im;
    re.init(wv.x, wv.z);
    im.init(wv.y, wv.w);
#pragma unroll
    for (int s = 0; s < KT; ++s) {
      const float4 v = vb[s * vs + p];
      // (hr + i hi)(vr + i vi) = (hr vr - hi vi) + i (hr vi + hi vr)
      re.msub(hrh[s], hrl[s], v.x, v.z);
      re.mac(hih[s], hil[s], v.y, v.w);
      im.msub(hrh[s], hrl[s], v.y, v.w);
      im.msub(hih[s], hil[s], v.x, v.z);
    }
    re.renorm();
    im.renorm();
    __stcs(&wc[p], make_float4(re.hi, im.hi, re.lo, im.lo));
    if (want_norm) {
      nn.mac(re.hi, re.lo, re.hi, re.lo);
      nn.mac(im.hi, im.lo, im.hi, im.lo);
    }
  }
  if (want_norm) {
    const double2 none[1] = {mk<double>(0, 0)};
    block_reduce_df<1>(none, 0, nn.to_double(), 1, pp, nblk);
  }
}

#define HZ_K_CASES(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16)

void launch_dots_df(Ctx& ctx, long long N, const float4* V, long long vstride, long long ld, int i0, int K,
                    const float4* w, long long wld, const int* cols, int ncols, int nblk, int want_norm,
                    double2* part, const int* mask) {
  if (ncols <= 0) return;
  dim3 grid(nblk, ncols);
  const double bytes = mask ? 0.0 : (double)N * ncols * (K + 1) * 16.0;
  switch (K) {
#define HZ_DDF_CASE(k)                                                                                      \
  case k:                                                                                                   \
    HZ_LAUNCH(ctx, "krylov_dots", bytes, k_dots_df<k>, grid, RT, 0, N, V, vstride, ld, i0, w, wld, cols, mask, \
              nblk, want_norm, part);                                                                       \
    break;
    HZ_DDF_CASE(0)
    HZ_K_CASES(HZ_DDF_CASE)
#undef HZ_DDF_CASE
    default:
      throw std::runtime_error("launch_dots_df: 0..16 vectors per pass");
  }
}

void launch_update_df(Ctx& ctx, long long N, const float4* V, long long vstride, long long ld, int i0, int K,
                      const double2* h, int hstride, float4* w, long long wld, const int* cols, int ncols, int nblk,
                      int want_norm, double2* part, const int* mask) {
  if (ncols <= 0) return;
  dim3 grid(nblk, ncols);
  const double bytes = mask ? 0.0 : (double)N * ncols * (K + 2) * 16.0;
  switch (K) {
#define HZ_UDF_CASE(k)                                                                                            \
  case k:                                                                                                         \
    HZ_LAUNCH(ctx, "krylov_update", bytes, k_update_df<k>, grid, RT, 0, N, V, vstride, ld, i0, h, hstride, w, wld, \
              cols, mask, nblk, want_norm, part);                                                                 \
    break;
    HZ_K_CASES(HZ_UDF_CASE)
#undef HZ_UDF_CASE
    default:
      throw std::runtime_error("launch_update_df: 1..16 vectors per pass");
  }
}

// ---- coarsest solve with emulated-FP64 window operators ---------------------
// Same schedule as k_band_coop (one cooperative launch, grid-wide barrier
// between block steps); operators T/G and the work vectors are df64.
__device__ __forceinline__ void cmac_df(DAcc& re, DAcc& im, const float4 m, const float4 v) {
  // (mr + i mi)(vr + i vi)
  re.mac(m.x, m.z, v.x, v.z);
  re.msub(m.y, m.w, v.y, v.w);
  im.mac(m.x, m.z, v.y, v.w);
  im.mac(m.y, m.w, v.x, v.z);
}

__device__ __forceinline__ float4 warp_sum_df(const DAcc& re, const DAcc& im) {
  double a = re.to_double(), b = im.to_double();
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  float rh, rl, ih, il;
  split(a, rh, rl);
  split(b, ih, il);
  return make_float4(rh, ih, rl, il);
}

static constexpr int BCW = 1;  // columns per warp item

template <typename T>
__global__ void __launch_bounds__(256) k_band_coop_df(long long N, int nbk, const BandBlock* __restrict__ blocks,
                                                      const float4* __restrict__ Tops, const float4* __restrict__ Gops,
                                                      const cplx<T>* __restrict__ b, long long ldb,
                                                      const int* __restrict__ cols, int ncols,
                                                      float4* __restrict__ work, cplx<T>* __restrict__ x,
                                                      long long ldx) {
  cg::grid_group grid = cg::this_grid();
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  float4* const Y0 = work;
  float4* const Y1 = work + (long long)ncols * N;
  float4* const X4 = work + 2LL * ncols * N;
  const int ngrp = (ncols + BCW - 1) / BCW;
  long long prev_end = 0;
  for (int I = 0; I < nbk; ++I) {
    const BandBlock B = blocks[I];
    const int split_k = (I == 0) ? 0 : (int)(prev_end - B.s);
    const float4* src0 = (I & 1) ? Y0 : Y1;
    float4* dst = (I & 1) ? Y1 : Y0;
    const long long items = (long long)B.W * ngrp;
    for (long long it = gw; it < items; it += nw) {
      const int i = (int)(it % B.W), c0 = (int)(it / B.W) * BCW;
      const float4* Mr = Tops + B.toff + (long long)i * B.W;
      DAcc re[BCW], im[BCW];
#pragma unroll
      for (int c = 0; c < BCW; ++c) {
        re[c].init(0.f, 0.f);
        im[c].init(0.f, 0.f);
      }
      for (int k = lane; k < B.W; k += 32) {
        const float4 m = Mr[k];
#pragma unroll
        for (int c = 0; c < BCW; ++c) {
          const int ci = c0 + c;
          if (ci < ncols) {
            float4 v;
            if (k < split_k) {
              v = src0[(long long)ci * N + B.s + k];
            } else {
              const cplx<T> bb = b[(long long)cols[ci] * ldb + B.s + k];
              v = make_float4((float)bb.x, (float)bb.y, 0.f, 0.f);  // FP32 input: exact as a df64 pair
            }
            cmac_df(re[c], im[c], m, v);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < BCW; ++c) {
        const float4 r = warp_sum_df(re[c], im[c]);
        if (lane == 0 && c0 + c < ncols) dst[(long long)(c0 + c) * N + B.s + i] = r;
      }
    }
    prev_end = B.s + B.W;
    grid.sync();
  }
  for (int I = nbk - 1; I >= 0; --I) {
    const BandBlock B = blocks[I];
    const float4* yb = (I & 1) ? Y1 : Y0;
    const long long items = (long long)B.nb * ngrp;
    for (long long it = gw; it < items; it += nw) {
      const int i = (int)(it % B.nb), c0 = (int)(it / B.nb) * BCW;
      const float4* Mr = Gops + B.goff + (long long)i * B.Wb;
      DAcc re[BCW], im[BCW];
#pragma unroll
      for (int c = 0; c < BCW; ++c) {
        re[c].init(0.f, 0.f);
        im[c].init(0.f, 0.f);
      }
      for (int k = lane; k < B.Wb; k += 32) {
        const float4 m = Mr[k];
#pragma unroll
        for (int c = 0; c < BCW; ++c) {
          const int ci = c0 + c;
          if (ci < ncols) {
            const long long q = (long long)ci * N + B.s + k;
            cmac_df(re[c], im[c], m, (k < B.nb) ? yb[q] : X4[q]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < BCW; ++c) {
        const float4 r = warp_sum_df(re[c], im[c]);
        const int ci = c0 + c;
        if (lane == 0 && ci < ncols) {
          X4[(long long)ci * N + B.s + i] = r;
          x[(long long)cols[ci] * ldx + B.s + i] =
              mk<T>((T)((double)r.x + (double)r.z), (T)((double)r.y + (double)r.w));
        }
      }
    }
    grid.sync();
  }
}

template <typename T>
void launch_band_solve_df(Ctx& ctx, const BandSolveOps& op, const cplx<T>* b, cplx<T>* x, long long ld,
                          const int* cols, int ncols, float4* work) {
  if (ncols <= 0) return;
  const long long N = op.N;
  const int nbk = (int)op.blocks.size();
  double bytes = 0.0;
  for (const BandBlock& B : op.blocks)
    bytes += ((double)B.W * B.W + (double)B.nb * B.Wb) * 16.0 + ncols * (2.0 * B.W + B.Wb + 2.0 * B.nb) * 16.0;
  static int capacity[kMaxDevices] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < kMaxDevices && capacity[dev] == 0) {
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_band_coop_df<T>, 256, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    capacity[dev] = std::max(1, std::min(per_sm, 4)) * std::max(1, sms);
  }
  const int grid = (dev >= 0 && dev < kMaxDevices) ? capacity[dev] : kSMs;
  static thread_local int id = -1;
  if (id < 0 || (size_t)id >= ctx.names.size() || ctx.names[id] != "band_solve") id = ctx.name_id("band_solve");
  cudaEvent_t ev = nullptr;
  ctx.before(id, &ev);
  const BandBlock* blk = op.dblocks;
  const float4* Tp = reinterpret_cast<const float4*>(op.T);
  const float4* Gp = reinterpret_cast<const float4*>(op.G);
  long long ldb = ld, ldx = ld;
  void* args[] = {(void*)&N,    (void*)&nbk,  (void*)&blk,   (void*)&Tp,   (void*)&Gp, (void*)&b,
                  (void*)&ldb,  (void*)&cols, (void*)&ncols, (void*)&work, (void*)&x,  (void*)&ldx};
  const cudaError_t e =
      cudaLaunchCooperativeKernel((const void*)k_band_coop_df<T>, dim3(grid), dim3(256), args, 0, ctx.stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("band_solve (emulated FP64) cooperative launch failed: ") +
                             cudaGetErrorString(e));
  }
  ctx.after(id, ev, bytes);
}
template void launch_band_solve_df<float>(Ctx&, const BandSolveOps&, const float2*, float2*, long long, const int*,
                                          int, float4*);

// ---- coarsest solve as a dense emulated-FP64 product X = A^{-1} B -------------
// Ainv is column-major N x N in df64 (A^{-1}(i, k) at k*N + i), computed once in
// FP64.  Thread = one row i and DCB columns; the k range is split KS ways
// (partials in FP64, folded by k_dense_fold), so every SM has work even for a
// few columns.  B and X are the cycle's complex FP32 columns.  Both FP32 parts
// of each A^{-1} entry multiply b; products are summed in FP32 over blocks of
// kDenseBlk rows and every block sum joins a double-float accumulator, so the
// rounding error is that of a 32-term FP32 sum per block, far below the FP32
// rounding of the result the cycle receives.
static constexpr int DCB = 8;
static constexpr int kDenseBlk = 32;  // rows per FP32 partial sum

__global__ void __launch_bounds__(256) k_dense_df(long long N, int ncols, int kchunk, const float4* __restrict__ Ainv,
                                                  const float2* __restrict__ b, long long ldb,
                                                  const int* __restrict__ cols, double2* __restrict__ part) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * DCB;
  const int ks = blockIdx.z;
  if (i >= N) return;
  const long long k0 = (long long)ks * kchunk, k1 = min(N, k0 + kchunk);
  DAcc re[DCB], im[DCB];
  const float2* bc[DCB];
#pragma unroll
  for (int c = 0; c < DCB; ++c) {
    re[c].init(0.f, 0.f);
    im[c].init(0.f, 0.f);
    bc[c] = b + (long long)cols[min(c0 + c, ncols - 1)] * ldb;
  }
  // blocks of kDenseBlk rows summed in FP32 (hi and lo parts of A^-1 both
  // applied), each block sum folded into the double-float accumulators
  for (long long kb = k0; kb < k1; kb += kDenseBlk) {
    const long long ke = min(k1, kb + kDenseBlk);
    float sr[DCB], si[DCB];
#pragma unroll
    for (int c = 0; c < DCB; ++c) sr[c] = si[c] = 0.f;
    for (long long k = kb; k < ke; ++k) {
      const float4 a = Ainv[k * N + i];
#pragma unroll
      for (int c = 0; c < DCB; ++c) {
        const float2 v = bc[c][k];  // same address across the warp: broadcast
        sr[c] = __fmaf_rn(a.x, v.x, sr[c]);
        sr[c] = __fmaf_rn(-a.y, v.y, sr[c]);
        si[c] = __fmaf_rn(a.x, v.y, si[c]);
        si[c] = __fmaf_rn(a.y, v.x, si[c]);
        sr[c] = __fmaf_rn(a.z, v.x, sr[c]);
        sr[c] = __fmaf_rn(-a.w, v.y, sr[c]);
        si[c] = __fmaf_rn(a.z, v.y, si[c]);
        si[c] = __fmaf_rn(a.w, v.x, si[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < DCB; ++c) {
      re[c].add(sr[c]);
      im[c].add(si[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < DCB; ++c)
    if (c0 + c < ncols) part[((long long)ks * ncols + c0 + c) * N + i] = mk<double>(re[c].to_double(), im[c].to_double());
}

__global__ void __launch_bounds__(256) k_dense_fold(long long N, int ncols, int KS, const double2* __restrict__ part,
                                                    float2* __restrict__ x, long long ldx, const int* __restrict__ cols) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int ci = blockIdx.y;
  if (i >= N) return;
  double ar = 0.0, ai = 0.0;
  for (int ks = 0; ks < KS; ++ks) {
    const double2 v = part[((long long)ks * ncols + ci) * N + i];
    ar += v.x;
    ai += v.y;
  }
  x[(long long)cols[ci] * ldx + i] = make_float2((float)ar, (float)ai);
}

int dense_df_splits(long long N, int ncols) {
  const long long threads = N * ((ncols + DCB - 1) / DCB);
  long long ks = (8LL * kSMs * 256 + threads - 1) / std::max(threads, 1LL);
  return (int)std::max(1LL, std::min(ks, std::max(1LL, N / 64)));
}

void launch_dense_df(Ctx& ctx, long long N, const float4* Ainv, const float2* b, float2* x, long long ld,
                     const int* cols, int ncols, double2* part) {
  if (ncols <= 0) return;
  const int KS = dense_df_splits(N, ncols);
  const int kchunk = (int)((N + KS - 1) / KS);
  const dim3 grid((unsigned)((N + 255) / 256), (unsigned)((ncols + DCB - 1) / DCB), (unsigned)KS);
  const double bytes = (double)N * N * 16.0 * ((ncols + DCB - 1) / DCB) + (double)ncols * N * 16.0;
  HZ_LAUNCH(ctx, "band_solve", bytes, k_dense_df, grid, 256, 0, N, ncols, kchunk, Ainv, b, ld, cols, part);
  HZ_LAUNCH(ctx, "dense_fold", (double)KS * ncols * N * 16.0, k_dense_fold,
            dim3((unsigned)((N + 255) / 256), (unsigned)ncols), 256, 0, N, ncols, KS, part, x, ld, cols);
}

// identity block (N columns) for computing the inverse with the FP64 band solve
__global__ void k_identity(long long N, double2* __restrict__ e) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < N * N; q += (long long)gridDim.x * blockDim.x)
    e[q] = mk<double>((q / N) == (q % N) ? 1.0 : 0.0, 0.0);
}
void launch_identity(Ctx& ctx, long long N, double2* e) {
  const long long nb = std::min<long long>((N * N + 255) / 256, 16LL * kSMs);
  HZ_LAUNCH(ctx, "identity", (double)N * N * 16.0, k_identity, (unsigned)nb, 256, 0, N, e);
}

// FP64 -> df64 in place (same 16 bytes per complex value)
__global__ void k_inplace_df(long long n, double2* __restrict__ a) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double2 v = a[q];
    float rh, rl, ih, il;
    split(v.x, rh, rl);
    split(v.y, ih, il);
    reinterpret_cast<float4*>(a)[q] = make_float4(rh, ih, rl, il);
  }
}
void launch_inplace_df(Ctx& ctx, long long n, double2* a) {
  const long long nb = std::min<long long>((n + 255) / 256, 16LL * kSMs);
  HZ_LAUNCH(ctx, "cast", (double)n * 32.0, k_inplace_df, (unsigned)nb, 256, 0, n, a);
}

// ---- solution update x += sum_i y_i Z_i (Z complex FP32, x FP64) -----------------
__global__ void __launch_bounds__(256, 4) k_update_x_df(long long N, const float2* __restrict__ Z, long long zstride,
                                                     long long ld, const int* __restrict__ kcol,
                                                     const double2* __restrict__ y, int ystride,
                                                     double2* __restrict__ x, long long xld,
                                                     const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const int k = kcol[c];
  // the coefficients of this column, split into FP32 pairs once per block and
  // read from shared memory (broadcast): registers stay free for occupancy
  __shared__ float sy[4][64];  // Re hi, Re lo, Im hi, Im lo; restart length <= 64
  for (int s = threadIdx.x; s < k; s += blockDim.x) {
    const double2 v = y[(long long)c * ystride + s];
    split(v.x, sy[0][s], sy[1][s]);
    split(v.y, sy[2][s], sy[3][s]);
  }
  __syncthreads();
  double2* xc = x + (long long)c * xld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
    DAcc re, im;
    re.init(0.f, 0.f);
    im.init(0.f, 0.f);
#pragma unroll
    for (int s = 0; s < KG; ++s) {
      if (s < k) {
        const float2 z = Z[((long long)s * zstride + c) * ld + p];
        // (yr + i yi)(zr + i zi)
        re.mac1(sy[0][s], sy[1][s], z.x);
        re.mac1(-sy[2][s], -sy[3][s], z.y);
        im.mac1(sy[0][s], sy[1][s], z.y);
        im.mac1(sy[2][s], sy[3][s], z.x);
      }
    }
    for (int s = KG; s < k; ++s) {  // restart lengths above KG
      const float2 z = Z[((long long)s * zstride + c) * ld + p];
      re.mac1(sy[0][s], sy[1][s], z.x);
      re.mac1(-sy[2][s], -sy[3][s], z.y);
      im.mac1(sy[0][s], sy[1][s], z.y);
      im.mac1(sy[2][s], sy[3][s], z.x);
    }
    const double2 xv = xc[p];
    xc[p] = mk<double>(xv.x + re.to_double(), xv.y + im.to_double());
  }
}

void launch_update_x_df(Ctx& ctx, long long N, const float2* Z, long long zstride, long long ld, const int* kcol,
                        const double2* y, int ystride, double2* x, long long xld, const int* cols, int ncols,
                        long long zcols) {
  if (ncols <= 0) return;
  const int nb = std::max(1, std::min((int)((N + 255) / 256), 8 * kSMs / std::max(ncols, 1) + 1));
  const double bytes = (double)N * (ncols * 2.0 * 16.0 + zcols * 8.0);
  HZ_LAUNCH(ctx, "update_x", bytes, k_update_x_df, dim3(nb, ncols), 256, 0, N, Z, zstride, ld, kcol, y, ystride, x,
            xld, cols);
}

// ---- conversions and scaling -------------------------------------------------
// y[:, c] = s[c] * x[:, c]: FP64 x into a df64 y (the start vector of a cycle)
__global__ void __launch_bounds__(256) k_to_df(long long N, const double2* __restrict__ x, long long xld,
                                               float4* __restrict__ y, long long yld, const double* __restrict__ s,
                                               const int* __restrict__ cols) {
  const int c = cols[blockIdx.y];
  const double sc = s[c];
  const double2* xc = x + (long long)c * xld;
  float4* yc = y + (long long)c * yld;
  // elements are independent (in place: each is read before it is written)
#pragma unroll 4
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
    const double2 v = __ldcs(&xc[p]);
    float rh, rl, ih, il;
    split(sc * v.x, rh, rl);
    split(sc * v.y, ih, il);
    __stcs(&yc[p], make_float4(rh, ih, rl, il));
  }
}

void launch_to_df(Ctx& ctx, long long N, const double2* x, long long xld, float4* y, long long yld, const double* s,
                  const int* cols, int ncols) {
  if (ncols <= 0) return;
  const int nb = std::max(1, std::min((int)((N + 255) / 256), 8 * kSMs / std::max(ncols, 1) + 1));
  HZ_LAUNCH(ctx, "scale_cols", (double)N * ncols * 32.0, k_to_df, dim3(nb, ncols), 256, 0, N, x, xld, y, yld, s,
            cols);
}

// df64 diag(H) from the FP64 array (once per handle)
__global__ void k_diag_to_df(long long N, const double2* __restrict__ d, float4* __restrict__ out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
    float rh, rl, ih, il;
    split(d[p].x, rh, rl);
    split(d[p].y, ih, il);
    out[p] = make_float4(rh, ih, rl, il);
  }
}

void launch_diag_to_df(Ctx& ctx, long long N, const double2* d, float4* out) {
  const long long nb = std::min<long long>((N + 255) / 256, 16LL * kSMs);
  HZ_LAUNCH(ctx, "cast", (double)N * 32.0, k_diag_to_df, (unsigned)nb, 256, 0, N, d, out);
}

}  // namespace hz
