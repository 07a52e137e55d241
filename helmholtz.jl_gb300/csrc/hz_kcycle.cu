// K-cycle coarse-grid correction: two steps of FGMRES on a coarse level's
// operator, right-preconditioned by that level's own cycle, for a block of
// columns at once (the Krylov-accelerated cycle Multigrid.jl offers as
// cycleType 'K', used by test/ShiftedLaplacianTest.jl:137-140).  The same
// kernels run the "Jac-GMRES" smoother (relaxType of that test, :138): one or
// two GMRES steps preconditioned by a damped-Jacobi sweep, added to the iterate.
//
// Per column c the scalars live on the device in ks[c*8 + slot]:
//   0 beta^2 (real), 1 h00, 2 h10^2 (real), 3 h01, 4 h11, 5 h21^2 (real), 6 y0, 7 y1.
// Vectors are level vectors in the cycle's precision T and so is the
// per-element arithmetic (a thread sums a few terms); block and column totals
// are accumulated in FP64 and folded in a fixed order (deterministic).
#include "hz_launch.cuh"

namespace hz {

namespace {

template <typename T> __device__ __forceinline__ double2 ld2(const cplx<T>& v) {
  return make_double2((double)v.x, (double)v.y);
}

// block reduction of up to 3 complex slots; thread 0 writes part[(pos*K1 + s)*nblk + blk]
__device__ __forceinline__ void block_sum3(double2 (&a)[3], int K1, double2* part, int pos, int nblk, int blk) {
  __shared__ double2 sh[3][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a[s].x += __shfl_xor_sync(0xffffffffu, a[s].x, o);
      a[s].y += __shfl_xor_sync(0xffffffffu, a[s].y, o);
    }
    if (lane == 0) sh[s][warp] = a[s];
  }
  __syncthreads();
  if (threadIdx.x < K1) {
    double2 t = make_double2(0.0, 0.0);
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) {
      t.x += sh[threadIdx.x][w].x;
      t.y += sh[threadIdx.x][w].y;
    }
    part[((long long)pos * K1 + threadIdx.x) * nblk + blk] = t;
  }
}

}  // namespace

// slots s < nd: conj(V_s) . W ; slot nd (want_norm): ||W||^2
template <typename T>
__global__ void __launch_bounds__(256) k_kc_sums(long long N, long long ld, const int* __restrict__ cols, int nd,
                                                 int want_norm, const cplx<T>* __restrict__ V0,
                                                 const cplx<T>* __restrict__ V1, const cplx<T>* __restrict__ W,
                                                 int nblk, double2* __restrict__ part) {
  const int pos = blockIdx.y, c = cols[pos], blk = blockIdx.x;
  const long long off = (long long)c * ld;
  // a thread's few terms are summed in the vectors' precision, blocks in FP64
  cplx<T> t0 = mk<T>(0, 0), t1 = mk<T>(0, 0);
  T tn = 0;
  for (long long p = (long long)blk * blockDim.x + threadIdx.x; p < N; p += (long long)nblk * blockDim.x) {
    const cplx<T> w = W[off + p];
    if (nd > 0) t0 = cfma_conj<T>(V0[off + p], w, t0);
    if (nd > 1) t1 = cfma_conj<T>(V1[off + p], w, t1);
    if (want_norm) tn = fma(w.x, w.x, fma(w.y, w.y, tn));
  }
  const double2 nrm = make_double2((double)tn, 0.0);
  double2 a[3];
  a[0] = nd > 0 ? ld2<T>(t0) : nrm;
  a[1] = nd > 1 ? ld2<T>(t1) : nrm;
  a[2] = nrm;
  block_sum3(a, nd + want_norm, part, pos, nblk, blk);
}

// W -= sum_{s<nd} h_s V_s (h_s = ks[c*8 + hb + s]), then ||W||^2 partials (slot 0)
template <typename T>
__global__ void __launch_bounds__(256) k_kc_update(long long N, long long ld, const int* __restrict__ cols, int nd,
                                                   int hb, const double2* __restrict__ ks,
                                                   const cplx<T>* __restrict__ V0, const cplx<T>* __restrict__ V1,
                                                   cplx<T>* __restrict__ W, int nblk, double2* __restrict__ part) {
  const int pos = blockIdx.y, c = cols[pos], blk = blockIdx.x;
  const long long off = (long long)c * ld;
  const double2 h0d = ks[c * 8 + hb];
  const double2 h1d = nd > 1 ? ks[c * 8 + hb + 1] : make_double2(0.0, 0.0);
  const cplx<T> h0 = mk<T>((T)h0d.x, (T)h0d.y), h1 = mk<T>((T)h1d.x, (T)h1d.y);
  T n2 = 0;
  for (long long p = (long long)blk * blockDim.x + threadIdx.x; p < N; p += (long long)nblk * blockDim.x) {
    cplx<T> w = cfms<T>(h0, V0[off + p], W[off + p]);
    if (nd > 1) w = cfms<T>(h1, V1[off + p], w);
    W[off + p] = w;
    n2 = fma(w.x, w.x, fma(w.y, w.y, n2));
  }
  double2 a[3] = {make_double2((double)n2, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  block_sum3(a, 1, part, pos, nblk, blk);
}

// Y = X / sqrt(ks[c*8 + slot].x)  (zero when the norm is zero)
template <typename T>
__global__ void __launch_bounds__(256) k_kc_scale(long long N, long long ld, const int* __restrict__ cols,
                                                  const double2* __restrict__ ks, int slot,
                                                  const cplx<T>* __restrict__ X, cplx<T>* __restrict__ Y) {
  const int c = cols[blockIdx.y];
  const double n2 = ks[c * 8 + slot].x;
  const T s = (T)(n2 > 0.0 ? 1.0 / sqrt(n2) : 0.0);
  const long long off = (long long)c * ld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
    Y[off + p] = cscale<T>(s, X[off + p]);
}

// X += y0 Z0 + y1 Z1 (the GMRES smoothing update of the current iterate)
template <typename T>
__global__ void __launch_bounds__(256) k_kc_combine_add(long long N, long long ld, const int* __restrict__ cols,
                                                        const double2* __restrict__ ks,
                                                        const cplx<T>* __restrict__ Z0,
                                                        const cplx<T>* __restrict__ Z1, cplx<T>* __restrict__ X) {
  const int c = cols[blockIdx.y];
  const double2 y0d = ks[c * 8 + 6], y1d = ks[c * 8 + 7];
  const cplx<T> y0 = mk<T>((T)y0d.x, (T)y0d.y), y1 = mk<T>((T)y1d.x, (T)y1d.y);
  const long long off = (long long)c * ld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
    X[off + p] = cfma<T>(y1, Z1[off + p], cfma<T>(y0, Z0[off + p], X[off + p]));
}

// X = y0 Z0 + y1 Z1
template <typename T>
__global__ void __launch_bounds__(256) k_kc_combine(long long N, long long ld, const int* __restrict__ cols,
                                                    const double2* __restrict__ ks, const cplx<T>* __restrict__ Z0,
                                                    const cplx<T>* __restrict__ Z1, cplx<T>* __restrict__ X) {
  const int c = cols[blockIdx.y];
  const double2 y0d = ks[c * 8 + 6], y1d = ks[c * 8 + 7];
  const cplx<T> y0 = mk<T>((T)y0d.x, (T)y0d.y), y1 = mk<T>((T)y1d.x, (T)y1d.y);
  const long long off = (long long)c * ld;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
    X[off + p] = cfma<T>(y1, Z1[off + p], cmul<T>(y0, Z0[off + p]));
}

// min || beta e0 - H y || with H = [[h00, h01], [h10, h11], [0, h21]] by two
// complex Givens rotations (h10, h21 real, stored squared), per column.
__global__ void k_kc_lsq(const int* __restrict__ cols, int nc, double2* __restrict__ ks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double2* s = ks + cols[i] * 8;
  const double beta = sqrt(fmax(s[0].x, 0.0));
  const double2 a = s[1], b = s[3], d = s[4];
  const double c10 = sqrt(fmax(s[2].x, 0.0)), e = sqrt(fmax(s[5].x, 0.0));
  double2 y0 = make_double2(0.0, 0.0), y1 = make_double2(0.0, 0.0);
  const double r1 = sqrt(a.x * a.x + a.y * a.y + c10 * c10);
  if (beta > 0.0 && r1 > 0.0) {
    const double2 cs = make_double2(a.x / r1, a.y / r1);  // G1 = [conj(cs) sn; -sn cs], sn = c10 / r1 (real)
    const double sn = c10 / r1;
    // row 0 after G1: (r1, b'), g0 = conj(cs) beta; row 1: (0, d'), g1 = -sn beta
    const double2 bp = make_double2(cs.x * b.x + cs.y * b.y + sn * d.x, cs.x * b.y - cs.y * b.x + sn * d.y);
    const double2 dp = make_double2(-sn * b.x + cs.x * d.x - cs.y * d.y, -sn * b.y + cs.x * d.y + cs.y * d.x);
    const double2 g0 = make_double2(cs.x * beta, -cs.y * beta);
    const double g1 = -sn * beta;
    const double r2 = sqrt(dp.x * dp.x + dp.y * dp.y + e * e);
    if (r2 > 0.0) {
      // G2 on rows 1, 2: g1' = conj(dp / r2) g1, y1 = g1' / r2
      y1 = make_double2(dp.x * g1 / (r2 * r2), -dp.y * g1 / (r2 * r2));
    }
    // y0 = (g0 - b' y1) / r1
    const double2 t = make_double2(g0.x - (bp.x * y1.x - bp.y * y1.y), g0.y - (bp.x * y1.y + bp.y * y1.x));
    y0 = make_double2(t.x / r1, t.y / r1);
  }
  s[6] = y0;
  s[7] = y1;
}

// One GMRES step: min || beta e0 - [h00; h10] y0 || = conj(h00) beta / (|h00|^2 + h10^2); y1 = 0.
__global__ void k_kc_lsq1(const int* __restrict__ cols, int nc, double2* __restrict__ ks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double2* s = ks + cols[i] * 8;
  const double beta = sqrt(fmax(s[0].x, 0.0));
  const double2 a = s[1];
  const double den = a.x * a.x + a.y * a.y + fmax(s[2].x, 0.0);
  double2 y0 = make_double2(0.0, 0.0);
  if (beta > 0.0 && den > 0.0) y0 = make_double2(a.x * beta / den, -a.y * beta / den);
  s[6] = y0;
  s[7] = make_double2(0.0, 0.0);
}

static int kc_nblk(long long N) {
  long long b = (N + 2047) / 2048;
  return (int)std::max<long long>(1, std::min<long long>(64, b));
}

template <typename T>
void launch_kc_sums(Ctx& ctx, long long N, long long ld, const int* cols, int nc, int nd, int want_norm,
                    const cplx<T>* V0, const cplx<T>* V1, const cplx<T>* W, double2* part, double2* ks, int base) {
  const int nblk = kc_nblk(N);
  const int K1 = nd + want_norm;
  HZ_LAUNCH(ctx, "kcycle_dots", (double)N * nc * (nd + 1) * sizeof(cplx<T>), k_kc_sums<T>, dim3(nblk, nc), 256, 0, N,
            ld, cols, nd, want_norm, V0, V1, W, nblk, part);
  launch_reduce(ctx, part, cols, nc, K1, nblk, ks + base, 8, 0);
}

template <typename T>
void launch_kc_update(Ctx& ctx, long long N, long long ld, const int* cols, int nc, int nd, int hb, double2* ks,
                      const cplx<T>* V0, const cplx<T>* V1, cplx<T>* W, double2* part, int norm_slot) {
  const int nblk = kc_nblk(N);
  HZ_LAUNCH(ctx, "kcycle_update", (double)N * nc * (nd + 2) * sizeof(cplx<T>), k_kc_update<T>, dim3(nblk, nc), 256, 0,
            N, ld, cols, nd, hb, ks, V0, V1, W, nblk, part);
  launch_reduce(ctx, part, cols, nc, 1, nblk, ks + norm_slot, 8, 0);
}

template <typename T>
void launch_kc_scale(Ctx& ctx, long long N, long long ld, const int* cols, int nc, const double2* ks, int slot,
                     const cplx<T>* X, cplx<T>* Y) {
  const int nblk = kc_nblk(N);
  HZ_LAUNCH(ctx, "kcycle_scale", (double)N * nc * 2 * sizeof(cplx<T>), k_kc_scale<T>, dim3(nblk, nc), 256, 0, N, ld,
            cols, ks, slot, X, Y);
}

template <typename T>
void launch_kc_combine(Ctx& ctx, long long N, long long ld, const int* cols, int nc, const double2* ks,
                       const cplx<T>* Z0, const cplx<T>* Z1, cplx<T>* X) {
  const int nblk = kc_nblk(N);
  HZ_LAUNCH(ctx, "kcycle_combine", (double)N * nc * 3 * sizeof(cplx<T>), k_kc_combine<T>, dim3(nblk, nc), 256, 0, N,
            ld, cols, ks, Z0, Z1, X);
}

void launch_kc_lsq(Ctx& ctx, const int* cols, int nc, double2* ks) {
  HZ_LAUNCH(ctx, "kcycle_lsq", (double)nc * 8 * 16, k_kc_lsq, (nc + 127) / 128, 128, 0, cols, nc, ks);
}

void launch_kc_lsq1(Ctx& ctx, const int* cols, int nc, double2* ks) {
  HZ_LAUNCH(ctx, "smooth_lsq", (double)nc * 8 * 16, k_kc_lsq1, (nc + 127) / 128, 128, 0, cols, nc, ks);
}

template <typename T>
void launch_kc_combine_add(Ctx& ctx, long long N, long long ld, const int* cols, int nc, const double2* ks,
                           const cplx<T>* Z0, const cplx<T>* Z1, cplx<T>* X) {
  const int nblk = kc_nblk(N);
  HZ_LAUNCH(ctx, "smooth_update", (double)N * nc * 4 * sizeof(cplx<T>), k_kc_combine_add<T>, dim3(nblk, nc), 256, 0,
            N, ld, cols, ks, Z0, Z1, X);
}

int kcycle_nblk(long long N) { return kc_nblk(N); }

#define HZ_KC_INST(T)                                                                                                \
  template void launch_kc_sums<T>(Ctx&, long long, long long, const int*, int, int, int, const cplx<T>*,            \
                                  const cplx<T>*, const cplx<T>*, double2*, double2*, int);                          \
  template void launch_kc_update<T>(Ctx&, long long, long long, const int*, int, int, int, double2*, const cplx<T>*, \
                                    const cplx<T>*, cplx<T>*, double2*, int);                                        \
  template void launch_kc_scale<T>(Ctx&, long long, long long, const int*, int, const double2*, int, const cplx<T>*, \
                                   cplx<T>*);                                                                        \
  template void launch_kc_combine<T>(Ctx&, long long, long long, const int*, int, const double2*, const cplx<T>*,    \
                                     const cplx<T>*, cplx<T>*);                                                      \
  template void launch_kc_combine_add<T>(Ctx&, long long, long long, const int*, int, const double2*,                \
                                         const cplx<T>*, const cplx<T>*, cplx<T>*);
HZ_KC_INST(float)
HZ_KC_INST(double)
#undef HZ_KC_INST

}  // namespace hz
