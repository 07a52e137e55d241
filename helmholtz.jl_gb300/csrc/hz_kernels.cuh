// Launch wrappers for the helmgpu kernels (implemented in hz_stencil.cu and
// hz_krylov.cu).  Every wrapper launches on ctx.stream, counts the launch and,
// when profiling is on, brackets it with CUDA events.
#pragma once

#include <string>
#include <vector>

#include "../../include/helmgpu.h"
#include "hz_common.cuh"
#include "hz_host.h"

namespace hz {

// Device ordinals the per-device caches of the library cover.
static constexpr int kMaxDevices = 64;

// Per-handle launch context: stream, launch counter and the optional
// per-kernel event timer.
struct Ctx {
  cudaStream_t stream = nullptr;
  long long launches = 0;
  bool profile = false;
  std::vector<std::string> names;  // kernel name table
  std::vector<long long> counts;   // launches per kernel
  std::vector<long long> timed;    // launches with an event pair (profiling on)
  std::vector<double> total_ms;    // event-timed milliseconds per kernel
  std::vector<double> alg_bytes;   // algorithmic bytes per kernel (all launches)
  std::vector<double> alg_flops;   // algorithmic flops per kernel (tensor-core and native-FP64 outer kernels; 0 elsewhere)
  struct Pending {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  int name_id(const char* name);
  void before(int id, cudaEvent_t* a);
  void after(int id, cudaEvent_t a, double bytes);
  void resolve();  // after a stream sync: fold pending event pairs into the table
  void add_bytes(const char* name, double bytes) { alg_bytes[name_id(name)] += bytes; }
  void add_flops(const char* name, double flops) { alg_flops[name_id(name)] += flops; }
  // launch-shape choices of the autotuner: CTAs aimed at per launch of the
  // fine-level and the Galerkin stencils (0: the default rule), which set how
  // many right-hand sides a block loops over
  int tune_fine = 0, tune_rap = 0;
  // 3D Galerkin stencils of the complex-FP32 cycle on staged tiles (k_rap_tile)
  // instead of k_rap: opt-in (HELMGPU_RAP_TILED=1) until timed on a GB300
  bool rap_tiled = false;
  void release();
};

// Jacobi / residual modes of the stencil kernels.
enum StencilMode { MODE_APPLY = 0, MODE_RESID = 1, MODE_JACOBI = 2 };

// Fine-level operator: constant-coefficient nodal Laplacian with the
// reference's ghost-reflection boundary rows plus a per-node complex diagonal.
struct FineOp {
  Grid g;
  double o[3];  // 1/h_d^2: interior off-diagonal magnitude per axis
  double b[3];  // BC/h_d^2: boundary-row off-diagonal magnitude per axis
  int adj;      // 1: apply the adjoint (transposed boundary rows, conjugated diagonal)
  int outer = 0;  // 1: the Krylov method's operator H (launch-table names outer_*), 0: a cycle operator
};

// y = op(x) on nodes of a fine level, for the columns cols[0..ncols) of the
// RHS block (column c starts at c*ld), computed in precision T.  b may be
// FP64 while x/y are FP32, and x may be FP32 while y is FP64.
template <typename T, typename TX, typename TB>
void launch_fine(Ctx& ctx, int mode, const FineOp& op, const cplx<T>* diag, const cplx<T>* dinv, const cplx<TX>* x,
                 const cplx<TB>* b, cplx<T>* y, long long ld, const int* cols, int ncols, double w);

// Galerkin level: 3^d stored complex coefficients per node, coef[k*cld + p]
// is the entry A(p, p + offset_k), offset_k = (k%3-1, k/3%3-1, k/9-1).
template <typename T, typename TB>
void launch_rap(Ctx& ctx, int mode, const Grid& g, const cplx<T>* coef, long long cld, const cplx<T>* dinv,
                const cplx<T>* x, const cplx<TB>* b, cplx<T>* y, long long ld, const int* cols, int ncols, double w);

// y = w * dinv .* b  (first Jacobi sweep from a zero guess); adj conjugates dinv.
template <typename T, typename TB>
void launch_jacobi0(Ctx& ctx, const Grid& g, const cplx<T>* dinv, int adj, const cplx<TB>* b, cplx<T>* y, long long ld,
                    const int* cols, int ncols, double w);

// Full-weighting restriction rc = P^T rf / 2^d (fine grid gf, coarse grid gc).
template <typename T>
void launch_restrict(Ctx& ctx, const Grid& gf, const Grid& gc, const cplx<T>* rf, long long ldf, cplx<T>* rc,
                     long long ldc, const int* cols, int ncols);

// xout = xin + P ec (bi/trilinear nodal prolongation); xin may be null (xout = P ec).
template <typename T>
void launch_prolong(Ctx& ctx, const Grid& gf, const Grid& gc, const cplx<T>* ec, long long ldc, const cplx<T>* xin,
                    cplx<T>* xout, long long ldf, const int* cols, int ncols);

// Coarsest-level direct solve: blocked banded LU (see band_block_operators);
// T / G are the device copies of the forward / backward block operators.
// work holds 3 * ncols * N FP64 complex values.
struct BandSolveOps {
  long long N = 0;
  std::vector<BandBlock> blocks;
  const BandBlock* dblocks = nullptr;  // device copy of blocks: one cooperative launch per solve
  const double2* T = nullptr;
  const double2* G = nullptr;
};
template <typename T>
void launch_band_solve(Ctx& ctx, const BandSolveOps& op, const cplx<T>* b, cplx<T>* x, long long ld, const int* cols,
                       int ncols, double2* work);

// Allocation-free Y = A X on device memory for hz_apply_noalloc: the column
// list lives in a static device array of kNoAllocMaxCols entries shared by all
// calls on a device.  Returns 0, -1 (bad size) or -2 (CUDA error) with *err set.
static constexpr int kNoAllocMaxCols = HZ_NOALLOC_MAX_COLS;
static constexpr int kNoAllocMaxDevices = 64;
int launch_fine_apply_noalloc(cudaStream_t stream, int dev, const FineOp& op, const double2* diag, const double2* x,
                              double2* y, long long ld, int nrhs, std::string* err);

// ---- emulated-FP64 outer FGMRES (hz_df64.cu) ---------------------------------
// w = H z with z complex FP32, accumulated in df64; w a df64 vector (TO =
// float4) or rounded to FP64 (TO = double2); dHd = diag(H) in df64.
template <typename TO>
void launch_fine_df64(Ctx& ctx, const FineOp& op, const float4* dHd, const float2* z, TO* y, long long ld,
                      const int* cols, int ncols);
void launch_dots_df(Ctx& ctx, long long N, const float4* V, long long vstride, long long ld, int i0, int K,
                    const float4* w, long long wld, const int* cols, int ncols, int nblk, int want_norm,
                    double2* part, const int* mask = nullptr);
void launch_update_df(Ctx& ctx, long long N, const float4* V, long long vstride, long long ld, int i0, int K,
                      const double2* h, int hstride, float4* w, long long wld, const int* cols, int ncols, int nblk,
                      int want_norm, double2* part, const int* mask = nullptr);
// y = s[c] x (FP64 x into df64 y; may run in place on the same memory)
void launch_to_df(Ctx& ctx, long long N, const double2* x, long long xld, float4* y, long long yld, const double* s,
                  const int* cols, int ncols);
void launch_diag_to_df(Ctx& ctx, long long N, const double2* d, float4* out);
// x += sum_{i<kcol[c]} y_i Z_i with the products and their sum in df64, x FP64.
void launch_update_x_df(Ctx& ctx, long long N, const float2* Z, long long zstride, long long ld, const int* kcol,
                        const double2* y, int ystride, double2* x, long long xld, const int* cols, int ncols,
                        long long zcols);
// Coarsest solve as a dense emulated-FP64 product x = Ainv b (Ainv column-major
// df64); part holds dense_df_splits(N, ncols) * ncols * N FP64 values.
int dense_df_splits(long long N, int ncols);
void launch_dense_df(Ctx& ctx, long long N, const float4* Ainv, const float2* b, float2* x, long long ld,
                     const int* cols, int ncols, double2* part);
void launch_identity(Ctx& ctx, long long N, double2* e);
void launch_inplace_df(Ctx& ctx, long long n, double2* a);
// Coarsest solve with the block operators stored as df64 (op.T / op.G point to
// float4 arrays); work holds 3 * ncols * N df64 values.
template <typename T>
void launch_band_solve_df(Ctx& ctx, const BandSolveOps& op, const cplx<T>* b, cplx<T>* x, long long ld,
                          const int* cols, int ncols, float4* work);

// ---- K-cycle (hz_kcycle.cu) ------------------------------------------------------
// Two-step FGMRES on a coarse level, per-column scalars ks[c*8 + slot] on the
// device (0 beta^2, 1 h00, 2 h10^2, 3 h01, 4 h11, 5 h21^2, 6 y0, 7 y1); part
// holds 3 * ncols * kcycle_nblk(N) partial sums.
int kcycle_nblk(long long N);
// slots base.. : conj(V_s) . W for s < nd, then ||W||^2 when want_norm
template <typename T>
void launch_kc_sums(Ctx& ctx, long long N, long long ld, const int* cols, int nc, int nd, int want_norm,
                    const cplx<T>* V0, const cplx<T>* V1, const cplx<T>* W, double2* part, double2* ks, int base);
// W -= sum_{s<nd} ks[hb+s] V_s, ||W||^2 into slot norm_slot
template <typename T>
void launch_kc_update(Ctx& ctx, long long N, long long ld, const int* cols, int nc, int nd, int hb, double2* ks,
                      const cplx<T>* V0, const cplx<T>* V1, cplx<T>* W, double2* part, int norm_slot);
// Y = X / sqrt(ks[slot])
template <typename T>
void launch_kc_scale(Ctx& ctx, long long N, long long ld, const int* cols, int nc, const double2* ks, int slot,
                     const cplx<T>* X, cplx<T>* Y);
// X = y0 Z0 + y1 Z1
template <typename T>
void launch_kc_combine(Ctx& ctx, long long N, long long ld, const int* cols, int nc, const double2* ks,
                       const cplx<T>* Z0, const cplx<T>* Z1, cplx<T>* X);
// the 3x2 least-squares problem of each column -> y0, y1
void launch_kc_lsq(Ctx& ctx, const int* cols, int nc, double2* ks);
// one-step least squares (y0 from slots 0-2, y1 = 0) and X += y0 Z0 + y1 Z1 (GMRES smoothing)
void launch_kc_lsq1(Ctx& ctx, const int* cols, int nc, double2* ks);
template <typename T>
void launch_kc_combine_add(Ctx& ctx, long long N, long long ld, const int* cols, int nc, const double2* ks,
                           const cplx<T>* Z0, const cplx<T>* Z1, cplx<T>* X);

// ---- setup kernels ---------------------------------------------------------
// Fine-level diagonals on the device from nodal m and gamma (device arrays):
// diag(H), diag(SH) with the shift i*shift*Re(w)^2*m, and 1/diag(SH).
void launch_fine_setup(Ctx& ctx, const Grid& g, int dim, const double* h, double wr, double wi, double shift, double BC,
                       int neumann_on_top, int sommerfeld, const double* m, const double* gamma, double2* dH,
                       double2* dSH, double2* iSH);
void launch_probe_init(Ctx& ctx, const Grid& gc, int dim, double2* out, long long ld);
void launch_probe_scatter(Ctx& ctx, const Grid& gc, int dim, const double2* y, long long ld, double2* coef,
                          long long cld);
void launch_coef_transpose(Ctx& ctx, const Grid& g, int dim, const double2* coef, double2* coefT, long long cld);
template <typename T>
void launch_center_inverse(Ctx& ctx, const Grid& g, int dim, const double2* coef, long long cld, cplx<T>* dinv);
template <typename To, typename From>
void launch_cast(Ctx& ctx, const cplx<From>* in, cplx<To>* out, long long n);
// Column-wise cast between RHS blocks (active columns only).
template <typename To, typename From>
void launch_cast_cols(Ctx& ctx, long long N, const cplx<From>* in, long long ldi, cplx<To>* out, long long ldo,
                      const int* cols, int ncols);
template <typename T>
void launch_zero_cols(Ctx& ctx, long long N, cplx<T>* x, long long ld, const int* cols, int ncols);

// ---- Krylov kernels (FP64) -------------------------------------------------
// Conventions: per-column device arrays are indexed by the column number c
// (not by the position in the active list); V_i column c lives at
// V + (i*vstride + c)*ld.  Partial sums go to part[(pos*K1 + slot)*nblk + blk]
// and are folded in a fixed order by launch_reduce (deterministic results).
int krylov_nblk(long long N, int ncols);
// slots i < K: conj(V_{i0+i}) . w ; slot K (want_norm): ||w||^2.  Columns with
// mask[c] == 0 (mask may be null) yield zeros; a masked launch adds no
// algorithmic bytes (the caller adds those of the columns that took it).
void launch_dots(Ctx& ctx, long long N, const double2* V, long long vstride, long long ld, int i0, int K,
                 const double2* w, long long wld, const int* cols, int ncols, int nblk, int want_norm, double2* part,
                 const int* mask = nullptr);
// w -= sum_{i<K} h[c*hstride + i0 + i] V_{i0+i}; with want_norm, slot 0 of the
// partials holds ||w_new||^2.  Columns with mask[c] == 0 are left untouched.
void launch_update(Ctx& ctx, long long N, const double2* V, long long vstride, long long ld, int i0, int K,
                   const double2* h, int hstride, double2* w, long long wld, const int* cols, int ncols, int nblk,
                   int want_norm, double2* part, const int* mask = nullptr);
// flag[c] = (after[c*astride] < before[c*bstride + bslot] / 2): DGKS test for a
// second Gram-Schmidt pass.
void launch_dgks(Ctx& ctx, const int* cols, int ncols, const double2* before, int bstride, int bslot,
                 const double2* after, int astride, int* flag);
// out[c*ostride + slot] = sum over blocks of part (slot < K1); accum adds to out.
void launch_reduce(Ctx& ctx, const double2* part, const int* cols, int ncols, int K1, int nblk, double2* out,
                   int ostride, int accum);
// Deferred normalisation of the FGMRES basis: stored v_i stands for sig_i v_i
// (sig[c*sstride + i]).  init: sig_0 = 1; coef_i = sig_i^2 d_i for i < K (the
// update's coefficients); true: hA_i, hB_i *= sig_i sig_j (i <= j) and the norm
// slots nr, nr2 *= sig_j^2; next: sig_{j+1} = sig_j * invhn; y_i *= sig_i.
void launch_sig_init(Ctx& ctx, const int* cols, int ncols, double* sig, int sstride);
void launch_sig_coef(Ctx& ctx, const int* cols, int ncols, int K, const double* sig, int sstride, const double2* d,
                     int hstride, double2* coef);
void launch_sig_true(Ctx& ctx, int j, const int* cols, int ncols, const double* sig, int sstride, double2* hA,
                     double2* hB, double2* nr, double2* nr2, int hstride);
void launch_sig_next(Ctx& ctx, int j, const int* cols, int ncols, double* sig, int sstride, const double* invhn);
void launch_sig_y(Ctx& ctx, const int* cols, int ncols, const int* kcol, const double* sig, int sstride, double2* y,
                  int ystride);
// y[:, c] = s[c] * x[:, c]
void launch_scale_cols(Ctx& ctx, long long N, const double2* x, long long xld, double2* y, long long yld,
                       const double* s, const int* cols, int ncols);
// x[:, c] += sum_{i < kcol[c]} y[c*ystride + i] Z_i[:, c], Z in precision TZ;
// zcols = sum of kcol over the active columns (for the byte count).
template <typename TZ>
void launch_update_x(Ctx& ctx, long long N, const cplx<TZ>* Z, long long zstride, long long ld, const int* kcol,
                     const double2* y, int ystride, double2* x, long long xld, const int* cols, int ncols,
                     long long zcols);
// nrm[c] = sqrt(Re red[c*stride + slot]), inv[c] = 1/nrm[c] (0 for a zero norm).
void launch_norms(Ctx& ctx, const double2* red, int stride, int slot, const int* cols, int ncols, double* nrm,
                  double* inv);
// g[c*(m+1) + 0] = beta[c], the other entries of g zero.
void launch_cycle_init(Ctx& ctx, int m, const int* cols, int ncols, const double* beta, double2* g);
// Arnoldi step j of column c: h = hA + hB (hB may be null), h_{j+1,j} =
// sqrt(Re nrm[c*hstride]) or, where flag[c] is set (second pass taken),
// sqrt(Re nrm2[c*hstride]); apply rotations 0..j-1, form rotation j, update
// g, est[c] = |g_{j+1}|, inv_hn[c] = 1/h_{j+1,j}.
// Hh[c*(m+1)*m + jj*(m+1) + i], cs/sn[c*m + i], g[c*(m+1) + i].
void launch_arnoldi_step(Ctx& ctx, int j, int m, const int* cols, int ncols, const double2* hA, const double2* hB,
                         const double2* nrm, const double2* nrm2, const int* flag, int hstride, double2* Hh,
                         double2* cs, double2* sn, double2* g, double* est, double* inv_hn);
// BiCGSTAB per-column scalars sc[c*8 + k] (0 rho, 1 rho_prev, 2 alpha, 3 omega,
// 4 beta) from reduced dots red[c*rstride + slot]: stage -1 init, 0 beta from
// <rh,r>, 1 alpha from <rh,v>, 2 omega from (conj<t,s>, ||t||^2).
void launch_bicg_scalars(Ctx& ctx, int stage, const int* cols, int ncols, const double2* red, int rstride,
                         double2* sc);
// mode 0: p = r + beta (p - omega v); mode 1: out = r - alpha v.  Blocks of N per column.
void launch_bicg_vec(Ctx& ctx, int mode, long long N, const double2* r, double2* p, const double2* v, double2* out,
                     const double2* sc, const int* cols, int ncols);
// x += alpha ph + omega sh; r = s - omega t.
template <typename TZ>
void launch_bicg_xr(Ctx& ctx, long long N, double2* x, const cplx<TZ>* ph, const cplx<TZ>* sh, const double2* s,
                    const double2* t, double2* r, const double2* sc, const int* cols, int ncols);
// Back substitution R y = g for the first kcol[c] entries: y[c*m + i].
void launch_lsq(Ctx& ctx, int m, const int* cols, int ncols, const int* kcol, const double2* Hh, const double2* g,
                double2* y);

}  // namespace hz
