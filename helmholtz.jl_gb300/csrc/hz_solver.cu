// helmgpu solver runtime and C ABI.
//
// One handle = one Helmholtz problem on one GPU: the matrix-free fine-level
// operator, a lazily built Galerkin multigrid hierarchy per orientation
// (H and its adjoint), the coarsest banded LU factors, the FGMRES workspace
// sized for the largest right-hand-side block seen so far, and the CUDA
// stream every kernel runs on.
//
// Reference path replaced: src/ShiftedLaplacianMultigridSolver.jl:33-102
// (solveLinearSystem: lazy MGsetup, shift operator, FGMRES on H
// preconditioned by one cycle on SH), src/GetHelmholtz.jl:33-50,81-95
// (operator assembly, shift, getHelmholtzFun).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../../include/helmgpu.h"
#include "hz_host.h"
#include "hz_kernels.cuh"
#include "hz_learn.h"

namespace {

using namespace hz;

struct HzError {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw HzError{code, buf};
}

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? HZ_ERR_ALLOC : HZ_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
}

// Device (re)allocations so far in this process: a captured CUDA graph holds
// raw pointers, so graphs captured before the latest allocation are dropped.
std::atomic<long long> g_alloc_gen{0};

// Owning device buffer.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t b) {
    if (b <= bytes && p) return;
    reset();
    if (b == 0) return;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      fail(HZ_ERR_ALLOC, "cudaMalloc of %.3f GB failed: %s", b / 1e9, cudaGetErrorString(e));
    }
    bytes = b;
    g_alloc_gen.fetch_add(1);
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

thread_local std::string g_thread_error;

struct Level {
  Grid g;
  long long ld = 0;  // leading dimension of the RHS blocks of this level
  // Galerkin coefficients (levels >= 1): FP64 master and FP32 copy
  DBuf coef64, coef32, dinv64, dinv32;
  // 5/7-point (fine-kind) level: level 0, or a re-discretised coarse level
  bool fine = false;
  FineOp fop{};
  const double2* fd64 = nullptr;  // diag(SH), 1/diag(SH) in FP64 and FP32
  const double2* fi64 = nullptr;
  const float2* fd32 = nullptr;
  const float2* fi32 = nullptr;
  DBuf own_d64, own_i64, own_d32, own_i32;  // storage of a re-discretised level
  std::vector<double> m, gamma;              // restricted nodal m and shifted gamma (host)
  // work buffers (precision of the cycle): x/t ping-pong, r residual, b right-hand side
  DBuf x, t, r, b;
  // K-cycle on this level: V0, V1, Z0, Z1, W blocks, per-column scalars, partial sums
  DBuf kv, ks, kp;
  // GMRES smoothing ("Jac-GMRES") on this level: the same layout, own storage (the
  // smoother runs inside the K-cycle's cycles on the same level)
  DBuf gv, gs, gp;
};

struct Hierarchy {
  bool built = false;
  int adj = 0;
  std::vector<std::unique_ptr<Level>> lv;
  // coarsest LU (band, FP64) as blocked operators
  long long nc = 0;
  int kl = 0, ku = 0;
  DBuf bandT, bandG, bandB, bandwork;
  BandSolveOps band;
  bool band_df = false;   // block operators stored as df64
  bool dense_df = false;  // coarsest solve as a dense df64 product with A^{-1}
  DBuf dense;             // A^{-1} (column-major, df64)
};

}  // namespace

struct hz_handle {
  hz_problem prob{};
  std::vector<double> m, gamma;
  hz_options opt{};
  int dev = 0;
  Ctx ctx;
  Grid g0{};
  FineOp fop{};
  // fine-level diagonals: H, SH (FP64), 1/diag(SH) (FP64), FP32 copies of SH
  DBuf diagH, diagSH, dinvSH, diagSH32, dinvSH32;
  DBuf diagHdf;  // diag(H) in df64 (emulated-FP64 outer arithmetic)
  Hierarchy hier[2];
  // FGMRES workspace
  int rcap = 0;
  int mcap = 0;
  DBuf Bd, Xd, V, Z, part, hA, hB, nr, nr2, flag, Hh, cs, sn, gv, yv, est, invhn, bnorm, bnorm_inv, beta, beta_inv,
      cols, kcol;
  DBuf bsc;         // BiCGSTAB per-column scalars
  DBuf sig, hC;     // FGMRES basis scales (stored v_i stands for sig_i v_i) and update coefficients
  DBuf tmpA, tmpB;  // hz_apply staging
  DBuf apply_cols;  // hz_apply's column list 0..nrhs-1, grown only when nrhs grows
  int apply_ncols = 0;
  cudaEvent_t order_ev = nullptr;  // orders the handle's stream after the legacy default stream
  double* h_est = nullptr;  // pinned
  double* h_nrm = nullptr;  // pinned
  int* h_flag = nullptr;    // pinned copy of the second-pass flags
  long long reorth = 0;     // second Gram-Schmidt passes taken (columns x steps)
  std::string err;
  double setup_time = 0, solve_time = 0;
  long long nprec = 0;
  std::vector<double> col_relres;
  std::vector<int> col_iters;
  long long h2d = 0, d2h = 0;
  // learned coarse-grid correction (the network is owned by the caller)
  hz::CoarseNet* net = nullptr;    // 2D network, or
  hz::CoarseNet3* net3 = nullptr;  // 3D network (at most one of the two is attached)
  int net_level = 0;         // level whose correction the network computes
  double net_stag = 0.5;     // restart-cycle residual ratio above which the plain cycle takes over
  bool net_active = false;   // network in use by the running solve
  long long net_calls = 0;   // network applications (blocks of columns)
  int net_fallbacks = 0;     // solves that fell back to the plain cycle
  int net_feat_level = -1;
  double net_h2 = 0.0;       // hx * hy of the network level
  DBuf net_feat;             // per node of the network level: (w^2 m hx hy, gamma / w), float2
  // CUDA graphs of the preconditioner application, one per (orientation, basis
  // index, active columns, form); launch-table deltas of the captured kernels
  struct CycleGraph {
    cudaGraphExec_t exec = nullptr;
    long long seen = 0;      // applications with this key (captured on the second)
    long long launches = 0;  // kernels in the graph
    double bytes = 0.0;
    double flops = 0.0;      // algorithmic flops of the captured kernels that count theirs
    std::vector<std::pair<int, long long>> counts;
  };
  std::map<std::tuple<int, int, int, int>, CycleGraph> graphs;
  long long graph_gen = -1;
  bool graphs_off = false;  // a capture failed: eager launches from then on
  int tuned_cols = -1;      // column count the stencil launch shapes were tuned for
  // capture of the right-hand sides handed to one level (training pairs)
  bool cap_on = false;
  int cap_level = 0;
  long long cap_count = 0, cap_max = 0;
  DBuf cap_buf;
};

namespace {

using clk = std::chrono::steady_clock;
double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

template <typename T> struct PrecT;
template <> struct PrecT<double> { static constexpr bool fp64 = true; };
template <> struct PrecT<float> { static constexpr bool fp64 = false; };

long long num_nodes(const hz_problem& p) {
  long long N = 1;
  for (int d = 0; d < p.dim; ++d) N *= (p.n[d] + 1);
  return N;
}

Grid make_grid(const hz_problem& p) {
  Grid g;
  g.nx = (int)(p.n[0] + 1);
  g.ny = (int)(p.n[1] + 1);
  g.nz = p.dim == 3 ? (int)(p.n[2] + 1) : 1;
  g.N = (long long)g.nx * g.ny * g.nz;
  return g;
}

Grid coarsen(const Grid& f, int dim) {
  if ((f.nx - 1) % 2 || (f.ny - 1) % 2 || (dim == 3 && (f.nz - 1) % 2))
    fail(HZ_ERR_ARG, "cannot coarsen a %dx%dx%d node grid: cell counts must be even on every level", f.nx, f.ny, f.nz);
  Grid c;
  c.nx = (f.nx - 1) / 2 + 1;
  c.ny = (f.ny - 1) / 2 + 1;
  c.nz = dim == 3 ? (f.nz - 1) / 2 + 1 : 1;
  if (c.nx < 2 || c.ny < 2 || (dim == 3 && c.nz < 2)) fail(HZ_ERR_ARG, "too many multigrid levels for this grid");
  c.N = (long long)c.nx * c.ny * c.nz;
  return c;
}

void set_device(hz_handle* h) { ck(cudaSetDevice(h->dev), "cudaSetDevice"); }

void sync(hz_handle* h) {
  ck(cudaStreamSynchronize(h->ctx.stream), "stream sync");
  h->ctx.resolve();
}

// The handle's stream does not synchronise with the legacy default stream by
// itself (it is non-blocking).  Calls that read or write caller-owned device
// memory first make it wait for the work already issued to the legacy default
// stream, where a caller that names no stream puts its copies and kernels.
void order_after_default_stream(hz_handle* h) {
  ck(cudaEventRecord(h->order_ev, cudaStreamLegacy), "record ordering event");
  ck(cudaStreamWaitEvent(h->ctx.stream, h->order_ev, 0), "order after the default stream");
}

// Device X and Y of an operator apply must not overlap: the stencil reads the
// neighbours of a node in X while it writes Y.
void check_no_overlap(const double* X, const double* Y, long long n, int nrhs) {
  const unsigned char* a = reinterpret_cast<const unsigned char*>(X);
  const unsigned char* b = reinterpret_cast<const unsigned char*>(Y);
  const size_t bytes = (size_t)n * (size_t)nrhs * 16;
  if (a < b + bytes && b < a + bytes)
    fail(HZ_ERR_ARG, "X and Y overlap: the operator apply does not work in place");
}

// Diagonals of H and SH on the node grid of problem p (5/7-point Laplacian
// diagonal with the boundary-row rule, plus the mass/Sommerfeld term, plus the
// shift i s w^2 m for SH) and 1/diag(SH).
void fine_diagonals(const hz_problem& p, double s, std::vector<std::complex<double>>& dH,
                    std::vector<std::complex<double>>& dSH, std::vector<std::complex<double>>& iSH) {
  const long long N = num_nodes(p);
  const Grid g = make_grid(p);
  std::vector<std::complex<double>> mass((size_t)N);
  int st = hz_helmholtz_mass(&p, reinterpret_cast<double*>(mass.data()));
  if (st != HZ_OK) fail(st, "invalid problem (mass term)");
  const double BC = p.order_neumann_bc == 1 ? 1.0 : 2.0;
  const double w2 = p.omega_re * p.omega_re;  // the shift uses real omega (GetHelmholtzShiftOP)
  dH.resize((size_t)N);
  dSH.resize((size_t)N);
  iSH.resize((size_t)N);
  for (long long q = 0; q < N; ++q) {
    const int i = (int)(q % g.nx), j = (int)((q / g.nx) % g.ny), k = (int)(q / ((long long)g.nx * g.ny));
    const int pos[3] = {i, j, k};
    const int nn[3] = {g.nx, g.ny, g.nz};
    double lap = 0.0;
    for (int d = 0; d < p.dim; ++d) {
      const bool bnd = pos[d] == 0 || pos[d] == nn[d] - 1;
      lap += (bnd ? BC : 2.0) / (p.h[d] * p.h[d]);
    }
    dH[(size_t)q] = lap + mass[(size_t)q];
    dSH[(size_t)q] = dH[(size_t)q] + std::complex<double>(0.0, s * w2 * p.m[q]);
    iSH[(size_t)q] = 1.0 / dSH[(size_t)q];
  }
}

FineOp make_fineop(const hz_problem& p, int adj) {
  FineOp f{};
  f.g = make_grid(p);
  const double BC = p.order_neumann_bc == 1 ? 1.0 : 2.0;
  for (int d = 0; d < 3; ++d) {
    const double hd = d < p.dim ? p.h[d] : 1.0;
    f.o[d] = 1.0 / (hd * hd);
    f.b[d] = BC / (hd * hd);
  }
  f.adj = adj;
  return f;
}

// Full-weighting average of a nodal field onto the next coarser grid
// (weights of P^T normalised to sum 1 at every coarse node).
std::vector<double> restrict_nodal(const std::vector<double>& f, const Grid& gf, const Grid& gc, int dim) {
  std::vector<double> c((size_t)gc.N);
  for (long long q = 0; q < gc.N; ++q) {
    const int I = (int)(q % gc.nx), J = (int)((q / gc.nx) % gc.ny), K = (int)(q / ((long long)gc.nx * gc.ny));
    double acc = 0.0, wsum = 0.0;
    for (int dk = (dim == 3 ? -1 : 0); dk <= (dim == 3 ? 1 : 0); ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          const int fi = 2 * I + di, fj = 2 * J + dj, fk = 2 * K + dk;
          if (fi < 0 || fi >= gf.nx || fj < 0 || fj >= gf.ny || fk < 0 || fk >= gf.nz) continue;
          const double wgt = (di ? 0.5 : 1.0) * (dj ? 0.5 : 1.0) * (dk ? 0.5 : 1.0);
          acc += wgt * f[(size_t)(fi + (long long)gf.nx * (fj + (long long)gf.ny * fk))];
          wsum += wgt;
        }
    c[(size_t)q] = acc / wsum;
  }
  return c;
}

// Largest coarsest level solved through a dense inverse in the emulated mode
// (A^{-1} takes N^2 x 16 bytes: 1 GiB at this size).
static constexpr long long kDenseCoarseMax = 8192;

// ---- hierarchy setup -------------------------------------------------------

// Stencil offsets per level are all within one node; the banded storage uses
// kl = ku = nx*ny + nx + 1 (3D) or nx + 1 (2D).
// Banded LU of one level's operator (host, FP64) and the dense block operators
// of its blocked solve.
void band_factor_level(hz_handle* h, const Hierarchy& H, const Level& L, std::vector<BandBlock>& blocks,
                       std::vector<std::complex<double>>& T, std::vector<std::complex<double>>& G, int& kl_out,
                       int& ku_out) {
  const Grid g = L.g;
  const int dim = h->prob.dim;
  const long long N = g.N;
  const int bw = dim == 3 ? g.nx * g.ny + g.nx + 1 : g.nx + 1;
  const int kl = bw, ku = bw;
  const long long ldab = 2LL * kl + ku + 1;
  const int ns = dim == 3 ? 27 : 9;
  // gather the stencil coefficients of the coarsest level on the host
  std::vector<std::complex<double>> coef((size_t)ns * N, 0.0);
  if (L.fine) {
    // 5/7-point coarsest level (single-level hierarchy or re-discretised levels)
    std::vector<std::complex<double>> d((size_t)N);
    ck(cudaMemcpy(d.data(), L.fd64, N * 16, cudaMemcpyDeviceToHost), "copy diag");
    for (long long p = 0; p < N; ++p) {
      const int i = (int)(p % g.nx), j = (int)((p / g.nx) % g.ny), k = (int)(p / ((long long)g.nx * g.ny));
      const int center = dim == 3 ? 13 : 4;
      coef[(size_t)center * N + p] = H.adj ? std::conj(d[(size_t)p]) : d[(size_t)p];
      const int pos[3] = {i, j, k};
      const int nn[3] = {g.nx, g.ny, g.nz};
      for (int ax = 0; ax < dim; ++ax) {
        const double o = L.fop.o[ax], b = L.fop.b[ax];
        const int q = pos[ax], n = nn[ax];
        double cl, cr;
        if (!H.adj) {
          cl = (q > 0) ? ((q == n - 1) ? b : o) : 0.0;
          cr = (q < n - 1) ? ((q == 0) ? b : o) : 0.0;
        } else {
          cl = (q > 0) ? ((q - 1 == 0) ? b : o) : 0.0;
          cr = (q < n - 1) ? ((q + 1 == n - 1) ? b : o) : 0.0;
        }
        const int stride = ax == 0 ? 1 : (ax == 1 ? 3 : 9);
        coef[(size_t)(center - stride) * N + p] = -cl;
        coef[(size_t)(center + stride) * N + p] = -cr;
      }
    }
  } else {
    ck(cudaMemcpy(coef.data(), L.coef64.p, (size_t)ns * N * 16, cudaMemcpyDeviceToHost), "copy coarse coef");
  }
  std::vector<std::complex<double>> ab((size_t)(ldab * N), 0.0);
  const int kv = kl + ku;
  for (long long p = 0; p < N; ++p) {
    const int i = (int)(p % g.nx), j = (int)((p / g.nx) % g.ny), k = (int)(p / ((long long)g.nx * g.ny));
    for (int s = 0; s < ns; ++s) {
      const std::complex<double> v = coef[(size_t)s * N + p];
      if (v == 0.0) continue;
      const int ox = s % 3 - 1, oy = (s / 3) % 3 - 1, oz = dim == 3 ? s / 9 - 1 : 0;
      const int ii = i + ox, jj = j + oy, kk = k + oz;
      if (ii < 0 || ii >= g.nx || jj < 0 || jj >= g.ny || kk < 0 || kk >= g.nz) continue;
      const long long q = ii + (long long)g.nx * (jj + (long long)g.ny * kk);
      ab[(size_t)(q * ldab + kv + p - q)] = v;  // A(p, q)
    }
  }
  std::vector<int> ipiv((size_t)N);
  int info = band_lu_factor(N, kl, ku, ab.data(), ipiv.data());
  if (info != 0) fail(HZ_ERR_NUMERIC, "banded LU of a %lld-node level: zero pivot in column %d", N, info);
  // dense block operators of the blocked banded solve, block size kl
  blocks.clear();
  band_block_operators(N, kl, ku, ab.data(), ipiv.data(), std::max(kl, 1), blocks, T, G);
  kl_out = kl;
  ku_out = ku;
}

void factor_coarsest(hz_handle* h, Hierarchy& H) {
  Level& L = *H.lv.back();
  const long long N = L.g.N;
  int kl = 0, ku = 0;
  std::vector<std::complex<double>> T, G;
  band_factor_level(h, H, L, H.band.blocks, T, G, kl, ku);
  H.nc = N;
  H.kl = kl;
  H.ku = ku;
  H.band_df = h->opt.precision == HZ_PREC_MIXED && h->opt.outer_arith == HZ_OUTER_EMULATED;
  H.dense_df = H.band_df && N <= kDenseCoarseMax;
  if (H.dense_df) {
    // emulated-FP64 cycles on a small coarsest level: compute A^{-1} once in FP64
    // (the blocked band solve applied to the identity), store it as df64 and
    // apply it as one dense product per cycle
    DBuf dT, dG, dB, E, W, dc;
    dT.alloc(T.size() * 16);
    dG.alloc(G.size() * 16);
    ck(cudaMemcpy(dT.p, T.data(), T.size() * 16, cudaMemcpyHostToDevice), "upload band forward operators");
    ck(cudaMemcpy(dG.p, G.data(), G.size() * 16, cudaMemcpyHostToDevice), "upload band backward operators");
    dB.alloc(H.band.blocks.size() * sizeof(BandBlock));
    ck(cudaMemcpy(dB.p, H.band.blocks.data(), H.band.blocks.size() * sizeof(BandBlock), cudaMemcpyHostToDevice),
       "upload band blocks");
    BandSolveOps ops;
    ops.N = N;
    ops.blocks = H.band.blocks;
    ops.dblocks = dB.as<BandBlock>();
    ops.T = dT.as<double2>();
    ops.G = dG.as<double2>();
    std::vector<int> all((size_t)N);
    for (long long c = 0; c < N; ++c) all[(size_t)c] = (int)c;
    dc.alloc((size_t)N * sizeof(int));
    ck(cudaMemcpy(dc.p, all.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice), "upload identity columns");
    E.alloc((size_t)N * N * 16);
    W.alloc((size_t)3 * N * N * 16);
    H.dense.alloc((size_t)N * N * 16);
    launch_identity(h->ctx, N, E.as<double2>());
    launch_band_solve<double>(h->ctx, ops, E.as<double2>(), H.dense.as<double2>(), N, dc.as<int>(), (int)N,
                              W.as<double2>());
    launch_inplace_df(h->ctx, N * N, H.dense.as<double2>());
    sync(h);
    H.band.N = N;
    return;
  }
  if (H.band_df) {
    // emulated-FP64 solves: each FP64 entry stored as a (hi, lo) float pair
    auto to_df = [](std::vector<std::complex<double>>& v) {
      for (auto& z : v) {
        const float rh = (float)z.real(), ih = (float)z.imag();
        const float rl = (float)(z.real() - (double)rh), il = (float)(z.imag() - (double)ih);
        float f[4] = {rh, ih, rl, il};
        std::memcpy(&z, f, sizeof(f));
      }
    };
    to_df(T);
    to_df(G);
  }
  H.bandT.alloc(T.size() * 16);
  H.bandG.alloc(G.size() * 16);
  ck(cudaMemcpy(H.bandT.p, T.data(), T.size() * 16, cudaMemcpyHostToDevice), "upload band forward operators");
  ck(cudaMemcpy(H.bandG.p, G.data(), G.size() * 16, cudaMemcpyHostToDevice), "upload band backward operators");
  H.band.N = N;
  H.band.T = H.bandT.as<double2>();
  H.band.G = H.bandG.as<double2>();
  H.bandB.alloc(H.band.blocks.size() * sizeof(BandBlock));
  ck(cudaMemcpy(H.bandB.p, H.band.blocks.data(), H.band.blocks.size() * sizeof(BandBlock), cudaMemcpyHostToDevice),
     "upload band blocks");
  H.band.dblocks = H.bandB.as<BandBlock>();
}

void build_hierarchy(hz_handle* h, int adj) {
  Hierarchy& H = h->hier[adj];
  const int dim = h->prob.dim;
  const int L = std::max(1, h->opt.levels);
  const bool mixed = h->opt.precision == HZ_PREC_MIXED;
  const int ns = dim == 3 ? 27 : 9;
  H.lv.clear();
  H.adj = adj;
  auto l0 = std::make_unique<Level>();
  l0->g = h->g0;
  l0->ld = h->g0.N;
  l0->fine = true;
  l0->fop = h->fop;
  l0->fop.adj = adj;
  l0->fd64 = h->diagSH.as<double2>();
  l0->fi64 = h->dinvSH.as<double2>();
  l0->fd32 = h->diagSH32.as<float2>();
  l0->fi32 = h->dinvSH32.as<float2>();
  H.lv.push_back(std::move(l0));
  if (h->opt.coarse_op == HZ_COARSE_REDISCRETIZE) {
    // the alternative MGsetup path of src/ShiftedLaplacianMultigridSolver.jl:51-62:
    // shift folded into gamma (getShiftedHelmholtzParam), m and gamma restricted
    // to each coarse mesh, operator re-assembled there (h doubles per level)
    const double sre = h->opt.shift * h->prob.omega_re;
    std::vector<double> mf = h->m, gf(h->gamma.size());
    for (size_t q = 0; q < gf.size(); ++q) gf[q] = h->gamma[q] + sre;
    hz_problem pl = h->prob;
    for (int l = 1; l < L; ++l) {
      Level& F = *H.lv[l - 1];
      auto C = std::make_unique<Level>();
      C->g = coarsen(F.g, dim);
      C->ld = C->g.N;
      C->m = restrict_nodal(l == 1 ? mf : F.m, F.g, C->g, dim);
      C->gamma = restrict_nodal(l == 1 ? gf : F.gamma, F.g, C->g, dim);
      for (int d = 0; d < dim; ++d) {
        pl.n[d] /= 2;
        pl.h[d] *= 2.0;
      }
      pl.m = C->m.data();
      pl.gamma = C->gamma.data();
      std::vector<std::complex<double>> dH, dSH, iSH;
      fine_diagonals(pl, 0.0, dH, dSH, iSH);  // the shift is already in gamma
      const long long Nc = C->g.N;
      C->own_d64.alloc((size_t)Nc * 16);
      C->own_i64.alloc((size_t)Nc * 16);
      ck(cudaMemcpy(C->own_d64.p, dSH.data(), Nc * 16, cudaMemcpyHostToDevice), "upload coarse diag");
      ck(cudaMemcpy(C->own_i64.p, iSH.data(), Nc * 16, cudaMemcpyHostToDevice), "upload coarse inverse diag");
      C->fine = true;
      C->fop = make_fineop(pl, adj);
      C->fd64 = C->own_d64.as<double2>();
      C->fi64 = C->own_i64.as<double2>();
      if (mixed) {
        C->own_d32.alloc((size_t)Nc * 8);
        C->own_i32.alloc((size_t)Nc * 8);
        launch_cast<float, double>(h->ctx, C->fd64, C->own_d32.as<float2>(), Nc);
        launch_cast<float, double>(h->ctx, C->fi64, C->own_i32.as<float2>(), Nc);
        C->fd32 = C->own_d32.as<float2>();
        C->fi32 = C->own_i32.as<float2>();
      }
      H.lv.push_back(std::move(C));
    }
    sync(h);
    factor_coarsest(h, H);
    H.built = true;
    return;
  }
  FineOp fop = h->fop;
  fop.adj = adj;
  DBuf pin, pf, pg;
  DBuf dcols;
  std::vector<int> seq(ns);
  for (int s = 0; s < ns; ++s) seq[s] = s;
  dcols.alloc(ns * sizeof(int));
  ck(cudaMemcpy(dcols.p, seq.data(), ns * sizeof(int), cudaMemcpyHostToDevice), "upload probe cols");
  const int* pc = dcols.as<int>();
  for (int l = 0; l + 1 < L; ++l) {
    Level& F = *H.lv[l];
    auto C = std::make_unique<Level>();
    C->g = coarsen(F.g, dim);
    C->ld = C->g.N;
    const long long Nf = F.g.N, Nc = C->g.N;
    pin.alloc((size_t)ns * Nc * 16);
    pf.alloc((size_t)ns * Nf * 16);
    pg.alloc((size_t)ns * Nf * 16);
    launch_probe_init(h->ctx, C->g, dim, pin.as<double2>(), Nc);
    launch_prolong<double>(h->ctx, F.g, C->g, pin.as<double2>(), Nc, nullptr, pf.as<double2>(), Nf, pc, ns);
    if (l == 0)
      launch_fine<double, double, double>(h->ctx, MODE_APPLY, fop, h->diagSH.as<double2>(), nullptr,
                                          pf.as<double2>(), (const double2*)nullptr, pg.as<double2>(), Nf, pc, ns,
                                          0.0);
    else
      launch_rap<double, double>(h->ctx, MODE_APPLY, F.g, F.coef64.as<double2>(), Nf, nullptr, pf.as<double2>(),
                                 (const double2*)nullptr, pg.as<double2>(), Nf, pc, ns, 0.0);
    launch_restrict<double>(h->ctx, F.g, C->g, pg.as<double2>(), Nf, pin.as<double2>(), Nc, pc, ns);
    C->coef64.alloc((size_t)ns * Nc * 16);
    launch_probe_scatter(h->ctx, C->g, dim, pin.as<double2>(), Nc, C->coef64.as<double2>(), Nc);
    C->dinv64.alloc((size_t)Nc * 16);
    launch_center_inverse<double>(h->ctx, C->g, dim, C->coef64.as<double2>(), Nc, C->dinv64.as<double2>());
    if (mixed) {
      C->coef32.alloc((size_t)ns * Nc * 8);
      launch_cast<float, double>(h->ctx, C->coef64.as<double2>(), C->coef32.as<float2>(), (long long)ns * Nc);
      C->dinv32.alloc((size_t)Nc * 8);
      launch_center_inverse<float>(h->ctx, C->g, dim, C->coef64.as<double2>(), Nc, C->dinv32.as<float2>());
    }
    H.lv.push_back(std::move(C));
  }
  sync(h);
  factor_coarsest(h, H);
  H.built = true;
}

// ---- workspace ---------------------------------------------------------------

void ensure_workspace(hz_handle* h, int nrhs) {
  const int m = std::max(1, h->opt.inner);
  if (nrhs <= h->rcap && m <= h->mcap) return;
  const int R = std::max(nrhs, h->rcap);
  const long long N = h->g0.N;
  const bool mixed = h->opt.precision == HZ_PREC_MIXED;
  const size_t zb = mixed ? 8 : 16;
  h->Bd.alloc((size_t)R * N * 16);
  h->Xd.alloc((size_t)R * N * 16);
  h->V.alloc((size_t)std::max(m + 1, 6) * R * N * 16);  // BiCGSTAB uses 6 FP64 blocks
  h->Z.alloc((size_t)std::max(m, 2) * R * N * zb);
  h->bsc.alloc((size_t)R * 8 * 16);
  h->sig.alloc((size_t)R * (m + 1) * sizeof(double));
  h->hC.alloc((size_t)R * (m + 2) * 16);
  const int nblk = krylov_nblk(N, 1);
  h->part.alloc((size_t)R * 18 * nblk * 16);
  const int HS = m + 2;
  h->hA.alloc((size_t)R * HS * 16);
  h->hB.alloc((size_t)R * HS * 16);
  h->nr.alloc((size_t)R * HS * 16);
  h->nr2.alloc((size_t)R * HS * 16);
  h->flag.alloc((size_t)R * sizeof(int));
  h->Hh.alloc((size_t)R * (m + 1) * m * 16);
  h->cs.alloc((size_t)R * m * 16);
  h->sn.alloc((size_t)R * m * 16);
  h->gv.alloc((size_t)R * (m + 1) * 16);
  h->yv.alloc((size_t)R * m * 16);
  h->est.alloc((size_t)R * 8);
  h->invhn.alloc((size_t)R * 8);
  h->bnorm.alloc((size_t)R * 8);
  h->bnorm_inv.alloc((size_t)R * 8);
  h->beta.alloc((size_t)R * 8);
  h->beta_inv.alloc((size_t)R * 8);
  h->cols.alloc((size_t)R * sizeof(int));
  h->kcol.alloc((size_t)R * sizeof(int));
  if (h->h_est) cudaFreeHost(h->h_est);
  if (h->h_nrm) cudaFreeHost(h->h_nrm);
  if (h->h_flag) cudaFreeHost(h->h_flag);
  h->h_est = nullptr;
  h->h_nrm = nullptr;
  h->h_flag = nullptr;
  ck(cudaMallocHost(&h->h_est, (size_t)R * 8), "pinned est");
  ck(cudaMallocHost(&h->h_nrm, (size_t)R * 8), "pinned nrm");
  ck(cudaMallocHost(&h->h_flag, (size_t)R * sizeof(int)), "pinned flags");
  // multigrid work buffers per level and orientation (allocated on demand in the cycle)
  h->rcap = R;
  h->mcap = m;
}

template <typename T>
void ensure_level_buffers(hz_handle* h, Hierarchy& H, int R) {
  const size_t es = sizeof(cplx<T>);
  for (size_t l = 0; l < H.lv.size(); ++l) {
    Level& L = *H.lv[l];
    const size_t bytes = (size_t)R * L.ld * es;
    if (l > 0) {
      L.b.alloc(bytes);
      L.x.alloc(bytes);
    }
    if (l + 1 < H.lv.size()) {
      L.t.alloc(bytes);
      L.r.alloc(bytes);
    }
    if (h->opt.cycle == 'K' && l > 0 && l + 1 < H.lv.size()) {
      L.kv.alloc(5 * bytes);
      L.ks.alloc((size_t)R * 8 * 16);
      L.kp.alloc((size_t)R * 3 * kcycle_nblk(L.g.N) * 16);
    }
    if (h->opt.relax_type == HZ_RELAX_JAC_GMRES && (int)l >= h->opt.relax_from && l + 1 < H.lv.size()) {
      L.gv.alloc(5 * bytes);
      L.gs.alloc((size_t)R * 8 * 16);
      L.gp.alloc((size_t)R * 3 * kcycle_nblk(L.g.N) * 16);
    }
  }
  // band work: 3 vectors per column; the dense product's split-K partials need
  // splits(ncols) * ncols vectors, largest over the active column counts
  long long wcols = 3LL * R;
  if (H.dense_df)
    for (int nc = 1; nc <= R; ++nc) wcols = std::max(wcols, (long long)dense_df_splits(H.nc, nc) * nc);
  H.bandwork.alloc((size_t)wcols * H.nc * 16);
}

// ---- multigrid cycle -----------------------------------------------------------

template <typename T> const cplx<T>* fine_diag(const Level& L);
template <> const double2* fine_diag<double>(const Level& L) { return L.fd64; }
template <> const float2* fine_diag<float>(const Level& L) { return L.fd32; }
template <typename T> const cplx<T>* fine_dinv(const Level& L);
template <> const double2* fine_dinv<double>(const Level& L) { return L.fi64; }
template <> const float2* fine_dinv<float>(const Level& L) { return L.fi32; }
template <typename T> const cplx<T>* lev_coef(Level& L);
template <> const double2* lev_coef<double>(Level& L) { return L.coef64.as<double2>(); }
template <> const float2* lev_coef<float>(Level& L) { return L.coef32.as<float2>(); }
template <typename T> const cplx<T>* lev_dinv(Level& L);
template <> const double2* lev_dinv<double>(Level& L) { return L.dinv64.as<double2>(); }
template <> const float2* lev_dinv<float>(Level& L) { return L.dinv32.as<float2>(); }

// One level operation in precision T with right-hand side of precision TB.
template <typename T, typename TB>
void lev_op(hz_handle* h, Hierarchy& H, int l, int mode, const cplx<T>* x, const cplx<TB>* b, cplx<T>* y,
            const int* cols, int nc) {
  Level& L = *H.lv[l];
  const double w = h->opt.relax_param;
  if (L.fine) {
    launch_fine<T, T, TB>(h->ctx, mode, L.fop, fine_diag<T>(L), fine_dinv<T>(L), x, b, y, L.ld, cols, nc, w);
  } else {
    launch_rap<T, TB>(h->ctx, mode, L.g, lev_coef<T>(L), L.g.N, lev_dinv<T>(L), x, b, y, L.ld, cols, nc, w);
  }
}

template <typename T, typename TB>
void lev_jacobi0(hz_handle* h, Hierarchy& H, int l, const cplx<TB>* b, cplx<T>* y, const int* cols, int nc) {
  Level& L = *H.lv[l];
  const cplx<T>* dinv = L.fine ? fine_dinv<T>(L) : lev_dinv<T>(L);
  launch_jacobi0<T, TB>(h->ctx, L.g, dinv, L.fine ? L.fop.adj : 0, b, y, L.ld, cols, nc, h->opt.relax_param);
}

// Network input features on level l: the medium restricted l times by nodal
// full weighting, as w^2 m hx hy and gamma / w (w = Re omega); hx hy (the
// square of the cell size for the cubic cells of the 3D grids) scales the
// network's output back to an error.
const float2* net_features(hz_handle* h, int l) {
  if (h->net_feat_level == l) return h->net_feat.as<float2>();
  const int dim = h->prob.dim;
  Grid g = h->g0;
  std::vector<double> m = h->m, gm = h->gamma;
  double hx = h->prob.h[0], hy = h->prob.h[1];
  for (int k = 0; k < l; ++k) {
    const Grid c = coarsen(g, dim);
    m = restrict_nodal(m, g, c, dim);
    gm = restrict_nodal(gm, g, c, dim);
    g = c;
    hx *= 2.0;
    hy *= 2.0;
  }
  const double w = h->prob.omega_re;
  std::vector<float2> f((size_t)g.N);
  for (long long p = 0; p < g.N; ++p) f[(size_t)p] = make_float2((float)(w * w * m[p] * hx * hy), (float)(gm[p] / w));
  h->net_feat.alloc((size_t)g.N * sizeof(float2));
  ck(cudaMemcpy(h->net_feat.p, f.data(), (size_t)g.N * sizeof(float2), cudaMemcpyHostToDevice), "upload features");
  h->net_feat_level = l;
  h->net_h2 = hx * hy;
  return h->net_feat.as<float2>();
}

// out = e_l for the active columns of b_l by the network: the coarse-grid
// correction below level l - 1 replaced by one inference (the adjoint solve
// feeds conj(b) and conjugates the result).
template <typename T>
void learned_correction(hz_handle* h, Hierarchy& H, int l, const cplx<T>* b, cplx<T>* out, const int* cols, int nc) {
  Level& L = *H.lv[l];
  const float2* feat = net_features(h, l);
  float* x4;
  float* sc;
  const float* y;
  if (h->net3) {
    hz::CoarseNet3* net = h->net3;
    x4 = net->input_staging(L.g.nx, L.g.ny, L.g.nz, nc);
    sc = net->scale_staging(nc);
    launch_net_pack<T>(h->ctx, L.g.N, b, L.ld, cols, nc, feat, H.adj, sc, x4);
    net->forward(h->ctx, x4, L.g.nx, L.g.ny, L.g.nz, nc);
    y = net->output();
  } else {
    hz::CoarseNet* net = h->net;
    x4 = net->input_staging(L.g.nx, L.g.ny, nc);
    sc = net->scale_staging(nc);
    launch_net_pack<T>(h->ctx, L.g.N, b, L.ld, cols, nc, feat, H.adj, sc, x4);
    net->forward(h->ctx, x4, L.g.nx, L.g.ny, nc);
    y = net->output();
  }
  launch_net_unpack<T>(h->ctx, L.g.N, y, sc, h->net_h2, H.adj, out, L.ld, cols, nc);
  h->net_calls += 1;
}

template <typename T, typename TB>
void mg_cycle(hz_handle* h, Hierarchy& H, int l, const cplx<TB>* b, cplx<T>* out, const int* cols, int nc);

// The preconditioner of a K-cycle step on level k: the level's own cycle, or
// the network when it is attached to level k (it then stands for everything
// below level k - 1 that the cycle would do: smoothing on level k and the
// recursion to the coarsest LU).
template <typename T>
void kcycle_precondition(hz_handle* h, Hierarchy& H, int k, const cplx<T>* v, cplx<T>* z, const int* cols, int nc) {
  if (h->net_active && k == h->net_level)
    learned_correction<T>(h, H, k, v, z, cols, nc);
  else
    mg_cycle<T, T>(h, H, k, v, z, cols, nc);
}

// out = e_k for the active columns of b_k by the K-cycle: two FGMRES steps on
// level k's operator, right-preconditioned by level k's own cycle (zero
// initial guess; Multigrid.jl cycleType 'K').
template <typename T>
void kcycle_correction(hz_handle* h, Hierarchy& H, int k, const cplx<T>* b, cplx<T>* out, const int* cols, int nc) {
  Level& L = *H.lv[k];
  Ctx& c = h->ctx;
  const long long N = L.g.N, ld = L.ld, vs = (long long)h->rcap * ld;
  cplx<T>* base = L.kv.as<cplx<T>>();
  cplx<T>* V0 = base;
  cplx<T>* V1 = base + vs;
  cplx<T>* Z0 = base + 2 * vs;
  cplx<T>* Z1 = base + 3 * vs;
  cplx<T>* W = base + 4 * vs;
  double2* ks = L.ks.as<double2>();
  double2* part = L.kp.as<double2>();
  const cplx<T>* none = nullptr;
  launch_kc_sums<T>(c, N, ld, cols, nc, 0, 1, none, none, b, part, ks, 0);  // beta^2
  launch_kc_scale<T>(c, N, ld, cols, nc, ks, 0, b, V0);
  kcycle_precondition<T>(h, H, k, V0, Z0, cols, nc);
  lev_op<T, T>(h, H, k, MODE_APPLY, Z0, none, W, cols, nc);
  launch_kc_sums<T>(c, N, ld, cols, nc, 1, 0, V0, none, W, part, ks, 1);  // h00
  launch_kc_update<T>(c, N, ld, cols, nc, 1, 1, ks, V0, none, W, part, 2);  // W -= h00 V0, h10^2
  launch_kc_scale<T>(c, N, ld, cols, nc, ks, 2, W, V1);
  kcycle_precondition<T>(h, H, k, V1, Z1, cols, nc);
  lev_op<T, T>(h, H, k, MODE_APPLY, Z1, none, W, cols, nc);
  launch_kc_sums<T>(c, N, ld, cols, nc, 2, 0, V0, V1, W, part, ks, 3);  // h01, h11
  launch_kc_update<T>(c, N, ld, cols, nc, 2, 3, ks, V0, V1, W, part, 5);  // h21^2
  launch_kc_lsq(c, cols, nc, ks);
  launch_kc_combine<T>(c, N, ld, cols, nc, ks, Z0, Z1, out);
}

// Record the right-hand sides handed to the capture level (FP64 cycles only).
template <typename TB>
void capture_rhs(hz_handle* h, Level& L, const cplx<TB>* b, const int* cols, int nc) {
  if constexpr (std::is_same<TB, double>::value) {
    const int k = (int)std::min<long long>(h->cap_max - h->cap_count, nc);
    if (k <= 0) return;
    launch_gather_cols(h->ctx, L.g.N, b, L.ld, cols, k, h->cap_buf.as<double2>() + h->cap_count * L.g.N);
    h->cap_count += k;
  }
}

// x += the relaxType "Jac-GMRES" smoothing step on level l: `steps` (1 or 2)
// Arnoldi steps of GMRES on the level's operator from the current x,
// right-preconditioned by one damped-Jacobi sweep (Z_j = w D^-1 V_j), and the
// least-squares update x += sum_j y_j Z_j per column.  The K-cycle's kernels
// with the smoother's own buffers; a column with zero residual is unchanged.
template <typename T, typename TB>
void gmres_smooth(hz_handle* h, Hierarchy& H, int l, const cplx<TB>* b, cplx<T>* x, const int* cols, int nc,
                  int steps) {
  Level& L = *H.lv[l];
  Ctx& c = h->ctx;
  const long long N = L.g.N, ld = L.ld, vs = (long long)h->rcap * ld;
  cplx<T>* base = L.gv.as<cplx<T>>();
  if (!base || !L.gs.p || !L.gp.p) fail(HZ_ERR_STATE, "internal: GMRES smoothing buffers missing on level %d", l);
  cplx<T>* V0 = base;
  cplx<T>* V1 = base + vs;
  cplx<T>* Z0 = base + 2 * vs;
  cplx<T>* Z1 = base + 3 * vs;
  cplx<T>* W = base + 4 * vs;
  double2* ks = L.gs.as<double2>();
  double2* part = L.gp.as<double2>();
  const cplx<T>* none = nullptr;
  lev_op<T, TB>(h, H, l, MODE_RESID, x, b, W, cols, nc);                    // W = b - A x
  launch_kc_sums<T>(c, N, ld, cols, nc, 0, 1, none, none, W, part, ks, 0);  // beta^2
  launch_kc_scale<T>(c, N, ld, cols, nc, ks, 0, W, V0);
  lev_jacobi0<T, T>(h, H, l, V0, Z0, cols, nc);                              // Z0 = w D^-1 V0
  lev_op<T, T>(h, H, l, MODE_APPLY, Z0, none, W, cols, nc);
  launch_kc_sums<T>(c, N, ld, cols, nc, 1, 0, V0, none, W, part, ks, 1);     // h00
  launch_kc_update<T>(c, N, ld, cols, nc, 1, 1, ks, V0, none, W, part, 2);   // W -= h00 V0, h10^2
  if (steps == 1) {
    launch_kc_lsq1(c, cols, nc, ks);
    launch_kc_combine_add<T>(c, N, ld, cols, nc, ks, Z0, Z0, x);  // y1 = 0
    return;
  }
  launch_kc_scale<T>(c, N, ld, cols, nc, ks, 2, W, V1);
  lev_jacobi0<T, T>(h, H, l, V1, Z1, cols, nc);                              // Z1 = w D^-1 V1
  lev_op<T, T>(h, H, l, MODE_APPLY, Z1, none, W, cols, nc);
  launch_kc_sums<T>(c, N, ld, cols, nc, 2, 0, V0, V1, W, part, ks, 3);       // h01, h11
  launch_kc_update<T>(c, N, ld, cols, nc, 2, 3, ks, V0, V1, W, part, 5);     // h21^2
  launch_kc_lsq(c, cols, nc, ks);
  launch_kc_combine_add<T>(c, N, ld, cols, nc, ks, Z0, Z1, x);
}

// C.x = the coarse-grid correction of level l + 1 for the right-hand sides in C.b:
// the network, a K-cycle step or a recursive cycle.
template <typename T>
void coarse_correction(hz_handle* h, Hierarchy& H, int l, const int* cols, int nc) {
  Level& C = *H.lv[l + 1];
  const int last = (int)H.lv.size() - 1;
  // K-cycle: the network preconditions the two FGMRES steps on its level
  // (kcycle_precondition); V and W cycles: it replaces the level's cycle
  if (h->net_active && l + 1 == h->net_level && !(h->opt.cycle == 'K' && l + 1 < last))
    learned_correction<T>(h, H, l + 1, C.b.as<cplx<T>>(), C.x.as<cplx<T>>(), cols, nc);
  else if (h->opt.cycle == 'K' && l + 1 < last)
    kcycle_correction<T>(h, H, l + 1, C.b.as<cplx<T>>(), C.x.as<cplx<T>>(), cols, nc);
  else
    mg_cycle<T, T>(h, H, l + 1, C.b.as<cplx<T>>(), C.x.as<cplx<T>>(), cols, nc);
}

// x_out = cycle(b) on level l with zero initial guess.
template <typename T, typename TB>
void mg_cycle(hz_handle* h, Hierarchy& H, int l, const cplx<TB>* b, cplx<T>* out, const int* cols, int nc) {
  Level& L = *H.lv[l];
  const int last = (int)H.lv.size() - 1;
  if (h->cap_on && l == h->cap_level) capture_rhs<TB>(h, L, b, cols, nc);
  if (l == last) {
    if (!std::is_same<T, TB>::value) fail(HZ_ERR_STATE, "single-level mixed hierarchy is not supported");
    if (H.dense_df)
      launch_dense_df(h->ctx, H.nc, H.dense.as<float4>(), (const float2*)b, (float2*)out, L.ld, cols, nc,
                      H.bandwork.as<double2>());
    else if (H.band_df)
      launch_band_solve_df<float>(h->ctx, H.band, (const float2*)b, (float2*)out, L.ld, cols, nc,
                                  H.bandwork.as<float4>());
    else
      launch_band_solve<T>(h->ctx, H.band, (const cplx<T>*)b, out, L.ld, cols, nc, H.bandwork.as<double2>());
    return;
  }
  Level& C = *H.lv[l + 1];
  const int pre = std::max(0, h->opt.relax_pre), post = std::max(0, h->opt.relax_post);
  cplx<T>* tb = L.t.as<cplx<T>>();
  cplx<T>* rb = L.r.as<cplx<T>>();
  // choose the first buffer so that the last Jacobi sweep lands in `out`
  const int writes = (pre > 0 ? pre : 0) + post;
  cplx<T>* cur;
  cplx<T>* oth;
  if (pre > 0) {
    cur = (writes % 2 == 1) ? out : tb;
    oth = (cur == out) ? tb : out;
  } else {
    cur = (post % 2 == 0) ? out : tb;
    oth = (cur == out) ? tb : out;
  }
  const int ncalls = (h->opt.cycle == 'W' && l + 1 < last) ? 2 : 1;
  if (h->opt.relax_type == HZ_RELAX_JAC_GMRES && l >= h->opt.relax_from) {
    // relaxType "Jac-GMRES": smoothing steps update `out` in place
    launch_zero_cols<T>(h->ctx, L.g.N, out, L.ld, cols, nc);
    if (pre > 0) gmres_smooth<T, TB>(h, H, l, b, out, cols, nc, pre);
    for (int call = 0; call < ncalls; ++call) {
      lev_op<T, TB>(h, H, l, MODE_RESID, out, b, rb, cols, nc);
      launch_restrict<T>(h->ctx, L.g, C.g, rb, L.ld, C.b.as<cplx<T>>(), C.ld, cols, nc);
      coarse_correction<T>(h, H, l, cols, nc);
      launch_prolong<T>(h->ctx, L.g, C.g, C.x.as<cplx<T>>(), C.ld, out, out, L.ld, cols, nc);
    }
    if (post > 0) gmres_smooth<T, TB>(h, H, l, b, out, cols, nc, post);
    return;
  }
  bool zero_guess = true;
  if (pre > 0) {
    lev_jacobi0<T, TB>(h, H, l, b, cur, cols, nc);
    for (int s = 1; s < pre; ++s) {
      lev_op<T, TB>(h, H, l, MODE_JACOBI, cur, b, oth, cols, nc);
      std::swap(cur, oth);
    }
    zero_guess = false;
  }
  for (int call = 0; call < ncalls; ++call) {
    if (zero_guess) {
      // residual = b: restrict b directly
      if (std::is_same<T, TB>::value) {
        launch_restrict<T>(h->ctx, L.g, C.g, (const cplx<T>*)b, L.ld, C.b.as<cplx<T>>(), C.ld, cols, nc);
      } else {
        launch_cast_cols<T, TB>(h->ctx, L.g.N, b, L.ld, rb, L.ld, cols, nc);
        launch_restrict<T>(h->ctx, L.g, C.g, rb, L.ld, C.b.as<cplx<T>>(), C.ld, cols, nc);
      }
    } else {
      lev_op<T, TB>(h, H, l, MODE_RESID, cur, b, rb, cols, nc);
      launch_restrict<T>(h->ctx, L.g, C.g, rb, L.ld, C.b.as<cplx<T>>(), C.ld, cols, nc);
    }
    coarse_correction<T>(h, H, l, cols, nc);
    launch_prolong<T>(h->ctx, L.g, C.g, C.x.as<cplx<T>>(), C.ld, zero_guess ? nullptr : cur, cur, L.ld, cols, nc);
    zero_guess = false;
  }
  for (int s = 0; s < post; ++s) {
    lev_op<T, TB>(h, H, l, MODE_JACOBI, cur, b, oth, cols, nc);
    std::swap(cur, oth);
  }
  if (cur != out) fail(HZ_ERR_STATE, "internal: cycle result not in output buffer");
}

// Z_j = M^{-1} V_j for the active columns.
void precondition(hz_handle* h, Hierarchy& H, const double2* vj, void* zj, const int* cols, int nc) {
  if (h->opt.precision == HZ_PREC_MIXED) {
    if (H.lv.size() == 1) {
      // single level: FP64 band solve then cast
      fail(HZ_ERR_ARG, "mixed precision needs at least 2 multigrid levels");
    }
    mg_cycle<float, double>(h, H, 0, vj, (float2*)zj, cols, nc);
  } else {
    mg_cycle<double, double>(h, H, 0, vj, (double2*)zj, cols, nc);
  }
}

// y = H x (outer operator, FP64 arithmetic) for the active columns.
template <typename TX>
void apply_H(hz_handle* h, int adj, int mode, const cplx<TX>* x, const double2* b, double2* y, const int* cols,
             int nc) {
  FineOp fop = h->fop;
  fop.adj = adj;
  fop.outer = 1;
  launch_fine<double, TX, double>(h->ctx, mode, fop, h->diagH.as<double2>(), nullptr, x, b, y, h->g0.N, cols, nc,
                                  0.0);
}

void upload_cols(hz_handle* h, const std::vector<int>& c) {
  ck(cudaMemcpyAsync(h->cols.p, c.data(), c.size() * sizeof(int), cudaMemcpyHostToDevice, h->ctx.stream),
     "upload cols");
  // the host vector must stay valid until the copy is done
  ck(cudaStreamSynchronize(h->ctx.stream), "sync cols");
}

// Column 2-norms of a block into host memory.
void col_norms(hz_handle* h, const double2* x, const std::vector<int>& cols, double* dev_nrm, double* dev_inv,
               double* host_out) {
  const long long N = h->g0.N;
  const int nc = (int)cols.size();
  const int nblk = krylov_nblk(N, nc);
  const int* dc = h->cols.as<int>();
  const int HS = h->mcap + 2;
  launch_dots(h->ctx, N, x, 0, N, 0, 0, x, N, dc, nc, nblk, 1, h->part.as<double2>());
  launch_reduce(h->ctx, h->part.as<double2>(), dc, nc, 1, nblk, h->nr.as<double2>(), HS, 0);
  launch_norms(h->ctx, h->nr.as<double2>(), HS, 0, dc, nc, dev_nrm, dev_inv);
  if (host_out) {
    ck(cudaMemcpyAsync(h->h_nrm, dev_nrm, (size_t)h->rcap * 8, cudaMemcpyDeviceToHost, h->ctx.stream), "norms d2h");
    sync(h);
    for (int c : cols) host_out[c] = h->h_nrm[c];
  }
}

// ---- autotuner -----------------------------------------------------------------
// The launch shape of the fine-level and Galerkin stencils (how many CTAs a
// launch aims at, hence how many right-hand sides each block loops over) is
// timed on the handle's own level sizes at its first solve with a given
// column count, and the fastest kept.  Results are cached per process and,
// when HELMGPU_TUNE_CACHE names a file, persisted there as "key fine rap" lines.
std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune;
bool g_tune_loaded = false;

std::string tune_key(const hz_handle* h, int ncols) {
  cudaDeviceProp pr{};
  cudaGetDeviceProperties(&pr, h->dev);
  std::string gpu = pr.name;
  for (char& ch : gpu)
    if (ch == ' ' || ch == '|') ch = '_';
  char buf[384];
  snprintf(buf, sizeof(buf), "%s|sm%d|d%d|%dx%dx%d|c%d|p%d|o%d|L%d|k%d", gpu.c_str(), pr.multiProcessorCount,
           h->prob.dim, h->g0.nx, h->g0.ny, h->g0.nz, ncols, h->opt.precision, h->opt.outer_arith, h->opt.levels,
           h->opt.coarse_op);
  return buf;
}

void tune_cache_load() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = std::getenv("HELMGPU_TUNE_CACHE");
  if (!path || !*path) return;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    std::string key;
    int a = 0, b = 0;
    if (is >> key >> a >> b && a >= 0 && b >= 0) g_tune[key] = {a, b};
  }
}

void tune_cache_store(const std::string& key, int fine, int rap) {
  g_tune[key] = {fine, rap};
  const char* path = std::getenv("HELMGPU_TUNE_CACHE");
  if (!path || !*path) return;
  std::ofstream f(path, std::ios::app);
  if (f) f << key << ' ' << fine << ' ' << rap << '\n';
}

// average milliseconds of one call of f on the handle's stream (1 untimed + 3 timed)
template <typename F>
double time_call(hz_handle* h, F&& f) {
  cudaEvent_t a, b;
  ck(cudaEventCreate(&a), "event");
  ck(cudaEventCreate(&b), "event");
  f();
  cudaEventRecord(a, h->ctx.stream);
  for (int r = 0; r < 3; ++r) f();
  cudaEventRecord(b, h->ctx.stream);
  ck(cudaEventSynchronize(b), "tune sync");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / 3.0;
}

template <typename T>
void autotune(hz_handle* h, Hierarchy& H, int nrhs) {
  const std::string key = tune_key(h, nrhs);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache_load();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      h->ctx.tune_fine = it->second.first;
      h->ctx.tune_rap = it->second.second;
      return;
    }
  }
  Ctx& c = h->ctx;
  // the tuning launches stay out of the launch table and the statistics
  const bool prof = c.profile;
  c.profile = false;
  const auto counts0 = c.counts;
  const auto bytes0 = c.alg_bytes;
  const auto flops0 = c.alg_flops;
  const long long l0 = c.launches;
  ensure_level_buffers<T>(h, H, h->rcap);
  std::vector<int> all(nrhs);
  for (int q = 0; q < nrhs; ++q) all[q] = q;
  upload_cols(h, all);
  const int* dc = h->cols.as<int>();
  static const int mult[] = {0, 1, 2, 4, 16, 32};  // CTAs per SM aimed at; 0: the default rule (8 per SM)
  int sms = 0;
  ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->dev), "SM count");
  auto pick = [&](int& knob, Level& L, cplx<T>* x, cplx<T>* bb, cplx<T>* y, int level) {
    const size_t bytes = (size_t)nrhs * L.ld * sizeof(cplx<T>);
    ck(cudaMemsetAsync(x, 0, bytes, c.stream), "tune zero");
    ck(cudaMemsetAsync(bb, 0, bytes, c.stream), "tune zero");
    double best = 1e300;
    int best_v = 0;
    for (int m : mult) {
      knob = m * sms;
      const double ms = time_call(h, [&] { lev_op<T, T>(h, H, level, MODE_RESID, x, bb, y, dc, nrhs); });
      if (ms < best * 0.97) {  // a change must win by 3 %
        best = ms;
        best_v = knob;
      }
    }
    knob = best_v;
  };
  Level& L0 = *H.lv[0];
  if (H.lv.size() > 1) {
    // level 0 has two work blocks of its own; the residual goes to the Z workspace
    pick(c.tune_fine, L0, L0.t.as<cplx<T>>(), L0.r.as<cplx<T>>(), reinterpret_cast<cplx<T>*>(h->Z.p), 0);
    if (H.lv.size() > 2 && !H.lv[1]->fine) {
      Level& L1 = *H.lv[1];
      pick(c.tune_rap, L1, L1.x.as<cplx<T>>(), L1.b.as<cplx<T>>(), L1.r.as<cplx<T>>(), 1);
    }
  }
  sync(h);
  c.counts = counts0;
  c.alg_bytes = bytes0;
  c.alg_flops = flops0;
  c.counts.resize(c.names.size(), 0);
  c.alg_bytes.resize(c.names.size(), 0.0);
  c.alg_flops.resize(c.names.size(), 0.0);
  c.timed.resize(c.names.size(), 0);
  c.total_ms.resize(c.names.size(), 0.0);
  c.launches = l0;
  c.profile = prof;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_cache_store(key, c.tune_fine, c.tune_rap);
}

void drop_graphs(hz_handle* h) {
  for (auto& kv : h->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  h->graphs.clear();
}

// Run body (the launches of one preconditioner application) through a CUDA
// graph: captured on the second application with the same key, replayed from
// then on.  The graph's kernels keep their launch counts in the table; with
// profiling on, a replay is timed as one "vcycle_graph" entry carrying the
// algorithmic bytes of all its kernels.  A failed capture (an API the graph
// cannot hold) turns graphs off for the handle and runs the body eagerly.
template <typename F>
void cycle_graph(hz_handle* h, int adj, int j, int nl, int form, F&& body) {
  if (!h->opt.cuda_graph || h->graphs_off || h->net_active || h->cap_on) {
    body();
    return;
  }
  const long long gen = g_alloc_gen.load();
  if (gen != h->graph_gen) {
    drop_graphs(h);
    h->graph_gen = gen;
  }
  Ctx& c = h->ctx;
  auto& cg = h->graphs[std::make_tuple(adj, j, nl, form)];
  if (!cg.exec) {
    if (++cg.seen < 2) {
      body();
      return;
    }
    const bool prof = c.profile;
    c.profile = false;
    const std::vector<long long> counts0 = c.counts;
    const std::vector<double> bytes0 = c.alg_bytes;
    const std::vector<double> flops0 = c.alg_flops;
    const long long l0 = c.launches;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      try {
        body();
      } catch (...) {
        ok = false;
      }
      const cudaError_t e = cudaStreamEndCapture(c.stream, &g);
      ok = ok && e == cudaSuccess && g != nullptr;
    }
    if (ok && cudaGraphInstantiate(&cg.exec, g, 0) != cudaSuccess) {
      ok = false;
      cg.exec = nullptr;
    }
    if (g) cudaGraphDestroy(g);
    c.profile = prof;
    // capture recorded the kernels in the launch table without running them: move the deltas to the graph
    cg.launches = c.launches - l0;
    c.launches = l0;
    cg.counts.clear();
    cg.bytes = 0.0;
    cg.flops = 0.0;
    for (size_t i = 0; i < c.counts.size(); ++i) {
      const long long c0 = i < counts0.size() ? counts0[i] : 0;
      const double b0 = i < bytes0.size() ? bytes0[i] : 0.0;
      const double f0 = i < flops0.size() ? flops0[i] : 0.0;
      if (c.counts[i] != c0) cg.counts.push_back({(int)i, c.counts[i] - c0});
      cg.bytes += c.alg_bytes[i] - b0;
      cg.flops += c.alg_flops[i] - f0;
      c.counts[i] = c0;
      c.alg_bytes[i] = b0;
      c.alg_flops[i] = f0;
    }
    if (!ok) {
      cudaGetLastError();
      h->graphs_off = true;
      if (h->opt.verbose) fprintf(stderr, "helmgpu: CUDA graph capture failed, cycles run eagerly\n");
      body();
      return;
    }
  }
  const int gid = c.name_id("vcycle_graph");
  cudaEvent_t a = nullptr;
  c.before(gid, &a);
  ck(cudaGraphLaunch(cg.exec, c.stream), "cudaGraphLaunch");
  c.after(gid, a, cg.bytes);
  if (cg.flops != 0.0) c.alg_flops[gid] += cg.flops;
  c.launches += cg.launches - 1;  // after() counted the graph as one launch
  for (auto& pc : cg.counts) c.counts[pc.first] += pc.second;
}

// FGMRES(m) on H (or H^H) right-preconditioned by one multigrid cycle.
int fgmres(hz_handle* h, int adj, int nrhs) {
  Hierarchy& H = h->hier[adj];
  const long long N = h->g0.N;
  const int m = h->mcap;
  const int HS = m + 2;
  const bool mixed = h->opt.precision == HZ_PREC_MIXED;
  const size_t zb = mixed ? 8 : 16;
  double2* B = h->Bd.as<double2>();
  double2* X = h->Xd.as<double2>();
  double2* V = h->V.as<double2>();
  const long long vstride = h->rcap;
  auto Vj = [&](int j) { return V + (long long)j * vstride * N; };
  auto Zj = [&](int j) { return (char*)h->Z.p + (size_t)j * vstride * N * zb; };
  double2* part = h->part.as<double2>();
  int* dc = h->cols.as<int>();

  std::vector<int> all(nrhs);
  for (int c = 0; c < nrhs; ++c) all[c] = c;
  upload_cols(h, all);
  std::vector<double> bn(nrhs, 0.0), rn(nrhs, 0.0);
  col_norms(h, B, all, h->bnorm.as<double>(), h->bnorm_inv.as<double>(), bn.data());
  launch_zero_cols<double>(h->ctx, N, X, N, dc, nrhs);
  h->col_relres.assign(nrhs, 0.0);
  h->col_iters.assign(nrhs, 0);
  std::vector<int> act;
  for (int c = 0; c < nrhs; ++c) {
    if (!std::isfinite(bn[c])) fail(HZ_ERR_NUMERIC, "right-hand side column %d holds NaN or Inf", c);
    if (bn[c] > 0) act.push_back(c);
  }
  if (act.empty()) return 0;
  // the network (a nonlinear preconditioner: FGMRES only) serves until a restart
  // cycle reduces some column's residual by less than net_stag
  struct NetScope {
    hz_handle* h;
    ~NetScope() { h->net_active = false; }
  } net_scope{h};
  h->net_active = h->net != nullptr || h->net3 != nullptr;
  std::vector<double> prev = bn;
  if (mixed)
    ensure_level_buffers<float>(h, H, h->rcap);
  else
    ensure_level_buffers<double>(h, H, h->rcap);
  const double tol = h->opt.rel_tol;
  // emulated-FP64 outer arithmetic: the basis V holds df64 values (float4, same size as double2)
  const bool df = mixed && h->opt.outer_arith == HZ_OUTER_EMULATED;
  float4* Vd = reinterpret_cast<float4*>(V);
  auto Vdj = [&](int j) { return Vd + (long long)j * vstride * N; };
  // r0 = b (x0 = 0): V_0 = b / ||b||
  upload_cols(h, act);
  if (df)
    launch_to_df(h->ctx, N, B, N, Vdj(0), N, h->bnorm_inv.as<double>(), dc, (int)act.size());
  else
    launch_scale_cols(h->ctx, N, B, N, Vj(0), N, h->bnorm_inv.as<double>(), dc, (int)act.size());
  launch_cycle_init(h->ctx, m, dc, (int)act.size(), h->bnorm.as<double>(), h->gv.as<double2>());
  // the basis is normalised lazily: stored v_i stands for sig_i v_i (V_0 is normalised)
  double* sig = h->sig.as<double>();
  double2* hC = h->hC.as<double2>();
  const int SS = m + 1;
  launch_sig_init(h->ctx, dc, (int)act.size(), sig, SS);
  std::vector<int> kcol(h->rcap, 0);
  int outer = 0;
  for (outer = 1; outer <= std::max(1, h->opt.max_outer); ++outer) {
    std::vector<int> live = act;
    std::fill(kcol.begin(), kcol.end(), 0);
    for (int j = 0; j < m && !live.empty(); ++j) {
      upload_cols(h, live);
      const int nl = (int)live.size();
      double2* w = Vj(j + 1);
      if (df) {
        // the cycle reads the high parts of the df64 basis vector as its FP32 right-hand side
        cycle_graph(h, adj, j, nl, 2, [&] { mg_cycle<float, df64_tag>(h, H, 0, Vdj(j), (float2*)Zj(j), dc, nl); });
        FineOp fop = h->fop;
        fop.adj = adj;
        launch_fine_df64(h->ctx, fop, h->diagHdf.as<float4>(), (const float2*)Zj(j), Vdj(j + 1), N, dc, nl);
      } else {
        cycle_graph(h, adj, j, nl, mixed ? 1 : 0, [&] { precondition(h, H, Vj(j), Zj(j), dc, nl); });
        if (mixed)
          apply_H<float>(h, adj, MODE_APPLY, (const float2*)Zj(j), nullptr, w, dc, nl);
        else
          apply_H<double>(h, adj, MODE_APPLY, (const double2*)Zj(j), nullptr, w, dc, nl);
      }
      // classical Gram-Schmidt with the DGKS test: pass 1 (dots + ||w||^2,
      // update + ||w'||^2) for every column, pass 2 only for the columns whose
      // norm dropped below 1/sqrt(2) of its value (masked on the device)
      const int K = j + 1;
      const int nblk = krylov_nblk(N, nl);
      double2* hA = h->hA.as<double2>();
      double2* hB = h->hB.as<double2>();
      int* flag = h->flag.as<int>();
      for (int pass = 0; pass < 2; ++pass) {
        double2* hh = pass == 0 ? hA : hB;
        double2* nrm = pass == 0 ? h->nr.as<double2>() : h->nr2.as<double2>();
        const int* mask = pass == 0 ? nullptr : flag;
        for (int i0 = 0; i0 < K; i0 += 16) {
          const int k = std::min(16, K - i0);
          const int wn = (pass == 0 && i0 + 16 >= K) ? 1 : 0;  // ||w||^2 before the update (slot K)
          if (df)
            launch_dots_df(h->ctx, N, Vd, vstride, N, i0, k, Vdj(j + 1), N, dc, nl, nblk, wn, part, mask);
          else
            launch_dots(h->ctx, N, V, vstride, N, i0, k, w, N, dc, nl, nblk, wn, part, mask);
          launch_reduce(h->ctx, part, dc, nl, k + wn, nblk, hh + i0, HS, 0);
        }
        // update coefficients for the stored vectors: sig_i^2 d_i
        launch_sig_coef(h->ctx, dc, nl, K, sig, SS, hh, HS, hC);
        for (int i0 = 0; i0 < K; i0 += 16) {
          const int k = std::min(16, K - i0);
          const int wn = (i0 + 16 >= K) ? 1 : 0;
          if (df)
            launch_update_df(h->ctx, N, Vd, vstride, N, i0, k, hC, HS, Vdj(j + 1), N, dc, nl, nblk, wn, part, mask);
          else
            launch_update(h->ctx, N, V, vstride, N, i0, k, hC, HS, w, N, dc, nl, nblk, wn, part, mask);
          if (wn) launch_reduce(h->ctx, part, dc, nl, 1, nblk, nrm, HS, 0);
        }
        if (pass == 0) launch_dgks(h->ctx, dc, nl, hA, HS, K, h->nr.as<double2>(), HS, flag);
      }
      // Hessenberg entries of the normalised basis: sig_i sig_j d_i, h_{j+1,j} = sig_j ||w''||
      launch_sig_true(h->ctx, j, dc, nl, sig, SS, hA, hB, h->nr.as<double2>(), h->nr2.as<double2>(), HS);
      launch_arnoldi_step(h->ctx, j, m, dc, nl, hA, hB, h->nr.as<double2>(), h->nr2.as<double2>(), flag, HS,
                          h->Hh.as<double2>(), h->cs.as<double2>(), h->sn.as<double2>(), h->gv.as<double2>(),
                          h->est.as<double>(), h->invhn.as<double>());
      // v_{j+1} = w'' stays unnormalised: sig_{j+1} = sig_j / h_{j+1,j}
      launch_sig_next(h->ctx, j, dc, nl, sig, SS, h->invhn.as<double>());
      ck(cudaMemcpyAsync(h->h_est, h->est.p, (size_t)h->rcap * 8, cudaMemcpyDeviceToHost, h->ctx.stream), "est");
      ck(cudaMemcpyAsync(h->h_flag, h->flag.p, (size_t)h->rcap * sizeof(int), cudaMemcpyDeviceToHost, h->ctx.stream),
         "flags");
      sync(h);
      {
        int n2 = 0;  // columns that took the second Gram-Schmidt pass
        for (int c : live) n2 += h->h_flag[c] ? 1 : 0;
        h->ctx.add_bytes("krylov_dots", (double)N * n2 * (K + 1) * 16.0);
        h->ctx.add_bytes("krylov_update", (double)N * n2 * (K + 2) * 16.0);
        if (!df) {  // the second pass's FP64 arithmetic (no ||w||^2 in its dots)
          h->ctx.add_flops("krylov_dots", (double)N * n2 * 8.0 * K);
          h->ctx.add_flops("krylov_update", (double)N * n2 * (8.0 * K + 4.0));
        }
        h->reorth += n2;
      }
      std::vector<int> still;
      for (int c : live) {
        kcol[c] = j + 1;
        h->col_iters[c] += 1;
        h->nprec += 1;
        const double e = h->h_est[c];
        if (!std::isfinite(e)) fail(HZ_ERR_NUMERIC, "FGMRES breakdown (NaN/Inf) in column %d", c);
        if (!(e / bn[c] <= tol)) still.push_back(c);
      }
      live.swap(still);
    }
    // x += Z y
    upload_cols(h, act);
    ck(cudaMemcpyAsync(h->kcol.p, kcol.data(), (size_t)h->rcap * sizeof(int), cudaMemcpyHostToDevice,
                       h->ctx.stream),
       "kcol");
    launch_lsq(h->ctx, m, dc, (int)act.size(), h->kcol.as<int>(), h->Hh.as<double2>(), h->gv.as<double2>(),
               h->yv.as<double2>());
    // Z_i = sig_i Z'_i (the cycles scale with their input): fold sig_i into y_i
    launch_sig_y(h->ctx, dc, (int)act.size(), h->kcol.as<int>(), sig, SS, h->yv.as<double2>(), m);
    long long zcols = 0;
    for (int c : act) zcols += kcol[c];
    if (df)
      launch_update_x_df(h->ctx, N, (const float2*)h->Z.p, vstride, N, h->kcol.as<int>(), h->yv.as<double2>(), m, X,
                         N, dc, (int)act.size(), zcols);
    else if (mixed)
      launch_update_x<float>(h->ctx, N, (const float2*)h->Z.p, vstride, N, h->kcol.as<int>(), h->yv.as<double2>(), m,
                             X, N, dc, (int)act.size(), zcols);
    else
      launch_update_x<double>(h->ctx, N, (const double2*)h->Z.p, vstride, N, h->kcol.as<int>(), h->yv.as<double2>(),
                              m, X, N, dc, (int)act.size(), zcols);
    // true residual r = b - H x into V_0, its norm, convergence test
    apply_H<double>(h, adj, MODE_RESID, X, B, Vj(0), dc, (int)act.size());
    col_norms(h, Vj(0), act, h->beta.as<double>(), h->beta_inv.as<double>(), rn.data());
    std::vector<int> next;
    for (int c : act) {
      h->col_relres[c] = rn[c] / bn[c];
      if (!std::isfinite(rn[c])) fail(HZ_ERR_NUMERIC, "residual of column %d is NaN or Inf", c);
      if (!(h->col_relres[c] <= tol)) next.push_back(c);
    }
    if (h->net_active) {
      for (int c : next)
        if (!(rn[c] <= h->net_stag * prev[c])) {
          h->net_active = false;
          h->net_fallbacks += 1;
          if (h->opt.verbose) fprintf(stderr, "helmgpu: learned correction stagnated, plain cycle takes over\n");
          break;
        }
    }
    for (int c : act) prev[c] = rn[c];
    act.swap(next);
    if (act.empty()) break;
    if (outer == std::max(1, h->opt.max_outer)) break;
    upload_cols(h, act);
    if (df)  // r (FP64) -> V_0 (df64) in place
      launch_to_df(h->ctx, N, Vj(0), N, Vdj(0), N, h->beta_inv.as<double>(), dc, (int)act.size());
    else
      launch_scale_cols(h->ctx, N, Vj(0), N, Vj(0), N, h->beta_inv.as<double>(), dc, (int)act.size());
    launch_cycle_init(h->ctx, m, dc, (int)act.size(), h->beta.as<double>(), h->gv.as<double2>());
    launch_sig_init(h->ctx, dc, (int)act.size(), sig, SS);
  }
  return std::min(outer, std::max(1, h->opt.max_outer));
}

// Right-preconditioned BiCGSTAB on H (or H^H), one multigrid cycle per
// preconditioner application (solveBiCGSTAB_MG, src/ShiftedLaplacianMultigridSolver.jl:91-93).
// Returns the iterations of the slowest column.
int bicgstab(hz_handle* h, int adj, int nrhs) {
  Hierarchy& H = h->hier[adj];
  const long long N = h->g0.N;
  const int HS = h->mcap + 2;
  const bool mixed = h->opt.precision == HZ_PREC_MIXED;
  const size_t zb = mixed ? 8 : 16;
  double2* B = h->Bd.as<double2>();
  double2* X = h->Xd.as<double2>();
  const long long bs = (long long)h->rcap * N;  // one block of rcap columns
  double2* V = h->V.as<double2>();
  double2 *r = V, *rh = V + bs, *p = V + 2 * bs, *v = V + 3 * bs, *sv = V + 4 * bs, *t = V + 5 * bs;
  char* ph = (char*)h->Z.p;
  char* sh = (char*)h->Z.p + (size_t)bs * zb;
  double2* part = h->part.as<double2>();
  double2* red = h->hA.as<double2>();
  double2* sc = h->bsc.as<double2>();
  int* dc = h->cols.as<int>();
  std::vector<int> all(nrhs);
  for (int c = 0; c < nrhs; ++c) all[c] = c;
  upload_cols(h, all);
  std::vector<double> bn(nrhs, 0.0), rn(nrhs, 0.0);
  col_norms(h, B, all, h->bnorm.as<double>(), h->bnorm_inv.as<double>(), bn.data());
  launch_zero_cols<double>(h->ctx, N, X, N, dc, nrhs);
  h->col_relres.assign(nrhs, 0.0);
  h->col_iters.assign(nrhs, 0);
  std::vector<int> act;
  for (int c = 0; c < nrhs; ++c) {
    if (!std::isfinite(bn[c])) fail(HZ_ERR_NUMERIC, "right-hand side column %d holds NaN or Inf", c);
    if (bn[c] > 0) act.push_back(c);
  }
  if (act.empty()) return 0;
  if (mixed)
    ensure_level_buffers<float>(h, H, h->rcap);
  else
    ensure_level_buffers<double>(h, H, h->rcap);
  const double tol = h->opt.rel_tol;
  // emulated-FP64 arithmetic for H z (rounded to FP64: the BiCGSTAB vectors stay FP64)
  const bool emu = mixed && h->opt.outer_arith == HZ_OUTER_EMULATED;
  FineOp fopa = h->fop;
  fopa.adj = adj;
  upload_cols(h, act);
  int na = (int)act.size();
  launch_cast_cols<double, double>(h->ctx, N, B, N, r, N, dc, na);   // r = b (x0 = 0)
  launch_cast_cols<double, double>(h->ctx, N, B, N, rh, N, dc, na);  // shadow residual
  launch_zero_cols<double>(h->ctx, N, p, N, dc, na);
  launch_zero_cols<double>(h->ctx, N, v, N, dc, na);
  launch_bicg_scalars(h->ctx, -1, dc, na, red, HS, sc);
  const int maxit = std::max(1, h->opt.max_outer);
  int it = 0;
  for (; it <= maxit; ++it) {
    na = (int)act.size();
    int nblk = krylov_nblk(N, na);
    // <rh, r> and ||r||^2 in one pass
    launch_dots(h->ctx, N, rh, 0, N, 0, 1, r, N, dc, na, nblk, 1, part);
    launch_reduce(h->ctx, part, dc, na, 2, nblk, red, HS, 0);
    launch_norms(h->ctx, red, HS, 1, dc, na, h->beta.as<double>(), nullptr);
    ck(cudaMemcpyAsync(h->h_nrm, h->beta.p, (size_t)h->rcap * 8, cudaMemcpyDeviceToHost, h->ctx.stream), "norms");
    sync(h);
    std::vector<int> still;
    for (int c : act) {
      const double e = h->h_nrm[c];
      if (!std::isfinite(e)) fail(HZ_ERR_NUMERIC, "BiCGSTAB breakdown (NaN/Inf) in column %d", c);
      if (!(e / bn[c] <= tol)) still.push_back(c);
    }
    if (still.size() != act.size()) {
      act.swap(still);
      if (act.empty()) break;
      upload_cols(h, act);
      na = (int)act.size();
      nblk = krylov_nblk(N, na);
    }
    if (it == maxit) break;
    launch_bicg_scalars(h->ctx, 0, dc, na, red, HS, sc);
    launch_bicg_vec(h->ctx, 0, N, r, p, v, nullptr, sc, dc, na);
    precondition(h, H, p, ph, dc, na);
    if (emu)
      launch_fine_df64<double2>(h->ctx, fopa, h->diagHdf.as<float4>(), (const float2*)ph, v, N, dc, na);
    else if (mixed)
      apply_H<float>(h, adj, MODE_APPLY, (const float2*)ph, nullptr, v, dc, na);
    else
      apply_H<double>(h, adj, MODE_APPLY, (const double2*)ph, nullptr, v, dc, na);
    launch_dots(h->ctx, N, rh, 0, N, 0, 1, v, N, dc, na, nblk, 0, part);
    launch_reduce(h->ctx, part, dc, na, 1, nblk, red, HS, 0);
    launch_bicg_scalars(h->ctx, 1, dc, na, red, HS, sc);
    launch_bicg_vec(h->ctx, 1, N, r, nullptr, v, sv, sc, dc, na);
    precondition(h, H, sv, sh, dc, na);
    if (emu)
      launch_fine_df64<double2>(h->ctx, fopa, h->diagHdf.as<float4>(), (const float2*)sh, t, N, dc, na);
    else if (mixed)
      apply_H<float>(h, adj, MODE_APPLY, (const float2*)sh, nullptr, t, dc, na);
    else
      apply_H<double>(h, adj, MODE_APPLY, (const double2*)sh, nullptr, t, dc, na);
    launch_dots(h->ctx, N, sv, 0, N, 0, 1, t, N, dc, na, nblk, 1, part);
    launch_reduce(h->ctx, part, dc, na, 2, nblk, red, HS, 0);
    launch_bicg_scalars(h->ctx, 2, dc, na, red, HS, sc);
    if (mixed)
      launch_bicg_xr<float>(h->ctx, N, X, (const float2*)ph, (const float2*)sh, sv, t, r, sc, dc, na);
    else
      launch_bicg_xr<double>(h->ctx, N, X, (const double2*)ph, (const double2*)sh, sv, t, r, sc, dc, na);
    for (int c : act) {
      h->col_iters[c] += 1;
      h->nprec += 2;
    }
  }
  // true residuals of every nonzero column
  std::vector<int> nz;
  for (int c = 0; c < nrhs; ++c)
    if (bn[c] > 0) nz.push_back(c);
  upload_cols(h, nz);
  apply_H<double>(h, adj, MODE_RESID, X, B, r, dc, (int)nz.size());
  col_norms(h, r, nz, h->beta.as<double>(), nullptr, rn.data());
  int worst = 0;
  for (int c : nz) {
    h->col_relres[c] = rn[c] / bn[c];
    worst = std::max(worst, h->col_iters[c]);
  }
  return worst;
}

void init_fine(hz_handle* h) {
  const hz_problem& p = h->prob;
  const long long N = num_nodes(p);
  h->g0 = make_grid(p);
  h->fop = make_fineop(p, 0);
  // operator setup on the device: upload m and gamma, compute the diagonals there
  h->diagH.alloc((size_t)N * 16);
  h->diagSH.alloc((size_t)N * 16);
  h->dinvSH.alloc((size_t)N * 16);
  {
    DBuf dm, dg;
    dm.alloc((size_t)N * 8);
    dg.alloc((size_t)N * 8);
    ck(cudaMemcpyAsync(dm.p, p.m, N * 8, cudaMemcpyHostToDevice, h->ctx.stream), "upload m");
    ck(cudaMemcpyAsync(dg.p, p.gamma, N * 8, cudaMemcpyHostToDevice, h->ctx.stream), "upload gamma");
    launch_fine_setup(h->ctx, h->g0, p.dim, p.h, p.omega_re, p.omega_im, h->opt.shift,
                      p.order_neumann_bc == 1 ? 1.0 : 2.0, p.neumann_on_top, p.sommerfeld, dm.as<double>(),
                      dg.as<double>(), h->diagH.as<double2>(), h->diagSH.as<double2>(), h->dinvSH.as<double2>());
    sync(h);
  }
  if (h->opt.precision == HZ_PREC_MIXED && h->opt.outer_arith == HZ_OUTER_EMULATED) {
    h->diagHdf.alloc((size_t)N * 16);
    launch_diag_to_df(h->ctx, N, h->diagH.as<double2>(), h->diagHdf.as<float4>());
  }
  if (h->opt.precision == HZ_PREC_MIXED) {
    h->diagSH32.alloc((size_t)N * 8);
    h->dinvSH32.alloc((size_t)N * 8);
    launch_cast<float, double>(h->ctx, h->diagSH.as<double2>(), h->diagSH32.as<float2>(), N);
    launch_cast<float, double>(h->ctx, h->dinvSH.as<double2>(), h->dinvSH32.as<float2>(), N);
    sync(h);
  }
}

void validate(const hz_problem* p, const hz_options* o) {
  if (!p || !o) fail(HZ_ERR_ARG, "null problem or options");
  if (p->dim != 2 && p->dim != 3) fail(HZ_ERR_ARG, "dim must be 2 or 3 (got %d)", p->dim);
  for (int d = 0; d < p->dim; ++d) {
    if (p->n[d] < 1) fail(HZ_ERR_ARG, "n[%d] must be >= 1", d);
    if (!(p->h[d] > 0)) fail(HZ_ERR_ARG, "h[%d] must be > 0", d);
  }
  if (!p->m || !p->gamma) fail(HZ_ERR_ARG, "m and gamma must be given");
  if (!(p->omega_re != 0.0)) fail(HZ_ERR_ARG, "omega must have a nonzero real part");
  if (o->levels < 1 || o->levels > 16) fail(HZ_ERR_ARG, "levels must be in [1, 16]");
  // the restart length only matters for FGMRES (the reference passes 0 with BiCGSTAB)
  if (o->krylov == HZ_KRYLOV_FGMRES && (o->inner < 1 || o->inner > 64))
    fail(HZ_ERR_ARG, "inner (restart length) must be in [1, 64]");
  if (o->inner < 0 || o->inner > 64) fail(HZ_ERR_ARG, "inner must be in [0, 64]");
  if (o->krylov != HZ_KRYLOV_FGMRES && o->krylov != HZ_KRYLOV_BICGSTAB) fail(HZ_ERR_ARG, "unknown Krylov method");
  if (o->cycle != 'V' && o->cycle != 'W' && o->cycle != 'K') fail(HZ_ERR_ARG, "cycle must be 'V', 'W' or 'K'");
  if (o->cycle == 'K' && o->krylov != HZ_KRYLOV_FGMRES)
    fail(HZ_ERR_ARG, "the K-cycle is a nonlinear preconditioner: it needs FGMRES");
  if (o->coarse_op != HZ_COARSE_GALERKIN && o->coarse_op != HZ_COARSE_REDISCRETIZE)
    fail(HZ_ERR_ARG, "coarse_op must be HZ_COARSE_GALERKIN or HZ_COARSE_REDISCRETIZE");
  if (o->precision != HZ_PREC_FP64 && o->precision != HZ_PREC_MIXED) fail(HZ_ERR_ARG, "unknown precision");
  if (o->precision == HZ_PREC_MIXED && o->levels < 2) fail(HZ_ERR_ARG, "mixed precision needs at least 2 levels");
  if (o->outer_arith != HZ_OUTER_FP64 && o->outer_arith != HZ_OUTER_EMULATED) fail(HZ_ERR_ARG, "unknown outer_arith");
  if (o->outer_arith == HZ_OUTER_EMULATED && o->precision != HZ_PREC_MIXED)
    fail(HZ_ERR_ARG, "emulated-FP64 outer arithmetic is part of the mixed form (precision = HZ_PREC_MIXED)");
  if (!(o->rel_tol > 0)) fail(HZ_ERR_ARG, "rel_tol must be > 0");
  if (o->relax_type != HZ_RELAX_JAC && o->relax_type != HZ_RELAX_JAC_GMRES)
    fail(HZ_ERR_ARG, "relax_type must be HZ_RELAX_JAC or HZ_RELAX_JAC_GMRES");
  if (o->relax_type == HZ_RELAX_JAC_GMRES) {
    if (o->krylov != HZ_KRYLOV_FGMRES)
      fail(HZ_ERR_ARG, "the Jac-GMRES smoother makes the cycle nonlinear: it needs FGMRES");
    if (o->relax_pre < 0 || o->relax_pre > 2 || o->relax_post < 0 || o->relax_post > 2)
      fail(HZ_ERR_ARG, "Jac-GMRES takes 0, 1 or 2 GMRES steps per smoothing (relax_pre, relax_post)");
    if (o->relax_from < 0 || o->relax_from >= o->levels) fail(HZ_ERR_ARG, "relax_from must be in [0, levels - 1]");
  }
}

void copy_in(hz_handle* h, const double* src, double2* dst, long long N, int nrhs, int mem) {
  const size_t bytes = (size_t)N * nrhs * 16;
  if (mem == HZ_MEM_HOST) {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->ctx.stream), "copy B to device");
    h->h2d += (long long)bytes;
  } else {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, h->ctx.stream), "copy B on device");
  }
}

void copy_out(hz_handle* h, const double2* src, double* dst, long long N, int nrhs, int mem) {
  const size_t bytes = (size_t)N * nrhs * 16;
  if (mem == HZ_MEM_HOST) {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->ctx.stream), "copy X to host");
    h->d2h += (long long)bytes;
  } else {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, h->ctx.stream), "copy X on device");
  }
}

template <typename F>
int guarded(hz_handle* h, F&& f) {
  try {
    f();
    return HZ_OK;
  } catch (const HzError& e) {
    if (h) h->err = e.msg;
    g_thread_error = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    if (h) h->err = e.what();
    g_thread_error = e.what();
    return HZ_ERR_CUDA;
  }
}

}  // namespace

// A trained or training coarse-correction network on one device.
struct hz_net {
  int dev = 0;
  std::unique_ptr<hz::CoarseNet> net;    // the 2D network, or
  std::unique_ptr<hz::CoarseNet3> net3;  // the 3D network
  cudaEvent_t order_ev = nullptr;  // orders the network's stream after the legacy default stream
  int dim() const { return net3 ? 3 : 2; }
  hz::Ctx& ctx() { return net3 ? net3->ctx : net->ctx; }
  ~hz_net() {
    if (order_ev) cudaEventDestroy(order_ev);
  }
};

namespace {
// As order_after_default_stream, for the network's own stream.
void net_order_after_default_stream(hz_net* net) {
  ck(cudaEventRecord(net->order_ev, cudaStreamLegacy), "record ordering event");
  ck(cudaStreamWaitEvent(net->ctx().stream, net->order_ev, 0), "order after the default stream");
}
}  // namespace

namespace {

Grid level_grid(const hz_handle* h, int level) {
  Grid g = h->g0;
  for (int k = 0; k < level; ++k) g = coarsen(g, h->prob.dim);
  return g;
}

void check_net_grid(long long nx, long long ny, int batch) {
  if (!hz::CoarseNet::supports(nx, ny))
    fail(HZ_ERR_ARG, "network grid %lldx%lld: node counts must be 8k+1 (k >= 1)", nx, ny);
  if (batch < 1) fail(HZ_ERR_ARG, "batch must be >= 1");
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int32_t hz_version(void) { return HZ_ABI_VERSION; }

const char* hz_last_error(const hz_handle* h) { return h ? h->err.c_str() : g_thread_error.c_str(); }

void hz_default_options(hz_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->levels = 3;
  o->max_outer = 50;
  o->rel_tol = 1e-8;
  o->relax_pre = 1;
  o->relax_post = 1;
  o->relax_param = 0.8;
  o->cycle = 'V';
  o->krylov = HZ_KRYLOV_FGMRES;
  o->inner = 10;
  o->shift = 0.5;
  o->precision = HZ_PREC_FP64;
  o->coarse_op = HZ_COARSE_GALERKIN;
  o->cuda_graph = 1;
  o->autotune = 1;
}

int hz_create(const hz_problem* prob, const hz_options* opt, hz_handle** out) {
  if (!out) return HZ_ERR_ARG;
  *out = nullptr;
  auto h = std::make_unique<hz_handle>();
  int st = guarded(nullptr, [&] {
    validate(prob, opt);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(HZ_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (opt->device < 0 || opt->device >= ndev) fail(HZ_ERR_ARG, "device %d out of range", opt->device);
    h->prob = *prob;
    h->opt = *opt;
    if (h->prob.order_neumann_bc != 1) h->prob.order_neumann_bc = 2;
    const long long N = num_nodes(*prob);
    h->m.assign(prob->m, prob->m + N);
    h->gamma.assign(prob->gamma, prob->gamma + N);
    h->prob.m = h->m.data();
    h->prob.gamma = h->gamma.data();
    h->dev = opt->device;
    set_device(h.get());
    ck(cudaStreamCreateWithFlags(&h->ctx.stream, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreateWithFlags(&h->order_ev, cudaEventDisableTiming), "ordering event");
    h->ctx.profile = opt->profile != 0;
    {
      const char* rt = std::getenv("HELMGPU_RAP_TILED");
      h->ctx.rap_tiled = rt && std::strcmp(rt, "1") == 0;
    }
    auto t0 = clk::now();
    init_fine(h.get());
    h->setup_time += secs(t0, clk::now());
  });
  if (st != HZ_OK) {
    if (h->order_ev) cudaEventDestroy(h->order_ev);
    if (h->ctx.stream) cudaStreamDestroy(h->ctx.stream);
    return st;
  }
  *out = h.release();
  return HZ_OK;
}

int hz_destroy(hz_handle* h) {
  if (!h) return HZ_OK;
  cudaSetDevice(h->dev);
  if (h->ctx.stream) cudaStreamSynchronize(h->ctx.stream);
  drop_graphs(h);
  h->ctx.release();
  if (h->h_est) cudaFreeHost(h->h_est);
  if (h->h_nrm) cudaFreeHost(h->h_nrm);
  if (h->h_flag) cudaFreeHost(h->h_flag);
  if (h->order_ev) cudaEventDestroy(h->order_ev);
  if (h->ctx.stream) cudaStreamDestroy(h->ctx.stream);
  delete h;
  return HZ_OK;
}

int hz_solve(hz_handle* h, const double* B, double* X, int64_t n, int32_t nrhs, int32_t transpose, int32_t mem,
             hz_stats* stats) {
  if (!h) return HZ_ERR_ARG;
  int conv_status = HZ_OK;
  int st = guarded(h, [&] {
    if (!B || !X) fail(HZ_ERR_ARG, "null B or X");
    if (n != h->g0.N) fail(HZ_ERR_ARG, "B has %lld rows, the grid has %lld nodes", (long long)n, h->g0.N);
    if (nrhs < 1) fail(HZ_ERR_ARG, "nrhs must be >= 1");
    if (transpose != 0 && transpose != 1) fail(HZ_ERR_ARG, "transpose must be 0 or 1");
    if (mem != HZ_MEM_HOST && mem != HZ_MEM_DEVICE) fail(HZ_ERR_ARG, "mem must be HZ_MEM_HOST or HZ_MEM_DEVICE");
    if (h->prob.omega_im != 0.0) fail(HZ_ERR_ARG, "the solver needs a real omega (GetHelmholtzShiftOP takes Float64)");
    set_device(h);
    const long long l0 = h->ctx.launches;
    h->h2d = h->d2h = 0;
    if (mem == HZ_MEM_DEVICE) order_after_default_stream(h);
    auto t0 = clk::now();
    if (!h->hier[transpose].built) build_hierarchy(h, transpose);
    ensure_workspace(h, nrhs);
    if (h->opt.autotune && h->tuned_cols != nrhs) {
      if (h->opt.precision == HZ_PREC_MIXED)
        autotune<float>(h, h->hier[transpose], nrhs);
      else
        autotune<double>(h, h->hier[transpose], nrhs);
      h->tuned_cols = nrhs;
    }
    auto t1 = clk::now();
    h->setup_time += secs(t0, t1);
    copy_in(h, B, h->Bd.as<double2>(), n, nrhs, mem);
    const long long np0 = h->nprec;
    int outer = (h->opt.krylov == HZ_KRYLOV_BICGSTAB) ? bicgstab(h, transpose, nrhs) : fgmres(h, transpose, nrhs);
    copy_out(h, h->Xd.as<double2>(), X, n, nrhs, mem);
    sync(h);
    // a tensor-core convolution of the attached network that gave up waiting makes the solve invalid
    if ((h->net && h->net->conv_path() != HZ_NET_CONV_WARP_MMA && h->net->tc_failed()) ||
        (h->net3 && h->net3->conv_path() != HZ_NET_CONV_WARP_MMA && h->net3->tc_failed()))
      fail(HZ_ERR_CUDA, "tensor-core convolution of the network timed out");
    auto t2 = clk::now();
    h->solve_time += secs(t1, t2);
    int nconv = 0, maxit = 0;
    double maxrr = 0.0;
    for (int c = 0; c < nrhs; ++c) {
      if (h->col_relres[c] <= h->opt.rel_tol) ++nconv;
      maxrr = std::max(maxrr, h->col_relres[c]);
      maxit = std::max(maxit, h->col_iters[c]);
    }
    if (nconv < nrhs) conv_status = HZ_NOT_CONVERGED;
    if (stats) {
      stats->outer = outer;
      stats->n_prec = (int32_t)(h->nprec - np0);
      stats->max_col_iters = maxit;
      stats->converged_cols = nconv;
      stats->max_relres = maxrr;
      stats->setup_time = h->setup_time;
      stats->solve_time = h->solve_time;
      stats->kernel_launches = h->ctx.launches - l0;
      stats->h2d_bytes = h->h2d;
      stats->d2h_bytes = h->d2h;
    }
    if (h->opt.verbose)
      fprintf(stderr, "helmgpu: %d columns, %d outer cycles, max rel. residual %.3e, solve %.3f s\n", nrhs, outer,
              maxrr, secs(t1, t2));
  });
  if (st != HZ_OK) return st;
  if (conv_status != HZ_OK) h->err = "not converged within max_outer restart cycles";
  return conv_status;
}

int hz_column_stats(const hz_handle* h, double* relres, int32_t* iters, int32_t nrhs) {
  if (!h) return HZ_ERR_ARG;
  if (nrhs > (int)h->col_relres.size()) return HZ_ERR_ARG;
  for (int c = 0; c < nrhs; ++c) {
    if (relres) relres[c] = h->col_relres[c];
    if (iters) iters[c] = h->col_iters[c];
  }
  return HZ_OK;
}

int hz_apply(hz_handle* h, int32_t op, int32_t transpose, const double* X, double* Y, int64_t n, int32_t nrhs,
             int32_t mem) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] {
    if (!X || !Y) fail(HZ_ERR_ARG, "null X or Y");
    if (n != h->g0.N) fail(HZ_ERR_ARG, "X has %lld rows, the grid has %lld nodes", (long long)n, h->g0.N);
    if (nrhs < 1) fail(HZ_ERR_ARG, "nrhs must be >= 1");
    if (op != HZ_OP_H && op != HZ_OP_SH) fail(HZ_ERR_ARG, "op must be HZ_OP_H or HZ_OP_SH");
    if (mem != HZ_MEM_HOST && mem != HZ_MEM_DEVICE) fail(HZ_ERR_ARG, "bad mem");
    if (transpose != 0 && transpose != 1) fail(HZ_ERR_ARG, "transpose must be 0 or 1");
    if (mem == HZ_MEM_DEVICE) check_no_overlap(X, Y, n, nrhs);
    set_device(h);
    h->h2d = h->d2h = 0;
    if (mem == HZ_MEM_DEVICE) order_after_default_stream(h);
    const double2* xd;
    double2* yd;
    const size_t bytes = (size_t)n * nrhs * 16;
    if (mem == HZ_MEM_HOST) {
      h->tmpA.alloc(bytes);
      h->tmpB.alloc(bytes);
      copy_in(h, X, h->tmpA.as<double2>(), n, nrhs, HZ_MEM_HOST);
      xd = h->tmpA.as<double2>();
      yd = h->tmpB.as<double2>();
    } else {
      xd = reinterpret_cast<const double2*>(X);
      yd = reinterpret_cast<double2*>(Y);
    }
    if (nrhs > h->apply_ncols) {
      // the list 0..nrhs-1 only grows: later calls with as many columns or fewer
      // reuse it and leave the allocation generation (and the solver's graphs) alone
      std::vector<int> all(nrhs);
      for (int c = 0; c < nrhs; ++c) all[c] = c;
      h->apply_cols.alloc(all.size() * sizeof(int));
      ck(cudaMemcpyAsync(h->apply_cols.p, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice,
                         h->ctx.stream),
         "cols");
      h->apply_ncols = nrhs;
    }
    FineOp fop = h->fop;
    fop.adj = transpose ? 1 : 0;
    const double2* diag = (op == HZ_OP_H) ? h->diagH.as<double2>() : h->diagSH.as<double2>();
    launch_fine<double, double, double>(h->ctx, MODE_APPLY, fop, diag, nullptr, xd, (const double2*)nullptr, yd, n,
                                        h->apply_cols.as<int>(), nrhs, 0.0);
    if (mem == HZ_MEM_HOST) copy_out(h, yd, Y, n, nrhs, HZ_MEM_HOST);
    sync(h);
  });
}

int hz_apply_noalloc(hz_handle* h, int32_t op, int32_t transpose, const double* X, double* Y, int64_t n,
                     int32_t nrhs) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] {
    if (!X || !Y) fail(HZ_ERR_ARG, "null X or Y");
    if (n != h->g0.N) fail(HZ_ERR_ARG, "X has %lld rows, the grid has %lld nodes", (long long)n, h->g0.N);
    if (nrhs < 1 || nrhs > HZ_NOALLOC_MAX_COLS)
      fail(HZ_ERR_ARG, "hz_apply_noalloc takes 1 to %d columns (got %d)", HZ_NOALLOC_MAX_COLS, (int)nrhs);
    if (op != HZ_OP_H && op != HZ_OP_SH) fail(HZ_ERR_ARG, "op must be HZ_OP_H or HZ_OP_SH");
    if (transpose != 0 && transpose != 1) fail(HZ_ERR_ARG, "transpose must be 0 or 1");
    check_no_overlap(X, Y, n, nrhs);
    set_device(h);
    order_after_default_stream(h);
    FineOp fop = h->fop;
    fop.adj = transpose;
    const double2* diag = (op == HZ_OP_H) ? h->diagH.as<double2>() : h->diagSH.as<double2>();
    std::string err;
    const int rc = launch_fine_apply_noalloc(h->ctx.stream, h->dev, fop, diag, reinterpret_cast<const double2*>(X),
                                             reinterpret_cast<double2*>(Y), n, nrhs, &err);
    if (rc == -1) fail(HZ_ERR_ARG, "%s", err.c_str());
    if (rc != 0) fail(HZ_ERR_CUDA, "%s", err.c_str());
    ck(cudaStreamSynchronize(h->ctx.stream), "stream sync");
  });
}

int hz_clear(hz_handle* h) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] {
    set_device(h);
    sync(h);
    drop_graphs(h);
    for (auto& H : h->hier) {
      H.lv.clear();
      H.bandT.reset();
      H.bandG.reset();
      H.bandB.reset();
      H.dense.reset();
      H.dense_df = false;
      H.band_df = false;
      H.bandwork.reset();
      H.band = BandSolveOps();
      H.built = false;
    }
  });
}

int hz_copy(const hz_handle* h, hz_handle** out) {
  if (!h || !out) return HZ_ERR_ARG;
  hz_problem p = h->prob;
  return hz_create(&p, &h->opt, out);
}

void* hz_stream(hz_handle* h) { return h ? (void*)h->ctx.stream : nullptr; }

// make the table's device current and fold its finished launches' events in;
// a device error (a failed launch before) is reported, not swallowed
static void ctx_settle(Ctx& c, int dev) {
  ck(cudaSetDevice(dev), "cudaSetDevice");
  if (c.stream) ck(cudaStreamSynchronize(c.stream), "synchronize the launch table's stream");
  c.resolve();
}

static int ctx_times(Ctx& c, int dev, int32_t idx, char* name, int32_t name_len, int64_t* launches,
                     int64_t* timed_launches, double* total_ms, double* alg_bytes, double* alg_flops) {
  ctx_settle(c, dev);
  const int n = (int)c.names.size();
  if (idx < 0 || idx >= n) return n;
  if (name && name_len > 0) {
    std::strncpy(name, c.names[idx].c_str(), (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  if (launches) *launches = c.counts[idx];
  if (timed_launches) *timed_launches = c.timed[idx];
  if (total_ms) *total_ms = c.total_ms[idx];
  if (alg_bytes) *alg_bytes = c.alg_bytes[idx];
  if (alg_flops) *alg_flops = c.alg_flops[idx];
  return n;
}

static void ctx_reset(Ctx& c, int dev) {
  ctx_settle(c, dev);
  std::fill(c.counts.begin(), c.counts.end(), 0);
  std::fill(c.timed.begin(), c.timed.end(), 0);
  std::fill(c.total_ms.begin(), c.total_ms.end(), 0.0);
  std::fill(c.alg_bytes.begin(), c.alg_bytes.end(), 0.0);
  std::fill(c.alg_flops.begin(), c.alg_flops.end(), 0.0);
}

int hz_kernel_times(hz_handle* h, int32_t idx, char* name, int32_t name_len, int64_t* launches,
                    int64_t* timed_launches, double* total_ms, double* alg_bytes) {
  if (!h) return HZ_ERR_ARG;
  int n = 0;
  const int st = guarded(h, [&] {
    n = ctx_times(h->ctx, h->dev, idx, name, name_len, launches, timed_launches, total_ms, alg_bytes, nullptr);
  });
  return st < 0 ? st : n;
}

int hz_kernel_flops(hz_handle* h, int32_t idx, double* alg_flops) {
  if (!h) return HZ_ERR_ARG;
  int n = 0;
  const int st = guarded(h, [&] {
    n = ctx_times(h->ctx, h->dev, idx, nullptr, 0, nullptr, nullptr, nullptr, nullptr, alg_flops);
  });
  return st < 0 ? st : n;
}

int hz_tune_info(const hz_handle* h, int32_t* fine_ctas, int32_t* rap_ctas) {
  if (!h) return HZ_ERR_ARG;
  if (fine_ctas) *fine_ctas = h->ctx.tune_fine;
  if (rap_ctas) *rap_ctas = h->ctx.tune_rap;
  return h->tuned_cols >= 0 ? HZ_OK : HZ_NOT_CONVERGED;
}

int hz_reset_kernel_times(hz_handle* h) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] { ctx_reset(h->ctx, h->dev); });
}

int hz_set_cuda_graph(hz_handle* h, int32_t on) {
  if (!h) return HZ_ERR_ARG;
  h->opt.cuda_graph = on != 0;
  return HZ_OK;
}

int hz_set_profile(hz_handle* h, int32_t on) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] {
    ctx_settle(h->ctx, h->dev);
    h->ctx.profile = on != 0;
  });
}

// ---- learned coarse-grid correction -------------------------------------------

namespace {
// A network on a device: the 2D encoder-decoder (dim 2) or the 3D one (dim 3).
int net_create(int32_t seed, int32_t device, int dim, hz_net** out) {
  if (!out) return HZ_ERR_ARG;
  *out = nullptr;
  auto n = std::make_unique<hz_net>();
  int st = guarded(nullptr, [&] {
    int cnt = 0;
    if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt == 0) {
      cudaGetLastError();
      fail(HZ_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= cnt) fail(HZ_ERR_ARG, "device %d out of range", device);
    ck(cudaSetDevice(device), "cudaSetDevice");
    n->dev = device;
    if (dim == 3)
      n->net3 = std::make_unique<hz::CoarseNet3>((unsigned)seed);
    else
      n->net = std::make_unique<hz::CoarseNet>((unsigned)seed);
    ck(cudaEventCreateWithFlags(&n->order_ev, cudaEventDisableTiming), "ordering event");
  });
  if (st == HZ_OK) *out = n.release();
  return st;
}

void check_net3_grid(long long nx, long long ny, long long nz, int batch) {
  if (!hz::CoarseNet3::supports(nx, ny, nz))
    fail(HZ_ERR_ARG, "network grid %lldx%lldx%lld: node counts must be 4k+1 (k >= 1)", nx, ny, nz);
  if (batch < 1) fail(HZ_ERR_ARG, "batch must be >= 1");
}

void need_dim(const hz_net* net, int dim, const char* what) {
  if (net->dim() != dim) fail(HZ_ERR_ARG, "%s takes a %dD network (this one is %dD)", what, dim, net->dim());
}
}  // namespace

int hz_net_create(int32_t seed, int32_t device, hz_net** out) { return net_create(seed, device, 2, out); }

int hz_net3d_create(int32_t seed, int32_t device, hz_net** out) { return net_create(seed, device, 3, out); }

int hz_net_dim(const hz_net* net) { return net ? net->dim() : HZ_ERR_ARG; }

int hz_net_destroy(hz_net* net) {
  if (!net) return HZ_OK;
  cudaSetDevice(net->dev);
  delete net;
  return HZ_OK;
}

int64_t hz_net_num_params(void) { return hz::CoarseNet::num_params(); }

int64_t hz_net3d_num_params(void) { return hz::CoarseNet3::num_params(); }

int hz_net_layer_shape(int32_t layer, int32_t* cin, int32_t* cout) {
  if (layer < 0 || layer >= hz::CoarseNet::kLayers || !cin || !cout) return HZ_ERR_ARG;
  int a = 0, b = 0;
  hz::CoarseNet::layer_shape(layer, &a, &b);
  *cin = a;
  *cout = b;
  return HZ_OK;
}

int hz_net3d_layer_shape(int32_t layer, int32_t* cin, int32_t* cout) {
  if (layer < 0 || layer >= hz::CoarseNet3::kLayers || !cin || !cout) return HZ_ERR_ARG;
  int a = 0, b = 0;
  hz::CoarseNet3::layer_shape(layer, &a, &b);
  *cin = a;
  *cout = b;
  return HZ_OK;
}

int hz_net_get_weights(hz_net* net, float* w) {
  if (!net || !w) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    if (net->net3)
      net->net3->get_weights(w);
    else
      net->net->get_weights(w);
  });
}

int hz_net_set_weights(hz_net* net, const float* w) {
  if (!net || !w) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    if (net->net3)
      net->net3->set_weights(w);
    else
      net->net->set_weights(w);
  });
}

namespace {
// y = net(x) for a batch on a grid of nz = 1 (2D) or nz > 1 (3D) planes
void net_forward(hz_net* net, const float* x, float* y, int64_t nx, int64_t ny, int64_t nz, int32_t batch,
                 int32_t mem) {
  if (mem != HZ_MEM_HOST && mem != HZ_MEM_DEVICE) fail(HZ_ERR_ARG, "mem must be HZ_MEM_HOST or HZ_MEM_DEVICE");
  ck(cudaSetDevice(net->dev), "cudaSetDevice");
  hz::Ctx& cx = net->ctx();
  const long long N = nx * ny * nz;
  const float* dx = x;
  if (mem == HZ_MEM_DEVICE) net_order_after_default_stream(net);
  if (mem == HZ_MEM_HOST) {
    float* st = net->net3 ? net->net3->input_staging((int)nx, (int)ny, (int)nz, batch)
                          : net->net->input_staging((int)nx, (int)ny, batch);
    ck(cudaMemcpyAsync(st, x, (size_t)batch * N * 16, cudaMemcpyHostToDevice, cx.stream), "copy x");
    dx = st;
  }
  const float* out;
  if (net->net3) {
    net->net3->forward(cx, dx, (int)nx, (int)ny, (int)nz, batch);
    out = net->net3->output();
  } else {
    net->net->forward(cx, dx, (int)nx, (int)ny, batch);
    out = net->net->output();
  }
  ck(cudaMemcpy2DAsync(y, 8, out, 32, 8, (size_t)batch * N,
                       mem == HZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, cx.stream),
     "copy y");
  ck(cudaStreamSynchronize(cx.stream), "sync");
  cx.resolve();
  if ((net->net && net->net->conv_path() != HZ_NET_CONV_WARP_MMA && net->net->tc_failed()) ||
      (net->net3 && net->net3->conv_path() != HZ_NET_CONV_WARP_MMA && net->net3->tc_failed()))
    fail(HZ_ERR_CUDA, "tensor-core convolution timed out");
}

void net_gradient(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t nz, int32_t batch,
                  int32_t mem, double* loss, float* grad) {
  if (mem != HZ_MEM_HOST && mem != HZ_MEM_DEVICE) fail(HZ_ERR_ARG, "mem must be HZ_MEM_HOST or HZ_MEM_DEVICE");
  ck(cudaSetDevice(net->dev), "cudaSetDevice");
  hz::Ctx& cx = net->ctx();
  const long long N = nx * ny * nz;
  DBuf bx, bt;
  const float* dx = x;
  const float* dt = t;
  if (mem == HZ_MEM_DEVICE) net_order_after_default_stream(net);
  if (mem == HZ_MEM_HOST) {
    bx.alloc((size_t)batch * N * 16);
    bt.alloc((size_t)batch * N * 8);
    ck(cudaMemcpyAsync(bx.p, x, (size_t)batch * N * 16, cudaMemcpyHostToDevice, cx.stream), "copy x");
    ck(cudaMemcpyAsync(bt.p, t, (size_t)batch * N * 8, cudaMemcpyHostToDevice, cx.stream), "copy t");
    dx = bx.as<float>();
    dt = bt.as<float>();
  }
  double l;
  if (net->net3) {
    net->net3->forward(cx, dx, (int)nx, (int)ny, (int)nz, batch, true);
    l = net->net3->backward(cx, dt, (int)nx, (int)ny, (int)nz, batch);
    if (grad) net->net3->get_grad(grad);
  } else {
    net->net->forward(cx, dx, (int)nx, (int)ny, batch, true);
    l = net->net->backward(cx, dt, (int)nx, (int)ny, batch);
    if (grad) net->net->get_grad(grad);
  }
  if (loss) *loss = l;
}
}  // namespace

int hz_net_forward(hz_net* net, const float* x, float* y, int64_t nx, int64_t ny, int32_t batch, int32_t mem) {
  if (!net || !x || !y) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    need_dim(net, 2, "hz_net_forward");
    check_net_grid(nx, ny, batch);
    net_forward(net, x, y, nx, ny, 1, batch, mem);
  });
}

int hz_net3d_forward(hz_net* net, const float* x, float* y, int64_t nx, int64_t ny, int64_t nz, int32_t batch,
                     int32_t mem) {
  if (!net || !x || !y) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    need_dim(net, 3, "hz_net3d_forward");
    check_net3_grid(nx, ny, nz, batch);
    net_forward(net, x, y, nx, ny, nz, batch, mem);
  });
}

int hz_net_gradient(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int32_t batch, int32_t mem,
                    double* loss, float* grad) {
  if (!net || !x || !t) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    need_dim(net, 2, "hz_net_gradient");
    check_net_grid(nx, ny, batch);
    net_gradient(net, x, t, nx, ny, 1, batch, mem, loss, grad);
  });
}

int hz_net3d_gradient(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t nz, int32_t batch,
                      int32_t mem, double* loss, float* grad) {
  if (!net || !x || !t) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    need_dim(net, 3, "hz_net3d_gradient");
    check_net3_grid(nx, ny, nz, batch);
    net_gradient(net, x, t, nx, ny, nz, batch, mem, loss, grad);
  });
}

int hz_net_train(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t npairs, int32_t batch,
                 int32_t epochs, double lr, int32_t seed, double* loss_hist) {
  if (!net || !x || !t) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    need_dim(net, 2, "hz_net_train");
    check_net_grid(nx, ny, batch);
    if (npairs < 1 || epochs < 1) fail(HZ_ERR_ARG, "npairs and epochs must be >= 1");
    if (!(lr > 0)) fail(HZ_ERR_ARG, "lr must be > 0");
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    hz::CoarseNet& c = *net->net;
    net_order_after_default_stream(net);
    c.train(c.ctx, x, t, (int)nx, (int)ny, npairs, batch, epochs, lr, (unsigned)seed, loss_hist);
  });
}

int hz_net3d_train(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t nz, int64_t npairs,
                   int32_t batch, int32_t epochs, double lr, int32_t seed, double* loss_hist) {
  if (!net || !x || !t) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    need_dim(net, 3, "hz_net3d_train");
    check_net3_grid(nx, ny, nz, batch);
    if (npairs < 1 || epochs < 1) fail(HZ_ERR_ARG, "npairs and epochs must be >= 1");
    if (!(lr > 0)) fail(HZ_ERR_ARG, "lr must be > 0");
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    hz::CoarseNet3& c = *net->net3;
    net_order_after_default_stream(net);
    c.train(c.ctx, x, t, (int)nx, (int)ny, (int)nz, npairs, batch, epochs, lr, (unsigned)seed, loss_hist);
  });
}

int hz_net_save(hz_net* net, const char* path) {
  if (!net || !path) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    if (net->net3)
      net->net3->save(path);
    else
      net->net->save(path);
  });
}

int hz_net_load(hz_net* net, const char* path) {
  if (!net || !path) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    long long n = 0, st = 0;
    const int rc = net->net3 ? hz::CoarseNet3::file_info(path, &n, &st) : hz::CoarseNet::file_info(path, &n, &st);
    if (rc < 0) fail(HZ_ERR_ARG, "%s: not a loadable %dD coarse-network file (code %d)", path, net->dim(), rc);
    if (net->net3)
      net->net3->load(path);
    else
      net->net->load(path);
  });
}

int hz_net_file_info(const char* path, int64_t* nparams, int64_t* adam_step) {
  if (!path) return HZ_ERR_ARG;
  long long n = 0, st = 0;
  int rc = hz::CoarseNet::file_info(path, &n, &st);
  if (rc == -2) rc = hz::CoarseNet3::file_info(path, &n, &st);  // not a 2D file: a 3D one?
  if (rc < 0) {
    g_thread_error = std::string(path) + ": not a loadable coarse-network file";
    return HZ_ERR_ARG;
  }
  if (nparams) *nparams = n;
  if (adam_step) *adam_step = st;
  return HZ_OK;
}

int hz_net_set_conv_path(hz_net* net, int32_t path) {
  if (!net) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    if (path != HZ_NET_CONV_WARP_MMA && path != HZ_NET_CONV_TCGEN05 && path != HZ_NET_CONV_AUTO)
      fail(HZ_ERR_ARG, "conv path must be HZ_NET_CONV_WARP_MMA, HZ_NET_CONV_TCGEN05 or HZ_NET_CONV_AUTO");
    ck(cudaSetDevice(net->dev), "cudaSetDevice");
    ck(cudaStreamSynchronize(net->ctx().stream), "synchronize the network's stream");
    if (net->net)
      net->net->set_conv_path(path);
    else if (net->net3)
      net->net3->set_conv_path(path);
  });
}

int hz_net_set_profile(hz_net* net, int32_t on) {
  if (!net) return HZ_ERR_ARG;
  return guarded(nullptr, [&] {
    ctx_settle(net->ctx(), net->dev);
    net->ctx().profile = on != 0;
  });
}

int hz_net_kernel_times(hz_net* net, int32_t idx, char* name, int32_t name_len, int64_t* launches,
                        int64_t* timed_launches, double* total_ms, double* alg_bytes, double* alg_flops) {
  if (!net) return HZ_ERR_ARG;
  int n = 0;
  const int st = guarded(nullptr, [&] {
    n = ctx_times(net->ctx(), net->dev, idx, name, name_len, launches, timed_launches, total_ms, alg_bytes,
                  alg_flops);
  });
  return st < 0 ? st : n;
}

int hz_net_reset_kernel_times(hz_net* net) {
  if (!net) return HZ_ERR_ARG;
  return guarded(nullptr, [&] { ctx_reset(net->ctx(), net->dev); });
}

int hz_attach_net(hz_handle* h, hz_net* net, int32_t level, double stag_ratio) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] {
    if (!net) {
      h->net = nullptr;
      h->net3 = nullptr;
      h->net_level = 0;
      return;
    }
    if (net->dim() != h->prob.dim)
      fail(HZ_ERR_ARG, "a %dD network cannot correct a %dD problem", net->dim(), h->prob.dim);
    if (h->opt.krylov != HZ_KRYLOV_FGMRES)
      fail(HZ_ERR_ARG, "the learned correction is a nonlinear preconditioner: it needs FGMRES");
    if (level < 1 || level >= h->opt.levels) fail(HZ_ERR_ARG, "level must be in [1, levels - 1]");
    if (!(stag_ratio > 0)) fail(HZ_ERR_ARG, "stag_ratio must be > 0");
    if (net->dev != h->dev) fail(HZ_ERR_ARG, "network and solver live on different devices");
    const Grid g = level_grid(h, level);
    if (h->prob.dim == 2)
      check_net_grid(g.nx, g.ny, 1);
    else
      check_net3_grid(g.nx, g.ny, g.nz, 1);
    h->net = net->net.get();
    h->net3 = net->net3.get();
    h->net_level = level;
    h->net_stag = stag_ratio;
  });
}

int hz_learned_stats(const hz_handle* h, int64_t* net_calls, int32_t* fallbacks) {
  if (!h) return HZ_ERR_ARG;
  if (net_calls) *net_calls = h->net_calls;
  if (fallbacks) *fallbacks = h->net_fallbacks;
  return HZ_OK;
}

namespace {
// 3D training targets for the right-hand sides captured on `level`: a band LU of
// a 3D coarse level is out of reach (65^3 nodes, bandwidth 4225), so the target
// e = A^{-1} r starts from one cycle on that level (what the network stands
// for: the level's cycle in V and W cycles, the preconditioner of the level's
// two FGMRES steps in the K-cycle) and takes sweeps - 1 restarted two-step
// FGMRES corrections e += K(r - A e) preconditioned by the level's cycle, in
// FP64.  Each minimises the residual over its space, so the residual never grows.
// On the coarsest level the cycle is the band LU: its solve is the target.
void collect_targets_iterative(hz_handle* h, Hierarchy& H, int level, int sweeps, long long cnt, float* x_out,
                               float* t_out, double* plain_err, double* target_relres) {
  const Grid g = level_grid(h, level);
  const long long N = g.N;
  const int R = h->rcap;
  const int last = (int)H.lv.size() - 1;
  if (level >= last) sweeps = 1;
  Level& Lv = *H.lv[level];
  if (sweeps > 1 && !Lv.kv.p) {  // the two-step corrections' vectors (allocated by the K-cycle itself otherwise)
    Lv.kv.alloc((size_t)5 * R * Lv.ld * sizeof(double2));
    Lv.ks.alloc((size_t)R * 8 * 16);
    Lv.kp.alloc((size_t)R * 3 * kcycle_nblk(Lv.g.N) * 16);
  }
  DBuf xe, res, ev, x1, idc, sc, nrm;
  xe.alloc((size_t)R * N * 16);
  res.alloc((size_t)R * N * 16);
  ev.alloc((size_t)R * N * 16);
  x1.alloc((size_t)R * N * 16);
  sc.alloc((size_t)R * 4);
  nrm.alloc((size_t)R * 6 * 8);
  idc.alloc((size_t)R * sizeof(int));
  std::vector<int> seq(R);
  for (int c = 0; c < R; ++c) seq[c] = c;
  ck(cudaMemcpy(idc.p, seq.data(), R * sizeof(int), cudaMemcpyHostToDevice), "upload cols");
  const int* dc = idc.as<int>();
  const float2* feat = net_features(h, level);
  auto plain = [&](const double2* b, double2* out, int k) { mg_cycle<double, double>(h, H, level, b, out, dc, k); };
  std::vector<double> hn((size_t)R * 6);
  double worst = 0.0;
  for (long long i0 = 0; i0 < cnt; i0 += R) {
    const int k = (int)std::min<long long>(R, cnt - i0);
    const double2* r = h->cap_buf.as<double2>() + i0 * N;
    double2* xd = xe.as<double2>();
    plain(r, x1.as<double2>(), k);  // what the network replaces
    ck(cudaMemcpyAsync(xd, x1.p, (size_t)k * N * 16, cudaMemcpyDeviceToDevice, h->ctx.stream), "first sweep");
    for (int s = 1; s < sweeps; ++s) {
      lev_op<double, double>(h, H, level, MODE_RESID, xd, r, res.as<double2>(), dc, k);
      kcycle_correction<double>(h, H, level, res.as<double2>(), ev.as<double2>(), dc, k);
      launch_axpy_compact(h->ctx, N, k, ev.as<double2>(), xd);
    }
    lev_op<double, double>(h, H, level, MODE_RESID, xd, r, res.as<double2>(), dc, k);
    launch_diff_norms(h->ctx, N, k, res.as<double2>(), r, nrm.as<double>());
    launch_diff_norms(h->ctx, N, k, x1.as<double2>(), xd, nrm.as<double>() + 3 * R);
    launch_pair_pack(h->ctx, N, r, xd, k, feat, h->net_h2, sc.as<float>(), x_out + i0 * N * 4, t_out + i0 * N * 2);
    ck(cudaMemcpyAsync(hn.data(), nrm.p, (size_t)R * 6 * 8, cudaMemcpyDeviceToHost, h->ctx.stream), "norms");
    sync(h);
    for (int c = 0; c < k; ++c) {
      const double rr = hn[3 * c + 2] > 0 ? std::sqrt(hn[3 * c + 1] / hn[3 * c + 2]) : 0.0;
      worst = std::max(worst, rr);
      const double* q = hn.data() + 3 * R + 3 * c;
      if (plain_err) plain_err[i0 + c] = q[2] > 0 ? std::sqrt(q[0] / q[2]) : 0.0;
    }
  }
  if (target_relres) *target_relres = worst;
}
}  // namespace

int hz_collect_pairs(hz_handle* h, const double* B, double* X, int64_t n, int32_t nrhs, int32_t mem, int32_t level,
                     int32_t sweeps, int64_t max_pairs, float* x_out, float* t_out, double* plain_err,
                     double* target_relres, int64_t* count) {
  if (!h) return HZ_ERR_ARG;
  return guarded(h, [&] {
    if (!x_out || !t_out || !count) fail(HZ_ERR_ARG, "null output");
    if (h->opt.precision != HZ_PREC_FP64) fail(HZ_ERR_ARG, "training pairs come from the FP64 solver");
    if (level < 1 || level >= h->opt.levels) fail(HZ_ERR_ARG, "level must be in [1, levels - 1]");
    if (sweeps < 1 || max_pairs < 1) fail(HZ_ERR_ARG, "sweeps and max_pairs must be >= 1");
    const Grid g = level_grid(h, level);
    if (h->prob.dim == 2)
      check_net_grid(g.nx, g.ny, 1);
    else
      check_net3_grid(g.nx, g.ny, g.nz, 1);
    set_device(h);
    const long long N = g.N;
    h->cap_buf.alloc((size_t)max_pairs * N * 16);
    hz::CoarseNet* saved = h->net;
    hz::CoarseNet3* saved3 = h->net3;
    h->net = nullptr;
    h->net3 = nullptr;
    h->cap_on = true;
    h->cap_level = level;
    h->cap_count = 0;
    h->cap_max = max_pairs;
    const int rc = hz_solve(h, B, X, n, nrhs, 0, mem, nullptr);
    h->cap_on = false;
    h->net = saved;
    h->net3 = saved3;
    if (rc < 0) fail(rc, "%s", h->err.c_str());
    Hierarchy& H = h->hier[0];
    const long long cnt = h->cap_count;
    const int R = h->rcap;
    if (h->prob.dim == 3) {
      collect_targets_iterative(h, H, level, sweeps, cnt, x_out, t_out, plain_err, target_relres);
      *count = cnt;
      return;
    }
    // targets: exact solves with a banded LU of the capture level's operator
    // (plain cycles as a stationary iteration need not converge on coarse levels)
    Level& Lv = *H.lv[level];
    std::vector<std::complex<double>> bT, bG;
    BandSolveOps lu;
    int kl = 0, ku = 0;
    band_factor_level(h, H, Lv, lu.blocks, bT, bG, kl, ku);
    DBuf dT, dG, dB, bw;
    dT.alloc(bT.size() * 16);
    dG.alloc(bG.size() * 16);
    dB.alloc(lu.blocks.size() * sizeof(BandBlock));
    ck(cudaMemcpy(dT.p, bT.data(), bT.size() * 16, cudaMemcpyHostToDevice), "upload band forward operators");
    ck(cudaMemcpy(dG.p, bG.data(), bG.size() * 16, cudaMemcpyHostToDevice), "upload band backward operators");
    ck(cudaMemcpy(dB.p, lu.blocks.data(), lu.blocks.size() * sizeof(BandBlock), cudaMemcpyHostToDevice),
       "upload band blocks");
    lu.N = N;
    lu.T = dT.as<double2>();
    lu.G = dG.as<double2>();
    lu.dblocks = dB.as<BandBlock>();
    bw.alloc((size_t)3 * R * N * 16);
    DBuf xe, res, ev, x1, idc, sc, nrm;
    xe.alloc((size_t)R * N * 16);
    res.alloc((size_t)R * N * 16);
    ev.alloc((size_t)R * N * 16);
    x1.alloc((size_t)R * N * 16);
    sc.alloc((size_t)R * 4);
    nrm.alloc((size_t)R * 6 * 8);
    idc.alloc((size_t)R * sizeof(int));
    std::vector<int> seq(R);
    for (int c = 0; c < R; ++c) seq[c] = c;
    ck(cudaMemcpy(idc.p, seq.data(), R * sizeof(int), cudaMemcpyHostToDevice), "upload cols");
    const int* dc = idc.as<int>();
    const float2* feat = net_features(h, level);
    std::vector<double> hn((size_t)R * 6);
    double worst = 0.0;
    for (long long i0 = 0; i0 < cnt; i0 += R) {
      const int k = (int)std::min<long long>(R, cnt - i0);
      const double2* r = h->cap_buf.as<double2>() + i0 * N;
      double2* xd = xe.as<double2>();
      // one plain cycle from this level (what the network replaces), then the exact solve
      mg_cycle<double, double>(h, H, level, r, x1.as<double2>(), dc, k);
      launch_band_solve<double>(h->ctx, lu, r, xd, N, dc, k, bw.as<double2>());
      for (int s = 1; s < sweeps; ++s) {  // iterative refinement with the same factors
        lev_op<double, double>(h, H, level, MODE_RESID, xd, r, res.as<double2>(), dc, k);
        launch_band_solve<double>(h->ctx, lu, res.as<double2>(), ev.as<double2>(), N, dc, k, bw.as<double2>());
        launch_axpy_compact(h->ctx, N, k, ev.as<double2>(), xd);
      }
      lev_op<double, double>(h, H, level, MODE_RESID, xd, r, res.as<double2>(), dc, k);
      launch_diff_norms(h->ctx, N, k, res.as<double2>(), r, nrm.as<double>());
      launch_diff_norms(h->ctx, N, k, x1.as<double2>(), xd, nrm.as<double>() + 3 * R);
      launch_pair_pack(h->ctx, N, r, xd, k, feat, h->net_h2, sc.as<float>(), x_out + i0 * N * 4, t_out + i0 * N * 2);
      ck(cudaMemcpyAsync(hn.data(), nrm.p, (size_t)R * 6 * 8, cudaMemcpyDeviceToHost, h->ctx.stream), "norms");
      sync(h);
      for (int c = 0; c < k; ++c) {
        const double rr = hn[3 * c + 2] > 0 ? std::sqrt(hn[3 * c + 1] / hn[3 * c + 2]) : 0.0;
        worst = std::max(worst, rr);
        const double* q = hn.data() + 3 * R + 3 * c;
        if (plain_err) plain_err[i0 + c] = q[2] > 0 ? std::sqrt(q[0] / q[2]) : 0.0;
      }
    }
    *count = cnt;
    if (target_relres) *target_relres = worst;
  });
}

}  // extern "C"
