/*
 * helmgpu -- GB300-native shifted-Laplacian multigrid Helmholtz solver (C ABI).
 *
 * Drop-in boundary for the acoustic path of JuliaInv/Helmholtz.jl.  Every
 * entry point takes plain pointers and sizes; no C++ or PyTorch types cross
 * this interface.  Complex values are interleaved (re, im) pairs of double
 * (Julia ComplexF64 / C99 double _Complex layout).  Node arrays are
 * column-major with axis 1 fastest, exactly the vec() ordering of the
 * reference (src/PlainNodalLaplacian.jl:32-46, src/getPointSource.jl:82-100).
 *
 * Device memory and streams: a call that reads caller-owned device memory
 * (mem = HZ_MEM_DEVICE, hz_apply_noalloc, the network's device inputs) first
 * makes its own stream wait for the work already issued to the legacy default
 * stream.  Work the caller queued on any other stream must be complete before
 * the call: synchronise that stream, or make hz_stream(h) wait on an event
 * recorded on it.  Every call returns after its outputs are complete.
 *
 * Status convention: 0 = ok, > 0 = finished but not converged (X is still
 * valid, the reference prints a warning: src/ShiftedLaplacianMultigridSolver.jl:97-99),
 * < 0 = error (the message is available from hz_last_error).  No exception
 * or C++ object crosses the ABI.  A handle is single-thread affine; it owns
 * its CUDA stream, device memory, multigrid hierarchy and coarsest LU factors.
 */
#ifndef HELMGPU_H
#define HELMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HZ_ABI_VERSION 1

/* status codes */
#define HZ_OK 0
#define HZ_NOT_CONVERGED 1
#define HZ_ERR_ARG (-1)
#define HZ_ERR_CUDA (-2)
#define HZ_ERR_ALLOC (-3)
#define HZ_ERR_NUMERIC (-4)
#define HZ_ERR_STATE (-5)
#define HZ_ERR_NO_DEVICE (-6)

/* where B / X / Y live */
#define HZ_MEM_HOST 0
#define HZ_MEM_DEVICE 1

/* precision of the multigrid preconditioner (the outer FGMRES is always FP64) */
#define HZ_PREC_FP64 0
#define HZ_PREC_MIXED 1 /* complex-FP32 V-cycle, FP64 coarsest LU */

/* outer FGMRES arithmetic: native FP64, or FP64 emulated with pairs of FP32
 * (basis stored as hi+lo, error-free FP32 transformations; ~2^-48 relative),
 * which runs on the FP32 pipe.  The true residual is native FP64 either way. */
#define HZ_OUTER_FP64 0
#define HZ_OUTER_EMULATED 1

#define HZ_KRYLOV_FGMRES 0
#define HZ_KRYLOV_BICGSTAB 1

#define HZ_COARSE_GALERKIN 0     /* A_{l+1} = R A_l P (reference default RAP path) */
#define HZ_COARSE_REDISCRETIZE 1 /* re-assembled 5/7-point operator from restricted m, gamma */

/* smoother (Multigrid.jl relaxType) */
#define HZ_RELAX_JAC 0       /* "Jac": relax_pre / relax_post damped-Jacobi sweeps */
#define HZ_RELAX_JAC_GMRES 1 /* "Jac-GMRES": relax_pre / relax_post (1 or 2) GMRES steps preconditioned by one
                                damped-Jacobi sweep, on the levels >= relax_from (finer levels: "Jac") */

#define HZ_OP_H 0  /* Helmholtz operator H */
#define HZ_OP_SH 1 /* shifted operator SH = H + i*shift*w^2*diag(m) */

/* The Helmholtz problem: the fields of HelmholtzParam (src/Helmholtz.jl:13-20)
 * plus the mesh (jInv RegularMesh: n cells per axis, h).  m and gamma are
 * copied at hz_create; the caller keeps ownership. */
typedef struct hz_problem {
  int32_t dim;             /* 2 or 3 */
  int64_t n[3];            /* cells per axis; nodes per axis = n + 1 */
  double h[3];             /* cell size per axis */
  double omega_re;         /* angular frequency (complex allowed for hz_apply only) */
  double omega_im;
  const double* m;         /* slowness squared at the nodes, prod(n+1) values */
  const double* gamma;     /* total attenuation at the nodes (absorbing layer included) */
  int32_t neumann_on_top;  /* HelmholtzParam.NeumannOnTop */
  int32_t sommerfeld;      /* HelmholtzParam.Sommerfeld */
  int32_t order_neumann_bc;/* 1 or 2 (reference default 2, src/PlainNodalLaplacian.jl:4-15) */
} hz_problem;

/* Solver options: the in-scope subset of Multigrid.jl getMGparam
 * (test/ShiftedLaplacianTest.jl:63-64) plus the solver constructor
 * arguments of getShiftedLaplacianMultigridSolver
 * (src/ShiftedLaplacianMultigridSolver.jl:24-30). */
typedef struct hz_options {
  int32_t levels;        /* multigrid levels (>= 1) */
  int32_t max_outer;     /* MGparam.maxOuterIter: FGMRES restart cycles */
  double rel_tol;        /* relative residual ||b - H x|| / ||b|| per column */
  int32_t relax_pre;     /* Jacobi sweeps (HZ_RELAX_JAC_GMRES: GMRES steps) before the coarse correction */
  int32_t relax_post;    /* Jacobi sweeps (HZ_RELAX_JAC_GMRES: GMRES steps) after the coarse correction */
  double relax_param;    /* Jacobi damping w */
  int32_t cycle;         /* 'V', 'W' or 'K' (K: two FGMRES steps per coarse level; FGMRES outer only) */
  int32_t krylov;        /* HZ_KRYLOV_* */
  int32_t inner;         /* FGMRES restart length */
  double shift;          /* s in SH = H + i s w^2 diag(m) */
  int32_t precision;     /* HZ_PREC_* */
  int32_t coarse_op;     /* HZ_COARSE_* */
  int32_t verbose;
  int32_t profile;       /* 1: time every kernel launch with CUDA events */
  int32_t device;        /* CUDA device ordinal */
  int32_t outer_arith;   /* FGMRES outer arithmetic: HZ_OUTER_FP64 (native) or HZ_OUTER_EMULATED */
  int32_t cuda_graph;    /* 1 (default): replay each FGMRES preconditioner application from a CUDA graph */
  int32_t autotune;      /* 1 (default): time the stencils' launch shapes at the first solve (see hz_tune_info) */
  int32_t relax_type;    /* HZ_RELAX_* (default HZ_RELAX_JAC) */
  int32_t relax_from;    /* HZ_RELAX_JAC_GMRES: first level smoothed by GMRES steps (0: every level) */
  int32_t reserved[2];
} hz_options;

typedef struct hz_stats {
  int32_t outer;           /* restart cycles performed */
  int32_t n_prec;          /* preconditioner applications (sum over columns) */
  int32_t max_col_iters;   /* most inner iterations taken by one column */
  int32_t converged_cols;  /* columns that reached rel_tol */
  double max_relres;       /* largest true relative residual over the columns */
  double setup_time;       /* seconds, accumulated like ShiftedLaplacianMultigridSolver.setupTime */
  double solve_time;       /* seconds, accumulated like .solveTime */
  int64_t kernel_launches; /* kernels launched by the last call */
  int64_t h2d_bytes;       /* host->device bytes copied by the last call */
  int64_t d2h_bytes;       /* device->host bytes copied by the last call */
} hz_stats;

typedef struct hz_handle hz_handle;

/* Library version (HZ_ABI_VERSION). */
int32_t hz_version(void);

/* Last error message of this handle, or of the calling thread when h is NULL. */
const char* hz_last_error(const hz_handle* h);

/* Fill options with the defaults of the reference's SLMG usage:
 * 3 levels, V(1,1) Jacobi w=0.8, FGMRES(10), shift 0.5, tol 1e-8. */
void hz_default_options(hz_options* opt);

/* Build a solver handle: replaces getShiftedLaplacianMultigridSolver
 * (src/ShiftedLaplacianMultigridSolver.jl:24-30) together with the operator
 * assembly of GetHelmholtzOperator (src/GetHelmholtz.jl:33-50) and
 * GetHelmholtzShiftOP (src/GetHelmholtz.jl:81-83), which the library keeps
 * matrix-free on the device.  The multigrid hierarchy is built lazily by the
 * first hz_solve, as MGsetup is (src/ShiftedLaplacianMultigridSolver.jl:50-66).
 * With the environment variable HELMGPU_RAP_TILED=1 at this call, the handle's
 * 3D Galerkin stencils in the complex-FP32 cycle use the staged-tile kernel
 * (same results; an experimental launch shape, off by default). */
int hz_create(const hz_problem* prob, const hz_options* opt, hz_handle** out);

/* Release everything the handle owns. */
int hz_destroy(hz_handle* h);

/* Solve H X = B (transpose = 0) or H^H X = B (transpose = 1) for nrhs columns:
 * replaces solveLinearSystem(ShiftedHT, B, param, doTranspose)
 * (src/ShiftedLaplacianMultigridSolver.jl:33-102).  B and X are n x nrhs
 * column-major complex, on the host or the device (mem).  Zero columns give
 * zero solutions; stats may be NULL. */
int hz_solve(hz_handle* h, const double* B, double* X, int64_t n, int32_t nrhs, int32_t transpose,
             int32_t mem, hz_stats* stats);

/* Per-column results of the last hz_solve: true relative residual and inner
 * iterations taken.  Either pointer may be NULL. */
int hz_column_stats(const hz_handle* h, double* relres, int32_t* iters, int32_t nrhs);

/* Y = op X with op = H or SH (transpose = 1: the adjoint): the matrix-free
 * replacement of getHelmholtzFun's closure (src/GetHelmholtz.jl:85-95) and of
 * the sparse products H*x the reference tests take.  The apply does not work in
 * place: device X and Y that overlap are rejected with HZ_ERR_ARG.  The column
 * list the kernel reads is kept in the handle and grows only with nrhs. */
int hz_apply(hz_handle* h, int32_t op, int32_t transpose, const double* X, double* Y, int64_t n, int32_t nrhs,
             int32_t mem);

/* Allocation-free variant of hz_apply, for callers that cannot allocate GPU
 * memory at the time they apply the operator: an application whose own pool
 * already holds the whole device, a solver loop whose memory footprint must
 * stay fixed, or code that must avoid cudaMalloc's implicit device-wide
 * synchronisation.  This entry point has no counterpart in the reference.
 * X and Y are device pointers (n x nrhs column-major complex); the call
 * allocates nothing: the column list the kernel needs lives in a static
 * device array of HZ_NOALLOC_MAX_COLS entries (16 KiB, held by every GPU that
 * loads the library until the process exits), so nrhs above that maximum is
 * rejected with HZ_ERR_ARG.  The first call on a device looks up that array's
 * device address (cudaGetSymbolAddress) with the device current; make that
 * first call before any stream capture.  All calls on a device share the
 * array: calls that overlap on the GPU (different handles or streams) race.
 * X must be complete before the call (see "Device memory and streams" above)
 * and must not overlap Y (HZ_ERR_ARG).  Returns after the result is complete,
 * like hz_apply. */
#define HZ_NOALLOC_MAX_COLS 4096
int hz_apply_noalloc(hz_handle* h, int32_t op, int32_t transpose, const double* X, double* Y, int64_t n,
                     int32_t nrhs);

/* Drop the multigrid hierarchy (clear!, src/ShiftedLaplacianMultigridSolver.jl:105-109). */
int hz_clear(hz_handle* h);

/* Independent copy of a handle's problem and options (copySolver,
 * src/ShiftedLaplacianMultigridSolver.jl:18-22); the hierarchy is rebuilt lazily. */
int hz_copy(const hz_handle* h, hz_handle** out);

/* The CUDA stream (cudaStream_t) every kernel of this handle runs on. */
void* hz_stream(hz_handle* h);

/* Per-kernel launch table of the handle: entry idx -> kernel name, launches,
 * launches timed with CUDA events (while profiling is on), their total
 * milliseconds, and the algorithmic bytes of all launches (each input read
 * once, each output written once).  Returns the number of entries (call with
 * idx = -1 to get it), or < 0 on error.  Output pointers may be NULL. */
int hz_kernel_times(hz_handle* h, int32_t idx, char* name, int32_t name_len, int64_t* launches,
                    int64_t* timed_launches, double* total_ms, double* alg_bytes);
int hz_reset_kernel_times(hz_handle* h);
/* Launch shapes chosen by the autotuner for this handle: CTAs aimed at per launch
 * of the fine-level and the Galerkin stencils (0 = the default rule).  Timed on the
 * handle's own level sizes at the first solve with a new column count; cached per
 * process and, when the environment variable HELMGPU_TUNE_CACHE names a file,
 * persisted there.  Returns HZ_OK once tuned, HZ_NOT_CONVERGED before. */
int hz_tune_info(const hz_handle* h, int32_t* fine_ctas, int32_t* rap_ctas);
/* Algorithmic flops of entry idx of the launch table: the tensor-core kernels of
 * the learned correction (BF16) and the native-FP64 kernels of the outer Krylov
 * method (krylov_dots, krylov_update, update_x, outer_apply, outer_resid: the
 * complex arithmetic they do in FP64); 0 for the other, memory-bound kernels. */
int hz_kernel_flops(hz_handle* h, int32_t idx, double* alg_flops);
/* Replay the preconditioner applications from CUDA graphs (1) or launch them
 * eagerly (0) from the next application on (options.cuda_graph at create time);
 * graphs already captured are kept for when replay is switched back on.  Eager
 * launches let per-launch profiling time each kernel of the cycle. */
int hz_set_cuda_graph(hz_handle* h, int32_t on);
/* Turn per-launch CUDA-event timing on (1) or off (0) (options.profile at create time). */
int hz_set_profile(hz_handle* h, int32_t on);

/* ---- learned coarse-grid correction ------------------------------------------
 * No counterpart in the reference: the reference's multigrid always recurses to
 * its coarsest LU.  A small 2D convolutional encoder-decoder (BF16 weights and
 * activations, FP32 accumulation on the tensor cores; 8 layers of 3x3
 * convolutions, 16-32-64-64 channels over four grid levels) replaces the
 * coarse-grid correction below one multigrid level.  It is trained on the GPU
 * by the library's own forward and backward kernels on (residual, error) pairs
 * the FP64 solver produces (hz_collect_pairs).
 *
 * Pair / input layout on a network grid of nx x ny nodes (axis 1 fastest, node
 * counts 8k+1): x [batch][nx*ny][4] FP32 = (Re r/s, Im r/s, w^2 m hx hy, gamma/w)
 * with s the RMS of r over the grid and hx, hy the level's cell sizes;
 * target / output [batch][nx*ny][2] FP32 = (Re, Im) of e / (hx hy s).
 * Weights (FP32 on the host): layer after layer, each [cout][9][cin] with tap
 * index 3 (dy + 1) + (dx + 1), dx along axis 1.  Loss: mean over the batch of
 * ||y - t||^2 / ||t||^2. */
typedef struct hz_net hz_net;

/* New network with seeded He-normal weights on a device. */
int hz_net_create(int32_t seed, int32_t device, hz_net** out);
int hz_net_destroy(hz_net* net);
/* Number of weights (FP32 values of hz_net_get_weights). */
int64_t hz_net_num_params(void);
/* Input and output channels of layer 0..7. */
int hz_net_layer_shape(int32_t layer, int32_t* cin, int32_t* cout);
int hz_net_get_weights(hz_net* net, float* w);
/* Replaces the weights (and resets the optimiser state). */
int hz_net_set_weights(hz_net* net, const float* w);
/* y = net(x) for a batch (x, y on the host or the device: mem). */
int hz_net_forward(hz_net* net, const float* x, float* y, int64_t nx, int64_t ny, int32_t batch, int32_t mem);
/* Loss and its gradient with respect to the weights (host array laid out like
 * the weights; may be NULL) for one batch; the weights are unchanged. */
int hz_net_gradient(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int32_t batch, int32_t mem,
                    double* loss, float* grad);
/* Adam over npairs device-resident pairs (x, t as above) in shuffled
 * mini-batches for epochs passes, learning rate lr with cosine decay to lr/20;
 * loss_hist (host, epochs entries, may be NULL) gets the mean loss per epoch. */
int hz_net_train(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t npairs, int32_t batch,
                 int32_t epochs, double lr, int32_t seed, double* loss_hist);
/* Versioned binary file of the weights and the Adam state ("HZCNET01", version,
 * layer shapes, parameter count, step, weights, moments): training resumes from a
 * loaded file.  Load rejects a file of another format, version or shape, a
 * truncated one, or one with non-finite values (HZ_ERR_ARG, weights unchanged).
 * hz_net_file_info checks a file on the host only (no GPU). */
int hz_net_save(hz_net* net, const char* path);
int hz_net_load(hz_net* net, const char* path);
int hz_net_file_info(const char* path, int64_t* nparams, int64_t* adam_step);
/* Launch table of the network's own stream (training, standalone inference),
 * as hz_kernel_times plus the algorithmic flops; profiling on/off and reset. */
int hz_net_set_profile(hz_net* net, int32_t on);
int hz_net_kernel_times(hz_net* net, int32_t idx, char* name, int32_t name_len, int64_t* launches,
                        int64_t* timed_launches, double* total_ms, double* alg_bytes, double* alg_flops);
int hz_net_reset_kernel_times(hz_net* net);
/* 3D variant (no counterpart in the reference either): a convolutional
 * encoder-decoder over three grid levels with 8-16-32 channels and 3x3x3
 * convolutions (six layers; BF16 weights and activations, FP32 accumulation on
 * the tensor cores).  Input and output layouts as above on an nx x ny x nz grid
 * (axis 1 fastest, node counts 4k+1); weights layer after layer, each
 * [cout][27][cin] with tap 9 (dz + 1) + 3 (dy + 1) + (dx + 1).  The functions
 * hz_net_get_weights, hz_net_set_weights, hz_net_save, hz_net_load,
 * hz_net_set_profile, hz_net_kernel_times, hz_net_reset_kernel_times and
 * hz_attach_net take either kind; hz_net_file_info reads either file format. */
int hz_net3d_create(int32_t seed, int32_t device, hz_net** out);
int64_t hz_net3d_num_params(void);
int hz_net3d_layer_shape(int32_t layer, int32_t* cin, int32_t* cout);
/* 2 or 3: the grid dimension of a network. */
int hz_net_dim(const hz_net* net);
int hz_net3d_forward(hz_net* net, const float* x, float* y, int64_t nx, int64_t ny, int64_t nz, int32_t batch,
                     int32_t mem);
int hz_net3d_gradient(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t nz, int32_t batch,
                      int32_t mem, double* loss, float* grad);
int hz_net3d_train(hz_net* net, const float* x, const float* t, int64_t nx, int64_t ny, int64_t nz, int64_t npairs,
                   int32_t batch, int32_t epochs, double lr, int32_t seed, double* loss_hist);
/* Convolution kernels of a network: HZ_NET_CONV_WARP_MMA (warp-level mma.sync,
 * every layer), HZ_NET_CONV_TCGEN05 (5th-generation tensor cores, tcgen05.mma
 * with the accumulator in tensor memory and the operands staged by the TMA
 * unit; 2D: the layers whose channel counts are multiples of 16, the 8-channel
 * output layer keeps the warp-level kernel; 3D: every layer, the 8-channel
 * layers computing 16 output channels and storing 8; the weight gradients
 * too) or HZ_NET_CONV_AUTO (the default: per layer the faster of the two; the
 * 2D network's tensor-core layers all, the 3D network's where its tiles waste
 * at most 3.5x the work on that layer's grid; the weight gradients on the
 * warp-level kernels, which measured faster). */
#define HZ_NET_CONV_WARP_MMA 0
#define HZ_NET_CONV_TCGEN05 1
#define HZ_NET_CONV_AUTO 2
int hz_net_set_conv_path(hz_net* net, int32_t path);
/* Use the network for the coarse-grid correction of multigrid level `level`
 * (1 .. levels-1; a network of the problem's dimension; FGMRES only: the
 * network is a nonlinear preconditioner).  With the K-cycle the network
 * preconditions the two FGMRES steps on its level in place of that level's
 * cycle; with the V and W cycles it replaces the level's cycle.
 * A restart cycle that reduces some column's residual by less than stag_ratio
 * hands the rest of that solve to the plain cycle.  net = NULL detaches.  The
 * handle does not own the network; keep it alive while attached, and use one
 * network with one solve at a time. */
int hz_attach_net(hz_handle* h, hz_net* net, int32_t level, double stag_ratio);
/* Network applications (blocks of columns) and fallbacks to the plain cycle so far. */
int hz_learned_stats(const hz_handle* h, int64_t* net_calls, int32_t* fallbacks);
/* Training pairs: solves H X = B (FP64 preconditioner, no network) like
 * hz_solve while recording the right-hand side r that each cycle hands to
 * `level` (at most max_pairs columns), then computes the target e = A^{-1} r on
 * that level: in 2D with a banded LU of its operator (FP64) followed by
 * sweeps - 1 steps of iterative refinement; in 3D (where the band LU of a
 * coarse level is out of reach) from one cycle on that level followed by
 * sweeps - 1 restarted FP64 two-step
 * FGMRES corrections e += K(r - A e) preconditioned by the level's cycle (which
 * never raise the residual); on the coarsest level the cycle is the band LU and
 * its solve is the target.  In 3D the grid is nx x ny x nz and plain_err
 * compares one cycle on that level (what the network stands for) with the target.
 * x_out [max_pairs][N][4] and t_out [max_pairs][N][2] are DEVICE FP32 arrays in
 * the layout above; plain_err (host, may be NULL) gets ||e1 - e|| / ||e|| of one
 * plain cycle e1 per pair, target_relres (may be NULL) the largest
 * ||r - A e|| / ||r|| of the targets, count the pairs written. */
int hz_collect_pairs(hz_handle* h, const double* B, double* X, int64_t n, int32_t nrhs, int32_t mem, int32_t level,
                     int32_t sweeps, int64_t max_pairs, float* x_out, float* t_out, double* plain_err,
                     double* target_relres, int64_t* count);

/* ---- host-side discretisation helpers (no GPU needed) ---------------------- */

/* getMaximalFrequency (src/GetHelmholtz.jl:75-79): 0.2*pi / (max(h) sqrt(max(m))). */
double hz_max_frequency(const double* m, int64_t count, const double* h, int32_t dim);

/* getABL (src/GetHelmholtz.jl:97-220): absorbing-layer gamma on the node grid
 * nodes[dim]; pad[dim] layer widths; writes prod(nodes) values. */
int hz_abl(int32_t dim, const int64_t* nodes, int32_t neumann_at_first_dim, const int64_t* pad, double amp,
           double* gamma_out);

/* getSommerfeldBC (src/GetHelmholtz.jl:222-247): complex boundary term on the
 * node grid (interleaved complex, prod(n+1) values). */
int hz_sommerfeld(int32_t dim, const int64_t* n, const double* h, const double* m, double omega,
                  int32_t neumann_on_top, int32_t order_neumann_bc, double* somm_out);

/* Diagonal of H (src/GetHelmholtz.jl:41-47): -w^2 m (1 - i gamma / Re w) - Somm.
 * Somm is getSommerfeldBC with its default order 2 whatever order_neumann_bc is:
 * the reference calls it without the order (src/GetHelmholtz.jl:45). */
int hz_helmholtz_mass(const hz_problem* prob, double* mass_out);

/* getAcousticPointSource with getTopPointSrc / loc2cs (src/getPointSource.jl:63-111):
 * 1-based node subscript src[dim]; writes a complex column of prod(n+1) values. */
int hz_point_source(int32_t dim, const int64_t* n, const double* h, const int64_t* src, double* q_out);

#ifdef __cplusplus
}
#endif

#endif /* HELMGPU_H */
