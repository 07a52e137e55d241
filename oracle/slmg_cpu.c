/*
 * CPU oracle / CPU baseline: plain complex-FP64 shifted-Laplacian multigrid
 * preconditioned FGMRES with threaded CSR sparse products.
 *
 * TEST INFRASTRUCTURE ONLY.  Called by tests/, __graft_entry__.smoke() and
 * the cpu_baseline / reference legs of bench.py through ctypes (see
 * oracle/slmg_cpu.py); the product never links or calls it.
 *
 * It restates the solve phase of the reference path:
 *   - SpMatMul / ParSpMatVec threaded CSR products (src/GetHelmholtz.jl:90-91;
 *     ParSpMatVec v0.1.1, C/OpenMP, pinned in Manifest.toml:106-110),
 *   - the Multigrid.jl V/W/K cycle with damped Jacobi or Jac-GMRES, full-weighting
 *     restriction and linear prolongation given as CSR matrices, and a
 *     direct (banded LU, partial pivoting) coarsest solve,
 *   - FGMRES(restart) per column with classical Gram-Schmidt and the DGKS
 *     second pass (where ||w'||^2 < ||w||^2/2), Givens rotations, relative-residual test,
 *     the same algorithm as oracle/helmholtz_oracle.py:fgmres
 *     (src/ShiftedLaplacianMultigridSolver.jl:89 calls it as solveGMRES_MG).
 * The hierarchy (A_l, P_l, R_l) is assembled by the Python oracle.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

typedef struct {
  int64_t nrows, ncols;
  const int64_t* indptr;
  const int64_t* indices;
  const cplx* data;
} csr_t;

typedef struct {
  int nlev;
  csr_t A[16], P[16], R[16];
  cplx* dinv[16];
  /* coarsest band LU */
  int64_t nc, kl, ku, ldab;
  cplx* ab;
  int64_t* ipiv;
} slmg_t;

static void spmm(const csr_t* A, const cplx* X, int64_t ldx, cplx* Y, int64_t ldy, int nrhs, int accumulate,
                 cplx alpha) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A->nrows; ++i) {
    for (int c = 0; c < nrhs; ++c) {
      cplx s = 0;
      const cplx* xc = X + (int64_t)c * ldx;
      for (int64_t k = A->indptr[i]; k < A->indptr[i + 1]; ++k) s += A->data[k] * xc[A->indices[k]];
      if (accumulate)
        Y[(int64_t)c * ldy + i] += alpha * s;
      else
        Y[(int64_t)c * ldy + i] = alpha * s;
    }
  }
}

static int band_factor(slmg_t* S, const csr_t* A) {
  const int64_t N = A->nrows;
  int64_t kl = 0, ku = 0;
  for (int64_t i = 0; i < N; ++i)
    for (int64_t k = A->indptr[i]; k < A->indptr[i + 1]; ++k) {
      int64_t j = A->indices[k];
      if (i - j > kl) kl = i - j;
      if (j - i > ku) ku = j - i;
    }
  const int64_t ldab = 2 * kl + ku + 1, kv = kl + ku;
  cplx* ab = (cplx*)calloc((size_t)(ldab * N), sizeof(cplx));
  int64_t* ipiv = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
  if (!ab || !ipiv) return -1;
#define AB(i, j) ab[(j) * ldab + kv + (i) - (j)]
  for (int64_t i = 0; i < N; ++i)
    for (int64_t k = A->indptr[i]; k < A->indptr[i + 1]; ++k) AB(i, A->indices[k]) += A->data[k];
  int64_t ju = 0;
  for (int64_t j = 0; j < N; ++j) {
    int64_t km = kl < N - 1 - j ? kl : N - 1 - j;
    int64_t jp = 0;
    double best = -1;
    for (int64_t r = 0; r <= km; ++r) {
      double m = fabs(creal(AB(j + r, j))) + fabs(cimag(AB(j + r, j)));
      if (m > best) {
        best = m;
        jp = r;
      }
    }
    ipiv[j] = j + jp;
    if (best == 0) return (int)(j + 1);
    int64_t t = j + ku + jp;
    if (t > N - 1) t = N - 1;
    if (t > ju) ju = t;
    if (jp)
      for (int64_t c = j; c <= ju; ++c) {
        cplx tmp = AB(j, c);
        AB(j, c) = AB(j + jp, c);
        AB(j + jp, c) = tmp;
      }
    if (km > 0) {
      cplx inv = 1.0 / AB(j, j);
      for (int64_t r = 1; r <= km; ++r) AB(j + r, j) *= inv;
#pragma omp parallel for schedule(static) if ((ju - j) * km > 16384)
      for (int64_t c = j + 1; c <= ju; ++c) {
        cplx a = AB(j, c);
        if (a != 0)
          for (int64_t r = 1; r <= km; ++r) AB(j + r, c) -= AB(j + r, j) * a;
      }
    }
  }
#undef AB
  S->nc = N;
  S->kl = kl;
  S->ku = ku;
  S->ldab = ldab;
  S->ab = ab;
  S->ipiv = ipiv;
  return 0;
}

static void band_solve(const slmg_t* S, const cplx* b, int64_t ldb, cplx* x, int64_t ldx, int nrhs) {
  const int64_t N = S->nc, kl = S->kl, kv = S->kl + S->ku, ldab = S->ldab;
  const cplx* ab = S->ab;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nrhs; ++c) {
    cplx* v = x + (int64_t)c * ldx;
    if (v != b + (int64_t)c * ldb) memcpy(v, b + (int64_t)c * ldb, sizeof(cplx) * (size_t)N);
    for (int64_t j = 0; j < N - 1; ++j) {
      int64_t lm = kl < N - 1 - j ? kl : N - 1 - j;
      int64_t l = S->ipiv[j];
      if (l != j) {
        cplx t = v[l];
        v[l] = v[j];
        v[j] = t;
      }
      const cplx* L = ab + j * ldab + kv;
      for (int64_t r = 1; r <= lm; ++r) v[j + r] -= L[r] * v[j];
    }
    for (int64_t j = N - 1; j >= 0; --j) {
      const cplx* U = ab + j * ldab + kv;
      v[j] /= U[0];
      int64_t lo = j - kv > 0 ? j - kv : 0;
      for (int64_t i = lo; i < j; ++i) v[i] -= U[i - j] * v[j];
    }
  }
}

void* slmg_create(int nlev, const int64_t* meta, const int64_t* const* indptr, const int64_t* const* indices,
                  const double* const* data) {
  /* matrices per level l: A_l at slot 3l, P_l at 3l+1, R_l at 3l+2 (P, R absent on the last level);
     meta[2*slot] = rows, meta[2*slot+1] = cols */
  slmg_t* S = (slmg_t*)calloc(1, sizeof(slmg_t));
  if (!S || nlev < 1 || nlev > 16) return NULL;
  S->nlev = nlev;
  for (int l = 0; l < nlev; ++l) {
    for (int k = 0; k < 3; ++k) {
      int slot = 3 * l + k;
      if (l == nlev - 1 && k > 0) continue;
      csr_t* M = k == 0 ? &S->A[l] : (k == 1 ? &S->P[l] : &S->R[l]);
      M->nrows = meta[2 * slot];
      M->ncols = meta[2 * slot + 1];
      M->indptr = indptr[slot];
      M->indices = indices[slot];
      M->data = (const cplx*)data[slot];
    }
    const csr_t* A = &S->A[l];
    S->dinv[l] = (cplx*)malloc(sizeof(cplx) * (size_t)A->nrows);
    for (int64_t i = 0; i < A->nrows; ++i) {
      cplx d = 0;
      for (int64_t k = A->indptr[i]; k < A->indptr[i + 1]; ++k)
        if (A->indices[k] == i) d += A->data[k];
      S->dinv[l][i] = 1.0 / d;
    }
  }
  if (band_factor(S, &S->A[nlev - 1]) != 0) return NULL;
  return S;
}

void slmg_destroy(void* h) {
  slmg_t* S = (slmg_t*)h;
  if (!S) return;
  for (int l = 0; l < S->nlev; ++l) free(S->dinv[l]);
  free(S->ab);
  free(S->ipiv);
  free(S);
}

int slmg_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

typedef struct {
  double w;
  int pre, post, wcycle; /* wcycle: 0 V, 1 W, 2 K */
  int relax;             /* 0 damped Jacobi ("Jac"), 1 "Jac-GMRES" */
  int gmres_from;        /* Jac-GMRES: first level smoothed by GMRES (finer levels: Jacobi) */
} cyc_t;

static void mg_cycle(const slmg_t* S, int l, const cplx* b, cplx* x, int nrhs, const cyc_t* cp);

/* relaxType "Jac-GMRES" (set by test/ShiftedLaplacianTest.jl:138; Multigrid.jl
   v0.8.0 is not vendored, so the published method is restated, as in
   oracle/helmholtz_oracle.py:gmres_relax): `steps` Arnoldi steps of GMRES on
   level l's operator from the current x, right-preconditioned by one damped
   Jacobi sweep (w D^-1), classical Gram-Schmidt, the (steps+1) x steps least
   squares by complex Givens rotations, then x += Z y per column. */
static void gmres_relax(const slmg_t* S, int l, const cplx* b, cplx* x, int nrhs, double w, int steps) {
  if (steps <= 0) return;
  const csr_t* A = &S->A[l];
  const int64_t n = A->nrows;
  const cplx* di = S->dinv[l];
  const int64_t blk = n * (int64_t)nrhs;
  cplx* V = (cplx*)malloc(sizeof(cplx) * (size_t)(steps + 1) * (size_t)blk);
  cplx* Z = (cplx*)malloc(sizeof(cplx) * (size_t)steps * (size_t)blk);
  cplx* u = (cplx*)malloc(sizeof(cplx) * (size_t)blk);
  cplx* Hm = (cplx*)calloc((size_t)(steps + 1) * steps * nrhs, sizeof(cplx)); /* Hm[(c*(steps+1)+i)*steps+j] */
  double* beta = (double*)calloc((size_t)nrhs, sizeof(double));
  spmm(A, x, n, u, n, nrhs, 0, 1.0);
  for (int c = 0; c < nrhs; ++c) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) {
      const cplx r = b[c * n + i] - u[c * n + i];
      V[c * n + i] = r;
      s += creal(r) * creal(r) + cimag(r) * cimag(r);
    }
    beta[c] = sqrt(s);
    const double inv = beta[c] > 0 ? 1.0 / beta[c] : 1.0;
    for (int64_t i = 0; i < n; ++i) V[c * n + i] *= inv;
  }
  for (int j = 0; j < steps; ++j) {
    cplx* Vj = V + (int64_t)j * blk;
    cplx* Zj = Z + (int64_t)j * blk;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < nrhs; ++c) Zj[c * n + i] = w * di[i] * Vj[c * n + i];
    spmm(A, Zj, n, u, n, nrhs, 0, 1.0);
    for (int c = 0; c < nrhs; ++c) {
      cplx* uc = u + (int64_t)c * n;
      cplx h[64];
      for (int i = 0; i <= j; ++i) {
        const cplx* Vi = V + (int64_t)i * blk + (int64_t)c * n;
        cplx d = 0;
        for (int64_t k = 0; k < n; ++k) d += conj(Vi[k]) * uc[k];
        h[i] = d;
      }
      double s = 0;
      for (int64_t k = 0; k < n; ++k) {
        cplx v = uc[k];
        for (int i = 0; i <= j; ++i) v -= h[i] * V[(int64_t)i * blk + (int64_t)c * n + k];
        uc[k] = v;
        s += creal(v) * creal(v) + cimag(v) * cimag(v);
      }
      const double hn = sqrt(s), inv = hn > 0 ? 1.0 / hn : 0.0;
      for (int i = 0; i <= j; ++i) Hm[((int64_t)c * (steps + 1) + i) * steps + j] = h[i];
      Hm[((int64_t)c * (steps + 1) + j + 1) * steps + j] = hn;
      cplx* Vn = V + (int64_t)(j + 1) * blk + (int64_t)c * n;
      for (int64_t k = 0; k < n; ++k) Vn[k] = inv * uc[k];
    }
  }
  for (int c = 0; c < nrhs; ++c) {
    if (beta[c] == 0) continue;
    cplx R[65][64], g[65], y[64];
    for (int i = 0; i <= steps; ++i) {
      g[i] = i == 0 ? beta[c] : 0;
      for (int j = 0; j < steps; ++j) R[i][j] = Hm[((int64_t)c * (steps + 1) + i) * steps + j];
    }
    for (int j = 0; j < steps; ++j) { /* rotate rows j, j+1 to zero R[j+1][j] */
      const cplx a = R[j][j], e = R[j + 1][j];
      const double r = sqrt(creal(a) * creal(a) + cimag(a) * cimag(a) + creal(e) * creal(e) + cimag(e) * cimag(e));
      if (r == 0) continue;
      const cplx cs = a / r, sn = e / r;
      for (int k = j; k < steps; ++k) {
        const cplx top = R[j][k], bot = R[j + 1][k];
        R[j][k] = conj(cs) * top + conj(sn) * bot;
        R[j + 1][k] = -sn * top + cs * bot;
      }
      const cplx gt = g[j], gb = g[j + 1];
      g[j] = conj(cs) * gt + conj(sn) * gb;
      g[j + 1] = -sn * gt + cs * gb;
    }
    for (int j = steps - 1; j >= 0; --j) {
      cplx v = g[j];
      for (int k = j + 1; k < steps; ++k) v -= R[j][k] * y[k];
      y[j] = R[j][j] != 0 ? v / R[j][j] : 0;
    }
    for (int j = 0; j < steps; ++j) {
      const cplx* Zj = Z + (int64_t)j * blk + (int64_t)c * n;
      for (int64_t k = 0; k < n; ++k) x[c * n + k] += y[j] * Zj[k];
    }
  }
  free(V);
  free(Z);
  free(u);
  free(Hm);
  free(beta);
}

/* K-cycle coarse correction on level l (Multigrid.jl cycleType 'K' of
   test/ShiftedLaplacianTest.jl:137-140, restated): two steps of FGMRES on the
   level's operator from a zero guess, right-preconditioned by the level's own
   cycle, per column (3x2 least squares by two complex Givens rotations). */
static void kcycle(const slmg_t* S, int l, const cplx* b, cplx* x, int nrhs, const cyc_t* cp) {
  const csr_t* A = &S->A[l];
  const int64_t n = A->nrows;
  const size_t bytes = sizeof(cplx) * (size_t)n * nrhs;
  cplx* V0 = (cplx*)malloc(bytes);
  cplx* V1 = (cplx*)malloc(bytes);
  cplx* Z0 = (cplx*)malloc(bytes);
  cplx* Z1 = (cplx*)malloc(bytes);
  cplx* W = (cplx*)malloc(bytes);
  double* beta = (double*)calloc((size_t)nrhs, sizeof(double));
  cplx* hs = (cplx*)calloc((size_t)nrhs * 6, sizeof(cplx)); /* h00 h10 h01 h11 h21 per column */
  for (int c = 0; c < nrhs; ++c) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += creal(b[c * n + i]) * creal(b[c * n + i]) + cimag(b[c * n + i]) * cimag(b[c * n + i]);
    beta[c] = sqrt(s);
    const double inv = beta[c] > 0 ? 1.0 / beta[c] : 0.0;
    for (int64_t i = 0; i < n; ++i) V0[c * n + i] = inv * b[c * n + i];
  }
  mg_cycle(S, l, V0, Z0, nrhs, cp);
  spmm(A, Z0, n, W, n, nrhs, 0, 1.0);
  for (int c = 0; c < nrhs; ++c) {
    cplx h00 = 0;
    for (int64_t i = 0; i < n; ++i) h00 += conj(V0[c * n + i]) * W[c * n + i];
    double s = 0;
    for (int64_t i = 0; i < n; ++i) {
      W[c * n + i] -= h00 * V0[c * n + i];
      s += creal(W[c * n + i]) * creal(W[c * n + i]) + cimag(W[c * n + i]) * cimag(W[c * n + i]);
    }
    const double h10 = sqrt(s), inv = h10 > 0 ? 1.0 / h10 : 0.0;
    for (int64_t i = 0; i < n; ++i) V1[c * n + i] = inv * W[c * n + i];
    hs[c * 6 + 0] = h00;
    hs[c * 6 + 1] = h10;
  }
  mg_cycle(S, l, V1, Z1, nrhs, cp);
  spmm(A, Z1, n, W, n, nrhs, 0, 1.0);
  for (int c = 0; c < nrhs; ++c) {
    cplx h01 = 0, h11 = 0;
    for (int64_t i = 0; i < n; ++i) {
      h01 += conj(V0[c * n + i]) * W[c * n + i];
      h11 += conj(V1[c * n + i]) * W[c * n + i];
    }
    double s = 0;
    for (int64_t i = 0; i < n; ++i) {
      const cplx v = W[c * n + i] - h01 * V0[c * n + i] - h11 * V1[c * n + i];
      s += creal(v) * creal(v) + cimag(v) * cimag(v);
    }
    const cplx a = hs[c * 6 + 0], bb = h01, d = h11;
    const double c10 = creal(hs[c * 6 + 1]), e = sqrt(s);
    cplx y0 = 0, y1 = 0;
    const double r1 = sqrt(creal(a) * creal(a) + cimag(a) * cimag(a) + c10 * c10);
    if (beta[c] > 0 && r1 > 0) {
      const cplx cs = a / r1;
      const double sn = c10 / r1;
      const cplx bp = conj(cs) * bb + sn * d, dp = -sn * bb + cs * d;
      const cplx g0 = conj(cs) * beta[c];
      const double g1 = -sn * beta[c];
      const double r2 = sqrt(creal(dp) * creal(dp) + cimag(dp) * cimag(dp) + e * e);
      if (r2 > 0) y1 = conj(dp) * g1 / (r2 * r2);
      y0 = (g0 - bp * y1) / r1;
    }
    for (int64_t i = 0; i < n; ++i) x[c * n + i] = y0 * Z0[c * n + i] + y1 * Z1[c * n + i];
  }
  free(V0);
  free(V1);
  free(Z0);
  free(Z1);
  free(W);
  free(beta);
  free(hs);
}

/* x = cycle(b) on level l, zero initial guess, nrhs columns (ld = level size). */
static void mg_cycle(const slmg_t* S, int l, const cplx* b, cplx* x, int nrhs, const cyc_t* cp) {
  const csr_t* A = &S->A[l];
  const int64_t n = A->nrows;
  if (l == S->nlev - 1) {
    band_solve(S, b, n, x, n, nrhs);
    return;
  }
  const size_t bytes = sizeof(cplx) * (size_t)n * nrhs;
  cplx* r = (cplx*)malloc(bytes);
  const int64_t nc = S->A[l + 1].nrows;
  cplx* bc = (cplx*)malloc(sizeof(cplx) * (size_t)nc * nrhs);
  cplx* xc = (cplx*)malloc(sizeof(cplx) * (size_t)nc * nrhs);
  memset(x, 0, bytes);
  const cplx* di = S->dinv[l];
  const int use_gmres = cp->relax == 1 && l >= cp->gmres_from;
  if (use_gmres) gmres_relax(S, l, b, x, nrhs, cp->w, cp->pre);
  for (int s = 0; s < (use_gmres ? 0 : cp->pre); ++s) {
    spmm(A, x, n, r, n, nrhs, 0, 1.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < nrhs; ++c) x[c * n + i] += cp->w * di[i] * (b[c * n + i] - r[c * n + i]);
  }
  int ncalls = (cp->wcycle == 1 && l < S->nlev - 2) ? 2 : 1;
  for (int call = 0; call < ncalls; ++call) {
    spmm(A, x, n, r, n, nrhs, 0, 1.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n * nrhs; ++i) r[i] = b[i] - r[i];
    spmm(&S->R[l], r, n, bc, nc, nrhs, 0, 1.0);
    if (cp->wcycle == 2 && l + 1 < S->nlev - 1)
      kcycle(S, l + 1, bc, xc, nrhs, cp);
    else
      mg_cycle(S, l + 1, bc, xc, nrhs, cp);
    spmm(&S->P[l], xc, nc, x, n, nrhs, 1, 1.0);
  }
  if (use_gmres) gmres_relax(S, l, b, x, nrhs, cp->w, cp->post);
  for (int s = 0; s < (use_gmres ? 0 : cp->post); ++s) {
    spmm(A, x, n, r, n, nrhs, 0, 1.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < nrhs; ++c) x[c * n + i] += cp->w * di[i] * (b[c * n + i] - r[c * n + i]);
  }
  free(r);
  free(bc);
  free(xc);
}

static double col_norm(const cplx* x, int64_t n) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += creal(x[i]) * creal(x[i]) + cimag(x[i]) * cimag(x[i]);
  return sqrt(s);
}

/* FGMRES(restart) on Hop right-preconditioned by the cycle; all columns
   batched, each with its own Arnoldi process.  use_x0 != 0 starts from the
   X passed in (a restarted solve continued over several calls takes the same
   iterates as one call), else from zero.  Returns restart cycles run. */
int slmg_solve(void* h, int64_t hn, const int64_t* hp, const int64_t* hi, const double* hd, const double* Bd,
               double* Xd, int nrhs, int restart, double tol, int max_outer, double w, int pre, int post, int wcycle,
               int relax, int gmres_from, int32_t* iters_out, double* relres_out, int use_x0) {
  slmg_t* S = (slmg_t*)h;
  const csr_t Hop = {hn, hn, hp, hi, (const cplx*)hd};
  const int64_t n = hn;
  const int m = restart;
  const cplx* B = (const cplx*)Bd;
  cplx* X = (cplx*)Xd;
  if (relax == 1 && (pre > 64 || post > 64)) return -1;
  const cyc_t cp = {w, pre, post, wcycle, relax, gmres_from};
  if (!use_x0) memset(X, 0, sizeof(cplx) * (size_t)n * nrhs);
  double* bn = (double*)calloc((size_t)nrhs, sizeof(double));
  int* conv = (int*)calloc((size_t)nrhs, sizeof(int));
  for (int c = 0; c < nrhs; ++c) {
    bn[c] = col_norm(B + (int64_t)c * n, n);
    conv[c] = bn[c] == 0;
    iters_out[c] = 0;
    relres_out[c] = 0;
  }
  cplx* Rr = (cplx*)malloc(sizeof(cplx) * (size_t)n * nrhs);
  memcpy(Rr, B, sizeof(cplx) * (size_t)n * nrhs);
  if (use_x0) {
    for (int c = 0; c < nrhs; ++c) {
      if (conv[c]) continue;
      cplx* r = Rr + (int64_t)c * n;
      const cplx* b = B + (int64_t)c * n;
      spmm(&Hop, X + (int64_t)c * n, n, r, n, 1, 0, 1.0);
#pragma omp parallel for schedule(static)
      for (int64_t p = 0; p < n; ++p) r[p] = b[p] - r[p];
      relres_out[c] = col_norm(r, n) / bn[c];
      if (relres_out[c] <= tol) conv[c] = 1;
    }
  }
  int* cols = (int*)malloc(sizeof(int) * (size_t)nrhs);
  cplx* V = (cplx*)malloc(sizeof(cplx) * (size_t)(m + 1) * n * nrhs);
  cplx* Z = (cplx*)malloc(sizeof(cplx) * (size_t)m * n * nrhs);
  cplx* Wk = (cplx*)malloc(sizeof(cplx) * (size_t)n * nrhs);
  cplx* Hh = (cplx*)calloc((size_t)(m + 1) * m * nrhs, sizeof(cplx));
  cplx* cs = (cplx*)calloc((size_t)m * nrhs, sizeof(cplx));
  cplx* sn = (cplx*)calloc((size_t)m * nrhs, sizeof(cplx));
  cplx* g = (cplx*)calloc((size_t)(m + 1) * nrhs, sizeof(cplx));
  cplx* hv = (cplx*)calloc((size_t)(m + 1) * nrhs, sizeof(cplx));
  int* kcol = (int*)calloc((size_t)nrhs, sizeof(int));
  int* live = (int*)calloc((size_t)nrhs, sizeof(int));
  int outer;
  for (outer = 1; outer <= max_outer; ++outer) {
    int nc = 0;
    for (int c = 0; c < nrhs; ++c)
      if (!conv[c]) cols[nc++] = c;
    if (nc == 0) {
      outer--;
      break;
    }
    /* packed per-active-column storage: block j column q at V + (j*nc + q)*n */
    for (int q = 0; q < nc; ++q) {
      const int c = cols[q];
      const cplx* r = Rr + (int64_t)c * n;
      double beta = col_norm(r, n);
      cplx* v0 = V + (int64_t)q * n;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) v0[i] = r[i] / beta;
      for (int i = 0; i <= m; ++i) g[q * (m + 1) + i] = 0;
      g[q * (m + 1)] = beta;
      kcol[q] = 0;
      live[q] = 1;
    }
    for (int j = 0; j < m; ++j) {
      int nl = 0;
      for (int q = 0; q < nc; ++q) nl += live[q];
      if (nl == 0) break;
      /* gather live columns of V_j, precondition, apply H */
      int* lq = (int*)malloc(sizeof(int) * (size_t)nl);
      int t = 0;
      for (int q = 0; q < nc; ++q)
        if (live[q]) lq[t++] = q;
      cplx* vin = (cplx*)malloc(sizeof(cplx) * (size_t)n * nl);
      cplx* zout = (cplx*)malloc(sizeof(cplx) * (size_t)n * nl);
      for (int a = 0; a < nl; ++a) memcpy(vin + (int64_t)a * n, V + ((int64_t)j * nc + lq[a]) * n, sizeof(cplx) * n);
      mg_cycle(S, 0, vin, zout, nl, &cp);
      for (int a = 0; a < nl; ++a) memcpy(Z + ((int64_t)j * nc + lq[a]) * n, zout + (int64_t)a * n, sizeof(cplx) * n);
      spmm(&Hop, zout, n, Wk, n, nl, 0, 1.0);
      for (int a = 0; a < nl; ++a) {
        const int q = lq[a];
        cplx* wv = Wk + (int64_t)a * n;
        for (int i = 0; i <= j; ++i) hv[q * (m + 1) + i] = 0;
        double before = col_norm(wv, n);
        before *= before;
        for (int pass = 0; pass < 2; ++pass) {
          cplx hh[64];
          for (int i = 0; i <= j; ++i) {
            const cplx* vi = V + ((int64_t)i * nc + q) * n;
            double sr = 0, si = 0;
#pragma omp parallel for reduction(+ : sr, si) schedule(static)
            for (int64_t p = 0; p < n; ++p) {
              cplx z = conj(vi[p]) * wv[p];
              sr += creal(z);
              si += cimag(z);
            }
            hh[i] = sr + I * si;
          }
#pragma omp parallel for schedule(static)
          for (int64_t p = 0; p < n; ++p) {
            cplx s = wv[p];
            for (int i = 0; i <= j; ++i) s -= hh[i] * V[((int64_t)i * nc + q) * n + p];
            wv[p] = s;
          }
          for (int i = 0; i <= j; ++i) hv[q * (m + 1) + i] += hh[i];
          if (pass == 0) {
            double after = col_norm(wv, n);
            if (!(after * after < 0.5 * before)) break; /* DGKS: second pass not needed */
          }
        }
        double hnrm = col_norm(wv, n);
        cplx* vn = V + ((int64_t)(j + 1) * nc + q) * n;
        double sc = hnrm > 0 ? 1.0 / hnrm : 1.0;
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; ++p) vn[p] = wv[p] * sc;
        cplx col[66];
        for (int i = 0; i <= j; ++i) col[i] = hv[q * (m + 1) + i];
        col[j + 1] = hnrm;
        for (int i = 0; i < j; ++i) {
          cplx ci = cs[q * m + i], si = sn[q * m + i];
          cplx tt = conj(ci) * col[i] + conj(si) * col[i + 1];
          col[i + 1] = -si * col[i] + ci * col[i + 1];
          col[i] = tt;
        }
        cplx a0 = col[j], b0 = col[j + 1];
        double den = sqrt(creal(a0) * creal(a0) + cimag(a0) * cimag(a0) + creal(b0) * creal(b0) +
                          cimag(b0) * cimag(b0));
        cplx cj = 1, sj = 0;
        if (den > 0) {
          cj = a0 / den;
          sj = b0 / den;
        }
        cs[q * m + j] = cj;
        sn[q * m + j] = sj;
        col[j] = den;
        col[j + 1] = 0;
        for (int i = 0; i <= j + 1; ++i) Hh[((int64_t)q * m + j) * (m + 1) + i] = col[i];
        cplx gj = g[q * (m + 1) + j];
        g[q * (m + 1) + j] = conj(cj) * gj;
        g[q * (m + 1) + j + 1] = -sj * gj;
        kcol[q] = j + 1;
        iters_out[cols[q]] += 1;
        if (cabs(g[q * (m + 1) + j + 1]) / bn[cols[q]] <= tol) live[q] = 0;
      }
      free(lq);
      free(vin);
      free(zout);
    }
    /* x += Z y per column */
    for (int q = 0; q < nc; ++q) {
      const int k = kcol[q], c = cols[q];
      cplx y[64];
      for (int i = k - 1; i >= 0; --i) {
        cplx s = g[q * (m + 1) + i];
        for (int l2 = i + 1; l2 < k; ++l2) s -= Hh[((int64_t)q * m + l2) * (m + 1) + i] * y[l2];
        y[i] = s / Hh[((int64_t)q * m + i) * (m + 1) + i];
      }
      cplx* xc = X + (int64_t)c * n;
#pragma omp parallel for schedule(static)
      for (int64_t p = 0; p < n; ++p) {
        cplx s = xc[p];
        for (int i = 0; i < k; ++i) s += y[i] * Z[((int64_t)i * nc + q) * n + p];
        xc[p] = s;
      }
    }
    /* true residual of the active columns */
    for (int q = 0; q < nc; ++q) {
      const int c = cols[q];
      spmm(&Hop, X + (int64_t)c * n, n, Rr + (int64_t)c * n, n, 1, 0, 1.0);
      cplx* r = Rr + (int64_t)c * n;
      const cplx* b = B + (int64_t)c * n;
#pragma omp parallel for schedule(static)
      for (int64_t p = 0; p < n; ++p) r[p] = b[p] - r[p];
      relres_out[c] = col_norm(r, n) / bn[c];
      if (relres_out[c] <= tol) conv[c] = 1;
    }
  }
  if (outer > max_outer) outer = max_outer;
  free(bn);
  free(conv);
  free(Rr);
  free(cols);
  free(V);
  free(Z);
  free(Wk);
  free(Hh);
  free(cs);
  free(sn);
  free(g);
  free(hv);
  free(kcol);
  free(live);
  return outer;
}
