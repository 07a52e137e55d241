// Host-side discretisation helpers of the C ABI and the banded LU
// factorisation of the coarsest multigrid level.
//
// hz_abl / hz_sommerfeld / hz_helmholtz_mass / hz_max_frequency /
// hz_point_source restate src/GetHelmholtz.jl:41-47,75-79,97-247 and
// src/getPointSource.jl:63-111 (setup work, O(N), run once per problem).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "../../include/helmgpu.h"
#include "hz_host.h"

using cd = std::complex<double>;

extern "C" double hz_max_frequency(const double* m, int64_t count, const double* h, int32_t dim) {
  if (!m || !h || count <= 0 || dim < 1 || dim > 3) return -1.0;
  double hmax = h[0];
  for (int d = 1; d < dim; ++d) hmax = std::max(hmax, h[d]);
  double mmax = m[0];
  for (int64_t i = 1; i < count; ++i) mmax = std::max(mmax, m[i]);
  return (0.1 * 2.0 * M_PI) / (hmax * std::sqrt(mmax));
}

extern "C" int hz_abl(int32_t dim, const int64_t* nodes, int32_t neumann, const int64_t* pad, double amp,
                      double* gamma) {
  if (!nodes || !pad || !gamma || (dim != 2 && dim != 3)) return HZ_ERR_ARG;
  for (int d = 0; d < dim; ++d)
    if (nodes[d] < 2 || pad[d] < 1 || pad[d] > nodes[d]) return HZ_ERR_ARG;
  if (dim == 2) {
    // quadratic sponge on the sides and bottom (and top unless Neumann);
    // overlapping corners combine as a + b - a*b
    const int64_t n1 = nodes[0], n2 = nodes[1], p1 = pad[0], p2 = pad[1];
    std::vector<double> g((size_t)(n1 * n2), 0.0);
    auto G = [&](int64_t i, int64_t j) -> double& { return g[(size_t)(i + n1 * j)]; };
    auto bwd = [](int64_t k, int64_t p) { double v = (double)(p - k); return v * v / (double)(p * p); };  // k=0..p-1
    auto fwd = [](int64_t k, int64_t p) { double v = (double)(k + 1); return v * v / (double)(p * p); };
    const int64_t I1 = n1 - p1, I2 = n2 - p2;
    if (!neumann) {
      for (int64_t j = 0; j < p2; ++j)
        for (int64_t i = 0; i < n1; ++i) G(i, j) += bwd(j, p2);
      for (int64_t j = 0; j < p2; ++j)
        for (int64_t i = 0; i < p1; ++i) G(i, j) -= bwd(i, p1) * bwd(j, p2);
      for (int64_t j = 0; j < p2; ++j)
        for (int64_t i = 0; i < p1; ++i) G(I1 + i, j) -= fwd(i, p1) * bwd(j, p2);
    }
    for (int64_t j = 0; j < p2; ++j)
      for (int64_t i = 0; i < n1; ++i) G(i, I2 + j) += fwd(j, p2);
    for (int64_t j = 0; j < n2; ++j)
      for (int64_t i = 0; i < p1; ++i) G(i, j) += bwd(i, p1);
    for (int64_t j = 0; j < n2; ++j)
      for (int64_t i = 0; i < p1; ++i) G(I1 + i, j) += fwd(i, p1);
    for (int64_t j = 0; j < p2; ++j)
      for (int64_t i = 0; i < p1; ++i) G(i, I2 + j) -= bwd(i, p1) * fwd(j, p2);
    for (int64_t j = 0; j < p2; ++j)
      for (int64_t i = 0; i < p1; ++i) G(I1 + i, I2 + j) -= fwd(i, p1) * fwd(j, p2);
    for (size_t q = 0; q < g.size(); ++q) gamma[q] = g[q] * amp;
    return HZ_OK;
  }
  // 3D: normalised squared distance into each layer, summed over the axes,
  // scaled by amp and clipped at amp
  std::vector<double> prof[3];
  for (int d = 0; d < 3; ++d) {
    const int64_t n = nodes[d], p = pad[d];
    const double lo = (d == 2) ? 0.0 : -1.0, hi = 1.0;
    auto x = [&](int64_t k) { return lo + (hi - lo) * (double)k / (double)(n - 1); };
    const bool left = !(d == 2 && neumann);
    std::vector<double> g((size_t)n, 0.0);
    if (left)
      for (int64_t k = 0; k < p; ++k) g[(size_t)k] += (x(k) - x(p - 1)) * (x(k) - x(p - 1));
    for (int64_t k = n - p; k < n; ++k) g[(size_t)k] += (x(k) - x(n - p)) * (x(k) - x(n - p));
    double mx = 0.0;
    for (double v : g) mx = std::max(mx, v);
    for (double& v : g) v /= (mx + 1e-5);
    prof[d] = g;
  }
  const int64_t n1 = nodes[0], n2 = nodes[1], n3 = nodes[2];
  for (int64_t k = 0; k < n3; ++k)
    for (int64_t j = 0; j < n2; ++j)
      for (int64_t i = 0; i < n1; ++i) {
        double v = (prof[0][(size_t)i] + prof[1][(size_t)j] + prof[2][(size_t)k]) * amp;
        if (v >= amp) v = amp;
        gamma[i + n1 * (j + n2 * k)] = v;
      }
  return HZ_OK;
}

extern "C" int hz_sommerfeld(int32_t dim, const int64_t* n, const double* h, const double* m, double omega,
                             int32_t neumann_on_top, int32_t order_bc, double* somm) {
  if (!n || !h || !m || !somm || (dim != 2 && dim != 3)) return HZ_ERR_ARG;
  const double BC = (order_bc == 1) ? 1.0 : 2.0;
  const int64_t n1 = n[0] + 1, n2 = n[1] + 1, n3 = (dim == 3) ? n[2] + 1 : 1;
  const int64_t N = n1 * n2 * n3;
  cd* S = reinterpret_cast<cd*>(somm);
  for (int64_t p = 0; p < N; ++p) S[p] = 0.0;
  const cd c(0.0, -omega * BC);
  auto add = [&](int64_t i, int64_t j, int64_t k, double hd) {
    const int64_t p = i + n1 * (j + n2 * k);
    S[p] += (c / hd) * std::sqrt(m[p]);
  };
  if (dim == 2) {
    if (!neumann_on_top)
      for (int64_t i = 0; i < n1; ++i) add(i, 0, 0, h[1]);
    for (int64_t i = 0; i < n1; ++i) add(i, n2 - 1, 0, h[1]);
    for (int64_t j = 0; j < n2; ++j) add(n1 - 1, j, 0, h[0]);
    for (int64_t j = 0; j < n2; ++j) add(0, j, 0, h[0]);
  } else {
    if (!neumann_on_top)
      for (int64_t j = 0; j < n2; ++j)
        for (int64_t i = 0; i < n1; ++i) add(i, j, 0, h[2]);
    for (int64_t j = 0; j < n2; ++j)
      for (int64_t i = 0; i < n1; ++i) add(i, j, n3 - 1, h[2]);
    for (int64_t k = 0; k < n3; ++k)
      for (int64_t i = 0; i < n1; ++i) add(i, 0, k, h[1]);
    for (int64_t k = 0; k < n3; ++k)
      for (int64_t i = 0; i < n1; ++i) add(i, n2 - 1, k, h[1]);
    for (int64_t k = 0; k < n3; ++k)
      for (int64_t j = 0; j < n2; ++j) add(0, j, k, h[0]);
    for (int64_t k = 0; k < n3; ++k)
      for (int64_t j = 0; j < n2; ++j) add(n1 - 1, j, k, h[0]);
  }
  return HZ_OK;
}

extern "C" int hz_helmholtz_mass(const hz_problem* pr, double* mass_out) {
  if (!pr || !mass_out || !pr->m || !pr->gamma || (pr->dim != 2 && pr->dim != 3)) return HZ_ERR_ARG;
  if (pr->omega_re == 0.0) return HZ_ERR_ARG;
  int64_t N = 1;
  for (int d = 0; d < pr->dim; ++d) N *= (pr->n[d] + 1);
  const cd w(pr->omega_re, pr->omega_im);
  const cd w2 = w * w;
  cd* M = reinterpret_cast<cd*>(mass_out);
  for (int64_t p = 0; p < N; ++p)
    M[p] = -w2 * pr->m[p] * cd(1.0, -pr->gamma[p] / pr->omega_re);
  if (pr->sommerfeld) {
    // src/GetHelmholtz.jl:45 calls getSommerfeldBC without orderNeumannBC, so the
    // boundary factor is its default BC = 2 (:222) whatever order the Laplacian uses
    std::vector<double> s((size_t)(2 * N));
    int st = hz_sommerfeld(pr->dim, pr->n, pr->h, pr->m, pr->omega_re, pr->neumann_on_top, 2, s.data());
    if (st != HZ_OK) return st;
    const cd* S = reinterpret_cast<const cd*>(s.data());
    for (int64_t p = 0; p < N; ++p) M[p] -= S[p];
  }
  return HZ_OK;
}

extern "C" int hz_point_source(int32_t dim, const int64_t* n, const double* h, const int64_t* src, double* q) {
  if (!n || !h || !src || !q || (dim != 2 && dim != 3)) return HZ_ERR_ARG;
  int64_t nn[3] = {n[0] + 1, n[1] + 1, dim == 3 ? n[2] + 1 : 1};
  int64_t N = nn[0] * nn[1] * nn[2];
  for (int d = 0; d < dim; ++d)
    if (src[d] < 1 || src[d] > nn[d]) return HZ_ERR_ARG;
  std::memset(q, 0, sizeof(double) * 2 * (size_t)N);
  int64_t cs = src[0] + (src[1] - 1) * nn[0];
  if (dim == 3) cs += (src[2] - 1) * nn[0] * nn[1];
  // 1 / norm(h)^2, the norm taken first as the reference writes it
  double hn2 = 0.0;
  for (int d = 0; d < dim; ++d) hn2 += h[d] * h[d];
  const double nrm = std::sqrt(hn2);
  q[2 * (cs - 1)] = 1.0 / (nrm * nrm);
  return HZ_OK;
}

namespace hz {

// Complex banded LU with partial pivoting, the unblocked LAPACK zgbtf2
// algorithm: ab is column-major with ldab = 2*kl + ku + 1 and A(i, j) at
// ab[j*ldab + kl + ku + i - j]; on return it holds U (kl + ku superdiagonals)
// and the multipliers of L below the diagonal, ipiv the 0-based pivot rows.
int band_lu_factor(long long N, int kl, int ku, std::complex<double>* ab, int* ipiv) {
  const long long ldab = 2LL * kl + ku + 1;
  const int kv = kl + ku;
  auto A = [&](long long i, long long j) -> cd& { return ab[j * ldab + kv + i - j]; };
  long long ju = 0;
  int info = 0;
  for (long long j = 0; j < N; ++j) {
    const int km = (int)std::min<long long>(kl, N - 1 - j);
    int jp = 0;
    double best = -1.0;
    for (int r = 0; r <= km; ++r) {
      const cd v = A(j + r, j);
      const double mag = std::fabs(v.real()) + std::fabs(v.imag());
      if (mag > best) {
        best = mag;
        jp = r;
      }
    }
    ipiv[j] = (int)(j + jp);
    if (best == 0.0) {
      if (!info) info = (int)j + 1;
      continue;
    }
    ju = std::max(ju, std::min<long long>(j + ku + jp, N - 1));
    if (jp != 0)
      for (long long c = j; c <= ju; ++c) std::swap(A(j, c), A(j + jp, c));
    if (km > 0) {
      const cd inv = 1.0 / A(j, j);
      for (int r = 1; r <= km; ++r) A(j + r, j) *= inv;
      const long long c0 = j + 1, c1 = ju;
#pragma omp parallel for schedule(static) if ((c1 - c0 + 1) * km > 16384)
      for (long long c = c0; c <= c1; ++c) {
        const cd ajc = A(j, c);
        if (ajc != 0.0)
          for (int r = 1; r <= km; ++r) A(j + r, c) -= A(j + r, j) * ajc;
      }
    }
  }
  return info;
}

}  // namespace hz

namespace hz {

// Block operators of the banded solve.  For block I (rows s..e, nb rows):
//  forward:  the elimination steps s..e of gbtrs (row interchange, then
//            rows j+1..j+kl -= L(.,j) v_j) touch only rows s .. e+kl, so their
//            composition is one dense W x W matrix T_I (W = min(nb+kl, N-s))
//            applied to that window;
//  backward: x_I = U_II^{-1} (y_I - U_{I,right} x_right), stored as
//            G_I = [U_II^{-1} | -U_II^{-1} U_{I,right}] (nb x Wb, Wb = min(nb+kv, N-s)).
// Both are row-major.  ab must hold the factors with the true U diagonal.
void band_block_operators(long long N, int kl, int ku, const std::complex<double>* ab, const int* ipiv, int nb,
                          std::vector<BandBlock>& blocks, std::vector<std::complex<double>>& T,
                          std::vector<std::complex<double>>& G) {
  const long long ldab = 2LL * kl + ku + 1;
  const int kv = kl + ku;
  auto A = [&](long long i, long long j) -> cd { return ab[j * ldab + kv + i - j]; };
  const long long nbk = (N + nb - 1) / nb;
  blocks.resize((size_t)nbk);
  long long toff = 0, goff = 0;
  for (long long I = 0; I < nbk; ++I) {
    BandBlock& B = blocks[(size_t)I];
    B.s = I * nb;
    B.nb = (int)std::min<long long>(nb, N - B.s);
    B.W = (int)std::min<long long>((long long)nb + kl, N - B.s);
    B.Wb = (int)std::min<long long>((long long)B.nb + kv, N - B.s);
    B.toff = toff;
    B.goff = goff;
    toff += (long long)B.W * B.W;
    goff += (long long)B.nb * B.Wb;
  }
  T.assign((size_t)toff, cd(0.0));
  G.assign((size_t)goff, cd(0.0));
#pragma omp parallel for schedule(dynamic)
  for (long long I = 0; I < nbk; ++I) {
    const BandBlock& B = blocks[(size_t)I];
    const int W = B.W;
    cd* t = T.data() + B.toff;
    for (int i = 0; i < W; ++i) t[(size_t)i * W + i] = 1.0;
    const long long jend = std::min<long long>(B.s + B.nb - 1, N - 2);
    for (long long j = B.s; j <= jend; ++j) {
      const int lm = (int)std::min<long long>(kl, N - 1 - j);
      const int rj = (int)(j - B.s);
      const int rl = (int)(ipiv[j] - B.s);
      if (rl != rj)
        for (int c = 0; c < W; ++c) std::swap(t[(size_t)rj * W + c], t[(size_t)rl * W + c]);
      for (int r = 1; r <= lm; ++r) {
        const cd l = A(j + r, j);
        if (l == 0.0) continue;
        cd* dst = t + (size_t)(rj + r) * W;
        const cd* src = t + (size_t)rj * W;
        for (int c = 0; c < W; ++c) dst[c] -= l * src[c];
      }
    }
    // backward operator
    const int n = B.nb, Wb = B.Wb;
    std::vector<cd> inv((size_t)n * n, 0.0);  // U_II^{-1}, row-major upper triangular
    for (int col = n - 1; col >= 0; --col) {
      // solve U_II z = e_col by back substitution (z has entries 0..col)
      inv[(size_t)col * n + col] = 1.0 / A(B.s + col, B.s + col);
      for (int i = col - 1; i >= 0; --i) {
        cd acc = 0.0;
        const int kmax = std::min(col, i + kv);
        for (int k = i + 1; k <= kmax; ++k) acc += A(B.s + i, B.s + k) * inv[(size_t)k * n + col];
        inv[(size_t)i * n + col] = -acc / A(B.s + i, B.s + i);
      }
    }
    cd* g = G.data() + B.goff;
    for (int i = 0; i < n; ++i)
      for (int k = i; k < n; ++k) g[(size_t)i * Wb + k] = inv[(size_t)i * n + k];
    // -U_II^{-1} U_right, U_right(k, c) = U(s+k, s+n+c) for c < Wb - n
    for (int i = 0; i < n; ++i) {
      for (int c = 0; c < Wb - n; ++c) {
        const long long gc = B.s + n + c;
        cd acc = 0.0;
        const int kmin = (int)std::max<long long>(i, gc - kv - B.s);  // U(s+k, gc) = 0 for gc-(s+k) > kv
        for (int k = kmin; k < n; ++k) acc += inv[(size_t)i * n + k] * A(B.s + k, gc);
        g[(size_t)i * Wb + n + c] = -acc;
      }
    }
  }
}

}  // namespace hz
