// Internal host-side routines shared between hz_host.cpp and the solver.
#pragma once

#include <complex>

namespace hz {

// Complex banded LU with partial pivoting (LAPACK zgbtf2 algorithm, gbtrf
// band layout with ldab = 2*kl + ku + 1).  Returns 0, or j+1 for an exactly
// zero pivot in column j.
int band_lu_factor(long long N, int kl, int ku, std::complex<double>* ab, int* ipiv);

}  // namespace hz
