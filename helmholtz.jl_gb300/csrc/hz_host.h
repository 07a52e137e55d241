// Internal host-side routines shared between hz_host.cpp and the solver.
#pragma once

#include <complex>
#include <vector>

namespace hz {

// One block of the blocked banded solve (see band_block_operators).
struct BandBlock {
  long long s;      // first row
  int nb;           // rows in the block
  int W;            // forward window (rows s .. s+W-1)
  int Wb;           // backward input window (rows s .. s+Wb-1)
  long long toff;   // offset of T_I (W x W) in the forward operator array
  long long goff;   // offset of G_I (nb x Wb) in the backward operator array
};

// Dense block operators of the banded LU solve (forward T_I, backward G_I).
void band_block_operators(long long N, int kl, int ku, const std::complex<double>* ab, const int* ipiv, int nb,
                          std::vector<BandBlock>& blocks, std::vector<std::complex<double>>& T,
                          std::vector<std::complex<double>>& G);

// Complex banded LU with partial pivoting (LAPACK zgbtf2 algorithm, gbtrf
// band layout with ldab = 2*kl + ku + 1).  Returns 0, or j+1 for an exactly
// zero pivot in column j.
int band_lu_factor(long long N, int kl, int ku, std::complex<double>* ab, int* ipiv);

}  // namespace hz
