// Two-centre metric decomposition and cderi build (decompose.cu): FP64 on the GPU.
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// Scratch of one decomposition (released with the object).
struct DecompWork {
  DevBuf A;     // [naux, naux]: j2c, then its lower Cholesky factor L (lower triangle)
  DevBuf U;     // [naux, naux]: U = L^T (upper, zeros below)
  DevBuf W, V, e;  // eigenvalue fallback: W = A V, V, eigenvalues
  DevBuf inv;   // inverses of the 128-wide diagonal blocks of L
  DevBuf S;     // [n, 128] panel of the triangular solve
  DevBuf flag, info;
  int sweeps = 0;
};

struct J2cDecomp {
  bool fallback = false;  // the eigenvalue-clamping fallback was taken
  int sweeps = 0;         // Jacobi sweeps of the fallback
  double min_diag = 0.0;  // min diag(U) of the returned factor
};

// decomp_j2c_cd(j2c, threshold, Upper) (src/ri_jk/pure_decompose.rs:29-57) for a device j2c
// [naux, naux]: afterwards w.A holds L (j2c = L L^T, lower triangle) and w.U = L^T.
// threshold < 0: no fallback (a failed factorisation is an error).
J2cDecomp j2c_cholesky(cphf_ctx* c, const double* j2c_dev, int64_t naux, double threshold, DecompWork& w);

// solve_by_j2c(j3c, Cd Upper, Right, flip_uplo = false) (pure_decompose.rs:205-252) in place:
// J [n, naux] (col-major, device) <- J U^-1 = J L^-T, with L from j2c_cholesky in w.A.
void solve_by_j2c_right(cphf_ctx* c, double* J, int64_t n, int64_t naux, DecompWork& w);

}  // namespace cphf
