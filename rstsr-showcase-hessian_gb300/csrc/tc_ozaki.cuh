// FP64-accurate tensor-core contraction of RI-K term 1 (tcgen05, exact BF16 slice products):
//   out[mu, (i,a)] += alpha * sum_P sum_nu B_P[mu,nu] T_P[nu,(i,a)],   T_P = bra_a O_P
// (src/ri_jk/hess_r.rs:168-170), ~1e-10 relative to sum |B||T|, for the FP64 residual of
// the mixed-precision solve.
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// true when the kernel can run on the context's device (sm_103 / sm_100 family)
bool oz_available(cphf_ctx* c);
// row-scaled 6-slice BF16 copy of the dense cderi (once per cderi)
void oz_prepare_cderi(cphf_ctx* c, OzState& z);
// out (FP64 [nao, nocc, nb], initialised) += alpha * sum_P B_P bra O_P;
// bra FP64 [nao, nocc, nb], O64 [nocc, nocc, naux]
void oz_k_term1(cphf_ctx* c, OzState& z, const double* bra, const double* O64, int64_t nocc, int64_t nb,
                double alpha, double* out);

}  // namespace cphf
