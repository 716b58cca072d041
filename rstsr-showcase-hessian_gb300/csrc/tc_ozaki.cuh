// FP64-accurate RI-K term on the tensor cores (tcgen05, exact BF16 slice products):
//   out[mu, (i,a)] += alpha * sum_P [ B_P bra_a O_P + Z_P (Z_P^T bra_a)^T ][mu, i]
// (src/ri_jk/hess_r.rs:159-176), ~1e-10 relative to sum |A||B| per contraction, for the FP64
// residual of the mixed-precision solve.
#pragma once
#include <cuda_fp16.h>

#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// true when the kernels can run on the context's device (sm_103 / sm_100 family)
bool oz_available(cphf_ctx* c);
// true when every K range fits the exact-accumulation bound (nao, nocc <= 3072)
bool oz_supported(const cphf_ctx* c);
// row-scaled 6-slice BF16 copy of the dense cderi (once per cderi)
void oz_prepare_cderi(cphf_ctx* c, OzState& z);
// out (FP64 [nao, nocc_s, nb], initialised) += alpha * K-term of spin s;
// bra FP64 [nao, nocc_s, nb]
void oz_k_terms(cphf_ctx* c, OzState& z, int s, const double* bra, int64_t nb, double alpha, double* out);

// Split-FP16 (hi/lo, three products, FP32 accumulation) contractions of the K term for the
// inner solves' operator, from the FP32 copies of O and Z:
// per call, the bra planes of spin s (bra FP32 [nao, nocc_s, nb])
void lp_begin(cphf_ctx* c, OzState& z, int s, const float* bra, int64_t nb);
// T[Pl][(i,a)][nu] = sum_j bra[nu,j,a] O_P[j,i] for P in [P0, P0 + npc) as FP16 hi / lo planes
// (row stride ldt) of s T; s from an upper bound of |T| written to *mx (launch_t_scale)
void lp_tgen_planes(cphf_ctx* c, OzState& z, int s, int64_t P0, int64_t npc, int64_t nb, int64_t ldt, __half* hi,
                    __half* lo, unsigned* mx, float* scale, float sA, float alpha, int* err);
// out (FP32 [nao, nocc_s, nb]) += alpha sum_{P in chunk} Z_P (Z_P^T bra)^T
void lp_w_term2(cphf_ctx* c, OzState& z, int s, int64_t P0, int64_t npc, int64_t nb, double alpha, float* out,
                int* err);

}  // namespace cphf
