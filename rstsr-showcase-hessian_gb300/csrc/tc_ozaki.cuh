// FP64-accurate RI-K term on the tensor cores (tcgen05, exact BF16 slice products):
//   out[mu, (i,a)] += alpha * sum_P [ B_P bra_a O_P + Z_P (Z_P^T bra_a)^T ][mu, i]
// (src/ri_jk/hess_r.rs:159-176), ~1e-10 relative to sum |A||B| per contraction, for the FP64
// residual of the mixed-precision solve.
#pragma once
#include <cuda_bf16.h>
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
// bra FP64 [nao, nocc_s, nb].  correction_slices 4 / 3: the contractions read slices 0-3 /
// 0-2 only (10 / 6 products, ~2^-23 / ~2^-17 relative to the operands' maxima), for a bra that
// is a small correction; 0: all six (21 products).
void oz_k_terms(cphf_ctx* c, OzState& z, int s, const double* bra, int64_t nb, double alpha, double* out,
                int correction_slices = 0);

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

// A stack of operand planes: plane t holds rows x ld elements at p + t rows ld; columns at
// and beyond kext read as zero (as do rows beyond `rows`).
struct PlaneMat {
  const void* p;
  int64_t rows, ld, kext;
};

// Split-FP16 contraction (hi / lo planes, three products, FP32 accumulation)
//   out[m + ld_out n] += rowscale[m] colscale[n] sum_{k < K} A[a_row0 + m, k] B[n, b_k0 + k]
// with FP32 atomics; b_k0 a multiple of 8.  The K range is split over CTAs in ranges of
// kb_per_cta blocks of 32 (0: as the autotuner finds best); with store and one range per
// tile the values are stored, not accumulated.
void lp_gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0, int64_t M,
             int64_t N, int64_t K, const double* rowscale, const double* colscale, float* out, int64_t ld_out,
             int* err, int kb_per_cta = 0, bool store = false);

// split-FP16 planes [t][r][ld] of FP32 rows r (K elements each, row stride rs); row exponents to e_out
void lp_slice_rows(cphf_ctx* c, const float* src, int64_t rows, int64_t K, int64_t rs, __half* dst, int64_t ld,
                   int* e_out);

// The same contraction reduced to rho1 in its epilogue (the XC response's first grid step):
//   rho[m + ld_rho a] += sum_i ao[m + ld_ao i] sum_k A[a_row0 + m, k] B[n = i + nocc a, b_k0 + k]
// (rowscale / colscale applied as above; rho FP32, accumulated with atomics).
struct RhoEpilogue {
  float* rho;
  const float* ao;
  int64_t ld_rho, ld_ao, nocc;
};
void lp_gemm_rho(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0,
                 int64_t M, int64_t N, int64_t K, const double* rowscale, const double* colscale,
                 const RhoEpilogue& rho, int* err, int kb_per_cta);

// The same contraction on exact BF16 slice planes (six per operand, 21 products, FP64 out,
// K ranges of at most 3072 per CTA so that the leading groups accumulate exactly); row and
// column scales are 2^e of the slicing exponents.
void oz_gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0, int64_t M,
             int64_t N, int64_t K, const double* rowscale, const double* colscale, double* out, int64_t ld_out,
             int* err, int kb_per_cta = 0, bool store = false);
// exact BF16 slice planes [t][r][ld] of FP64 rows r (K elements each, row stride rs); exponents to e_out
void oz_slice_rows(cphf_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, __nv_bfloat16* dst,
                   int64_t ld, int* e_out);
// the same contraction and slicer in correction precision: the leading `slices` (3 or 4) planes,
// the products with t + u < slices
void oz_gemm_corr(cphf_ctx* c, OzState& z, int slices, const PlaneMat& A, int64_t a_row0, const PlaneMat& B,
                  int64_t b_k0, int64_t M, int64_t N, int64_t K, const double* rowscale, const double* colscale,
                  double* out, int64_t ld_out, int* err, int kb_per_cta = 0, bool store = false);
void oz_slice_rows_corr(cphf_ctx* c, int slices, const double* src, int64_t rows, int64_t K, int64_t rs,
                        __nv_bfloat16* dst, int64_t ld, int* e_out);

}  // namespace cphf
