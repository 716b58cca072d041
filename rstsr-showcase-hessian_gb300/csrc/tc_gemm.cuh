// Tensor-core (tcgen05 / TMEM / TMA) split-FP16 contraction of the RI-K term
//   out[mu, (i,a)] += alpha * sum_P sum_nu B_P[mu,nu] T_P[nu,(i,a)],   T_P = bra_a O_P
// (src/ri_jk/hess_r.rs:168-170), with B and T each split into FP16 hi + lo and the three
// products hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory.
#pragma once
#include <cuda_fp16.h>

#include <cstdint>
#include <functional>

#include "ctx.cuh"

namespace cphf {

// true when the tensor-core path can run on the context's device (sm_103 / sm_100 family)
bool tc_available(cphf_ctx* c);
// FP16 hi/lo copies of the dense cderi, rows of length ldk (K-major for the MMA)
void tc_prepare_cderi(cphf_ctx* c, DevBuf& hi, DevBuf& lo, int64_t& ldk);
// T plane generator: FP16 hi / lo planes [Pl][(i,a)][nu] (row stride ldk) of s T_P,
// T_P[nu, (i,a)] = sum_j bra[nu,j,a] O_P[j,i] for P in [P0, P0 + npc), with *mx = max |T| (float
// bits) and scale[0] = s, scale[1] = alpha / (sA s) as launch_t_scale writes them
using TPlanes =
    std::function<void(int64_t P0, int64_t npc, __half* hi, __half* lo, unsigned* mx, float* scale)>;
// out (FP32 [nao, nocc, nb]) += alpha * sum_P B_P T_P with T_P's FP16 planes and scale from
// `tplanes` (alpha enters through scale[1])
void tc_k_term1(cphf_ctx* c, const DevBuf& Bhi, const DevBuf& Blo, int64_t ldk, int64_t nocc, int64_t nb,
                float* out, DevBuf& Thi, DevBuf& Tlo, const TPlanes& tplanes);
// out[m + ld_out n] += rowscale[m] colscale[n] sum_{Pl < npc} sum_{k < K} A_(a_off+Pl)[m, k] B_Pl[n, k]
// over split-FP16 planes (hi / lo, three products) with the term-1 kernel's 256-wide tiles:
// A planes [a_depth][M][ld] per plane array, B planes [npc][N][ld]; FP32 atomics into out;
// `scale` (device, nullable) multiplies every element.
void tc_planes_term(cphf_ctx* c, const __half* a_hi, const __half* a_lo, int64_t a_depth, int64_t a_off,
                    const __half* b_hi, const __half* b_lo, int64_t npc, int64_t M, int64_t N, int64_t K, int64_t ld,
                    const double* rowscale, const double* colscale, float* out, int64_t ld_out, int* err,
                    const float* scale = nullptr);
// W generation as one GEMM over a chunk of aux functions: rows m = j + no a of A (bra's FP16
// planes, K-major, [M][ldk]), columns n = i + no Pl from B rows b_row0 + n (Z's planes, rows
// (i, P)); writes the FP16 hi / lo planes of W * (*wscale) (a power of two) to
// out[j + ldj i + s_a a + s_p Pl], with 2^(e_row[m] + e_col[b_row0 + n] - 28) undoing the
// operands' plane scales.  Offsets must fit 32 bits.
void tc_wgen_planes(cphf_ctx* c, const __half* a_hi, const __half* a_lo, int64_t M, const __half* b_hi,
                    const __half* b_lo, int64_t b_rows, int64_t b_row0, int64_t N, int64_t K, int64_t ldk,
                    const int* e_row, const int* e_col, const float* wscale, int64_t no, int64_t ldj, int64_t s_a,
                    int64_t s_p, __half* out_hi, __half* out_lo, int* err);
// scale[0] = 2^(14 - e) for max |T| = *mx < 2^e, scale[1] = alpha / (sA scale[0])
void launch_t_scale(const unsigned* mx, float sA, float alpha, float* scale, cudaStream_t stream);

}  // namespace cphf
