// Generic strided, batched GEMM on the CUDA cores (FP64 and FP32).
//
// C(m,n) = alpha * sum_k A(m,k) B(k,n) + beta * C(m,n), every operand addressed
// by explicit element strides, with two batch levels.  This is the contraction
// engine of the plain-FP64 path (the reference does every contraction of the
// response in FP64 BLAS: src/ri_jk/hess_r.rs:131-176, src/hessian/rscf.rs:212-216,
// src/util/krylov_block.rs:121-122, 207-214) and of the FP32 mid-size
// contractions of the mixed path.
//
// On GB300 the FP64 pipe retires about two DFMA per clock per SM, so an FP64
// tile of 64x64x16 needs ~32k clocks of arithmetic for 16 KB of operands: any
// reasonable tiling is bound by the FP64 pipe, and the design only has to keep
// all 152 SMs busy (split-K for narrow outputs) and stay deterministic.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cphf {

struct GemmDesc {
  int64_t M = 0, N = 0, K = 0;
  const void* A = nullptr;
  int64_t a_m = 0, a_k = 0;  // A(m,k) at A[m*a_m + k*a_k]
  const void* B = nullptr;
  int64_t b_k = 0, b_n = 0;  // B(k,n) at B[k*b_k + n*b_n]
  void* C = nullptr;
  int64_t c_m = 0, c_n = 0;  // C(m,n) at C[m*c_m + n*c_n]
  int64_t batch1 = 1, batch2 = 1;
  int64_t a_b1 = 0, a_b2 = 0, b_b1 = 0, b_b2 = 0, c_b1 = 0, c_b2 = 0;
  double alpha = 1.0, beta = 0.0;
  // Optional two-level row / column index: with m_div > 0, row m = m0 + m_div * m1 sits at
  // m0 * a_m + m1 * a_m2 in A and m0 * c_m + m1 * c_m2 in C (likewise n_div for B and C
  // columns).  Lets a batch of narrow GEMMs run as one tall GEMM.
  int64_t m_div = 0, a_m2 = 0, c_m2 = 0;
  int64_t n_div = 0, b_n2 = 0, c_n2 = 0;
};

enum class Prec { F64, F32 };

// Types: A and B are read as TA/TB and converted to the compute type; C is
// written as TC.  Supported combinations are instantiated in gemm_simt.cu.
// `workspace` (bytes `ws_bytes`) is used for split-K partial sums; pass
// nullptr to disable split-K.  Returns cudaSuccess or the launch error.
template <typename TCompute, typename TA, typename TB, typename TC>
cudaError_t gemm(const GemmDesc& d, cudaStream_t stream, void* workspace = nullptr,
                 size_t ws_bytes = 0, int num_sms = 152);

// Workspace bytes that gemm<> may use for split-K on descriptor d.
size_t gemm_workspace_bytes(const GemmDesc& d, size_t elem_bytes, int num_sms = 152);

// FP64 operands and result, products and sums in double-float arithmetic on the FP32 pipes
// (about 2^-46 relative per term; GB300 runs FP32 ~60x faster than FP64).
cudaError_t gemm_f64_emulated(const GemmDesc& d, cudaStream_t stream, void* workspace = nullptr,
                              size_t ws_bytes = 0, int num_sms = 152);

}  // namespace cphf
