// Persistent grouped GEMMs of the XC response over uneven grid batches (xc_grouped.cu).
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// One grid batch inside a chunk, as the kernels read it.
struct XcGroupDev {
  int64_t p_local;     // first point of the batch inside the chunk
  int64_t npts;        // points of the batch
  int64_t lo, nwin;    // AO window
  int64_t phi_off;     // element offset of the batch block in phi
  int64_t tile_begin;  // first flat work item of the batch in the first GEMM
};

// XC response (bra form) of all batches, FP64 (T = double) or FP32 (T = float) operands:
// out[s] (+)= fac * sum_g phi_g^T (w f rho1 o phi_g Cocc_s),  fac = 4 (RKS) or 2 (UKS).
template <typename T>
void xc_response_grouped(cphf_ctx* c, const T* const* bra, int64_t nb, T* const* out, bool accumulate,
                         const T* phi, const T* const* aobra, DevBuf& ket_buf, DevBuf& rho_buf);

template <typename T>
void xc_grouped_gemm1(cphf_ctx* c, const XcGroupDev* groups_dev, int ngroups, int64_t total_tiles, const T* phi,
                      const T* bra, int64_t N, int64_t pchunk, T* ket);
template <typename T>
void xc_grouped_gemm2(cphf_ctx* c, const XcGroupDev* groups_dev, int ngroups, const T* phi, const T* q, int64_t N,
                      int64_t pchunk, T* out, double alpha, double beta);
// chunk plan of the grid batches for element size esize and nb columns (cached per width)
XcPlan& xc_plan(cphf_ctx* c, size_t esize, int64_t nb);
int64_t xc_tiles_m(int64_t npts, bool f64);
int64_t xc_tiles_n(int64_t N, bool f64);

}  // namespace cphf
