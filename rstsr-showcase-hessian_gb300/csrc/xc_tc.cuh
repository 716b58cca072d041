// XC response of the split-precision operator on the tensor cores (xc_tc.cu).
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// out[s] (+)= fac sum_g phi_g^T (w f rho1 o phi_g Cocc_s) with split-FP16 tcgen05 GEMMs over
// the dense-AO form of phi; bra[s], out[s] FP32 [nao, nocc_s, nb]; fac = 4 (RKS) or 2 (UKS).
void xc_response_tc(cphf_ctx* c, const float* const* bra, int64_t nb, float* const* out, bool accumulate);

}  // namespace cphf
