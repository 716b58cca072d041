// XC response on the tensor cores over a dense-AO phi (xc_tc.cu).
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// out[s] (+)= fac sum_g phi_g^T (w f rho1 o phi_g Cocc_s) with split-FP16 tcgen05 GEMMs over
// the dense-AO form of phi; bra[s], out[s] FP32 [nao, nocc_s, nb]; fac = 4 (RKS) or 2 (UKS).
void xc_response_tc(cphf_ctx* c, const float* const* bra, int64_t nb, float* const* out, bool accumulate);
// the same with exact BF16 slices (FP64 bra / out, ~2^-34 relative to the row maxima): the XC
// part of the mixed solve's FP64-accurate residual; throws if a bounded pipeline wait expired
void xc_response_tc64(cphf_ctx* c, const double* const* bra, int64_t nb, double* const* out, bool accumulate);

}  // namespace cphf
