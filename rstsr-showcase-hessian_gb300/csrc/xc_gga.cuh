// XC response of gradient-dependent functionals (SIGMA / GGA, TAU / meta-GGA), xc_gga.cu.
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

// aobra_c = phi_c Cocc_s, c = 0..3, for every spin (FP64, [ngrids, nocc, 4])
void xc_gga_prepare(cphf_ctx* c);

// out[s] (+)= fac * XC response of bra[s] (fac 4 RKS, 2 UKS); T = double (plain FP64 path and the
// mixed solve's FP64-accurate residual) or float (the mixed solve's inner operator).
// phi [ngrids, nao, 4], aob[s] [ngrids, nocc_s, 4] in T.
template <typename T>
void xc_response_gga(cphf_ctx* c, const T* const* bra, int64_t nb, T* const* out, bool accumulate, const T* phi,
                     const T* const* aob, DevBuf& ket_buf, DevBuf& rho_buf);

}  // namespace cphf
