// Tensor-core split-BF16 K-term contraction (placeholder until the tcgen05 kernel lands).
#include "tc_gemm.cuh"

namespace cphf {

bool tc_available(cphf_ctx*) { return false; }
void tc_prepare_cderi(cphf_ctx*, DevBuf&, DevBuf&, int64_t& ldk) { ldk = 0; }
void tc_k_term1(cphf_ctx*, const DevBuf&, const DevBuf&, int64_t, const float*, const float*, int64_t,
                int64_t, double, float*, DevBuf&, DevBuf&) {
  throw Error(CPHF_ERR_STATE, "tensor-core path unavailable");
}

}  // namespace cphf
