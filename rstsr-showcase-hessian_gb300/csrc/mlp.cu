// Learned initial guess / preconditioner (per-(i,a)-pair MLP).  Weights are held by the context.
#include <vector>

#include "ctx.cuh"


using namespace cphf;

extern "C" cphf_status cphf_mlp_set_weights(cphf_ctx* c, const float* weights, int64_t nweights) {
  if (!c) return CPHF_ERR_ARG;
  const int64_t expect = 64 * 3 + 64 + 64 * 64 + 64 + 2 * 64 + 2;
  if (!weights || nweights != expect) {
    c->last_error = "MLP weights must hold " + std::to_string(expect) + " floats";
    return CPHF_ERR_SHAPE;
  }
  try {
    cudaSetDevice(c->device);
    if (!c->mlp) c->mlp.reset(new MlpState());
    c->mlp->host.assign(weights, weights + nweights);
    c->mlp->w.ensure(nweights * 4, c->counter());
    CPHF_CUDA(cudaMemcpyAsync(c->mlp->w.p, weights, nweights * 4, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  } catch (const Error& e) {
    c->last_error = e.what();
    return e.status;
  }
  return CPHF_OK;
}
