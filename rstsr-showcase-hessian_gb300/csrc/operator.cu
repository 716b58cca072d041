// CPHF operator over the Krylov vector layout (FP64 path).
//
// Reference: response_mo (src/hessian/rscf.rs:210-220, uscf.rs:203-218) and
// response_dimless_cphf (rscf.rs:237-263, uscf.rs:230-265).  The Krylov vector is
// [n, nb] with n = sum_s nmo*nocc_s; spin blocks are stacked alpha first in each
// column (uscf.rs:292-304).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"

namespace cphf {

int64_t krylov_n(const cphf_ctx* c) {
  int64_t n = 0;
  for (int s = 0; s < c->nspin; ++s) n += c->spin[s].nmo * c->spin[s].nocc;
  return n;
}

static int64_t spin_offset(const cphf_ctx* c, int s) {
  return s == 0 ? 0 : c->spin[0].nmo * c->spin[0].nocc;
}

void response_mo_fp64(cphf_ctx* c, const double* x, int64_t nb, double* y, bool dimless) {
  const int ns = c->nspin;
  const int64_t nao = c->nao, n = krylov_n(c);
  int64_t tot_occ = 0, max_occ = 0, max_nmo = 0;
  for (int s = 0; s < ns; ++s) {
    tot_occ += c->spin[s].nocc;
    max_occ = std::max(max_occ, c->spin[s].nocc);
    max_nmo = std::max(max_nmo, c->spin[s].nmo);
  }
  c->s_c1.ensure((size_t)nao * tot_occ * nb * 8, c->counter());
  c->s_resp.ensure((size_t)nao * tot_occ * nb * 8, c->counter());
  c->s_y.ensure((size_t)max_nmo * max_occ * nb * 8, c->counter());
  if (ns == 2) c->s_x.ensure((size_t)n * nb * 8, c->counter());
  double* c1[2] = {nullptr, nullptr};
  double* rb[2] = {nullptr, nullptr};
  const double* xs[2] = {nullptr, nullptr};
  int64_t off_occ = 0;
  for (int s = 0; s < ns; ++s) {
    const SpinState& sp = c->spin[s];
    c1[s] = c->s_c1.as<double>() + nao * off_occ * nb;
    rb[s] = c->s_resp.as<double>() + nao * off_occ * nb;
    off_occ += sp.nocc;
    const int64_t len = sp.nmo * sp.nocc;
    if (ns == 1) {
      xs[s] = x;
    } else {
      double* dst = c->s_x.as<double>() + (s == 0 ? 0 : spin_offset(c, 1) * nb);
      if (len > 0)
        CPHF_CUDA(cudaMemcpy2DAsync(dst, len * 8, x + spin_offset(c, s), n * 8, len * 8, nb,
                                    cudaMemcpyDeviceToDevice, c->stream));
      xs[s] = dst;
    }
    if (sp.nocc == 0) continue;
    GemmDesc d;  // ubra = C mo1  (rscf.rs:212)
    d.M = nao; d.N = sp.nocc * nb; d.K = sp.nmo;
    d.A = sp.C.p; d.a_m = 1; d.a_k = nao;
    d.B = xs[s]; d.b_k = 1; d.b_n = sp.nmo;
    d.C = c1[s]; d.c_m = 1; d.c_n = nao;
    gemm64(c, d);
  }
  bool acc = false;
  if (c->has_rijk) {
    rijk_response_fp64(c, c1, nb, rb, acc);
    acc = true;
  }
  if (c->has_xc) {
    xc_response_fp64(c, c1, nb, rb, acc);
    acc = true;
  }
  if (!acc) {
    for (int s = 0; s < ns; ++s)
      CPHF_CUDA(cudaMemsetAsync(rb[s], 0, (size_t)nao * c->spin[s].nocc * nb * 8, c->stream));
  }
  for (int s = 0; s < ns; ++s) {
    const SpinState& sp = c->spin[s];
    const int64_t no = sp.nocc, nmo = sp.nmo;
    const int64_t r0 = dimless ? no : 0;  // only virtual rows survive the dimensionless epilogue
    const int64_t nrow = nmo - r0;
    double* yo = y + spin_offset(c, s);
    if (no == 0) continue;
    if (nrow > 0) {
      GemmDesc d;  // resp = C^T resp_bra  (rscf.rs:216)
      d.M = nrow; d.N = no * nb; d.K = nao;
      d.A = sp.C.as<double>() + r0 * nao; d.a_m = nao; d.a_k = 1;
      d.B = rb[s]; d.b_k = 1; d.b_n = nao;
      d.C = c->s_y.p; d.c_m = 1; d.c_n = nrow;
      gemm64(c, d);
    }
    if (dimless) {
      launch_dimless(c->s_y.as<double>(), xs[s], ns == 1 ? n : nmo * no, sp.e.as<double>(), nmo, no,
                     nb, c->cfg.level_shift, yo, n, c->stream);
    } else {
      CPHF_CUDA(cudaMemcpy2DAsync(yo, n * 8, c->s_y.p, nmo * no * 8, nmo * no * 8, nb,
                                  cudaMemcpyDeviceToDevice, c->stream));
    }
  }
}

double fp64_residual(cphf_ctx* c, const double* b, const double* x, int64_t nset, double* r,
                     cphf_stats* st) {
  const int64_t n = krylov_n(c);
  c->k_norm.ensure((size_t)(nset + residual_partials_size(n, nset)) * 8, c->counter());
  response_mo_fp64(c, x, nset, r, true);
  if (st) st->fp64_matvec_columns += nset;
  double* norms = c->k_norm.as<double>();
  launch_residual_norms(b, x, r, r, n, nset, norms, norms + nset, c->stream);
  std::vector<double> h(nset);
  CPHF_CUDA(cudaMemcpyAsync(h.data(), norms, nset * 8, cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  double mx = 0.0;
  for (double v : h) mx = std::max(mx, std::sqrt(v));
  for (double v : h)
    if (!std::isfinite(v)) throw Error(CPHF_ERR_NONFINITE, "non-finite residual");
  return mx;
}

}  // namespace cphf
