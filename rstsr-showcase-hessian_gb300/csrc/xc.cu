// XC (fxc) response in bra form, RHO / LDA branch, over uneven grid batches (FP64 path).
//
// Reference: get_rks_response_bra(_batched) (src/numint_matmul/hess_rks.rs:570-605, 752-797),
// get_rho_from_one_bra_mult_ket_with_output (pure_eval_rho.rs:216-334, RHO terms 283-287),
// rks_fxc_pot_with_eff_bra_trans_with_output + contract_ao_wv_bra (pure_xcpot.rs:285-465),
// get_uks_response_bra (hess_uks.rs:390-441) with uks_fxc_pot_with_eff_bra_trans_with_output
// (pure_xcpot.rs:921-1028).
//
// Per grid batch b (e.g. one atom's points) only the AO window [lo, lo+nwin) with
// non-zero values is stored and contracted:
//   ket[g,(i,a)]  = sum_mu phi_b[g,mu] bra[lo+mu,(i,a)]
//   rho1[g,a]     = sum_i aobra[g,i] ket[g,i,a]            (aobra = phi Cocc, once per preparation)
//   wv_s[g,a]     = w_g sum_t fxc[g,t,s] rho1_t[g,a]
//   out_s[lo+mu,(i,a)] += fac * sum_g phi_b[g,mu] wv_s[g,a] aobra_s[g,i]   (fac 4 RKS, 2 UKS)
#include <algorithm>

#include "ctx.cuh"
#include "kernels.cuh"

namespace cphf {

void xc_prepare(cphf_ctx* c) {
  for (int s = 0; s < c->nspin; ++s) {
    SpinState& sp = c->spin[s];
    const int64_t no = sp.nocc;
    sp.aobra.ensure((size_t)c->ngrids * std::max<int64_t>(no, 1) * 8, c->counter());
    if (no == 0) continue;
    for (const XcBatch& b : c->xc_batches) {
      if (b.npts == 0) continue;
      if (b.nwin == 0) {
        CPHF_CUDA(cudaMemset2DAsync(sp.aobra.as<double>() + b.g0, c->ngrids * 8, 0, b.npts * 8, no, c->stream));
        continue;
      }
      GemmDesc d;
      d.M = b.npts; d.N = no; d.K = b.nwin;
      d.A = c->phi.as<double>() + b.phi_off; d.a_m = 1; d.a_k = b.npts;
      d.B = sp.C.as<double>() + b.lo; d.b_k = 1; d.b_n = c->nao;
      d.C = sp.aobra.as<double>() + b.g0; d.c_m = 1; d.c_n = c->ngrids;
      gemm64(c, d);
    }
  }
}

void xc_response_fp64(cphf_ctx* c, const double* const* bra, int64_t nb, double* const* out,
                      bool accumulate) {
  const int ns = c->nspin;
  const int64_t nao = c->nao;
  if (!accumulate) {
    for (int s = 0; s < ns; ++s)
      if (c->spin[s].nocc > 0)
        CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * 8, c->stream));
  }
  int64_t max_pts = 0;
  for (const XcBatch& b : c->xc_batches) max_pts = std::max(max_pts, b.npts);
  int64_t ket_per_spin = 0;
  for (int s = 0; s < ns; ++s) ket_per_spin = std::max(ket_per_spin, max_pts * c->spin[s].nocc * nb);
  c->s_ket.ensure((size_t)std::max<int64_t>(1, ket_per_spin * ns) * 8, c->counter());
  c->s_rho.ensure((size_t)std::max<int64_t>(1, max_pts * nb * 2) * 8, c->counter());
  const double fac = ns == 1 ? 4.0 : 2.0;  // hess_rks.rs:603, hess_uks.rs:438-439
  double* ket = c->s_ket.as<double>();
  double* rho = c->s_rho.as<double>();
  for (const XcBatch& b : c->xc_batches) {
    if (b.npts == 0 || b.nwin == 0) continue;
    const double* phi = c->phi.as<double>() + b.phi_off;
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      double* ket_s = ket + s * ket_per_spin;
      double* rho_s = rho + s * b.npts * nb;
      if (no == 0) {
        CPHF_CUDA(cudaMemsetAsync(rho_s, 0, (size_t)b.npts * nb * 8, c->stream));
        continue;
      }
      GemmDesc d;
      d.M = b.npts; d.N = no * nb; d.K = b.nwin;
      d.A = phi; d.a_m = 1; d.a_k = b.npts;
      d.B = bra[s] + b.lo; d.b_k = 1; d.b_n = nao;
      d.C = ket_s; d.c_m = 1; d.c_n = b.npts;
      gemm64(c, d);
      launch_xc_rho(c->spin[s].aobra.as<double>() + b.g0, c->ngrids, ket_s, b.npts, no, nb, rho_s,
                    b.npts, c->stream);
    }
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      if (no == 0) continue;
      double* ket_s = ket + s * ket_per_spin;
      launch_xc_q(c->spin[s].aobra.as<double>() + b.g0, c->ngrids, c->weights.as<double>() + b.g0,
                  c->fxc.as<double>() + b.g0, c->ngrids, ns, s, rho, b.npts, b.npts * nb, b.npts, no,
                  nb, ket_s, c->stream);
      GemmDesc d;
      d.M = b.nwin; d.N = no * nb; d.K = b.npts;
      d.A = phi; d.a_m = b.npts; d.a_k = 1;
      d.B = ket_s; d.b_k = 1; d.b_n = b.npts;
      d.C = out[s] + b.lo; d.c_m = 1; d.c_n = nao;
      d.alpha = fac; d.beta = 1.0;
      gemm64(c, d);
    }
  }
}

}  // namespace cphf
