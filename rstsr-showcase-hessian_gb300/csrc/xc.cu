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
// The two contractions run as persistent grouped GEMMs over all batches of a chunk
// (xc_grouped.cu).
#include <algorithm>

#include "ctx.cuh"
#include "kernels.cuh"
#include "xc_gga.cuh"
#include "xc_grouped.cuh"
#include "xc_tc.cuh"

namespace cphf {

void xc_prepare(cphf_ctx* c) {
  if (c->xc_den != 0) {
    xc_gga_prepare(c);
    return;
  }
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
  if (c->xc_den != 0) {  // GGA / meta-GGA (double-float GEMMs inside the FP64-accurate residual)
    const double* aob[2] = {c->spin[0].aobG.as<double>(), c->nspin > 1 ? c->spin[1].aobG.as<double>() : nullptr};
    xc_response_gga<double>(c, bra, nb, out, accumulate, c->phiG.as<double>(), aob, c->s_gket, c->s_grho);
    return;
  }
  if (c->oz_xc && c->lowp) {
    xc_response_tc64(c, bra, nb, out, accumulate);
    return;
  }
  const double* aobra[2] = {c->spin[0].aobra.as<double>(), c->nspin > 1 ? c->spin[1].aobra.as<double>() : nullptr};
  xc_response_grouped<double>(c, bra, nb, out, accumulate, c->phi.as<double>(), aobra, c->s_ket, c->s_rho);
}

}  // namespace cphf
