// RI-J / RI-K response in bra form (FP64 path) and its preparation.
//
// Reference: get_rijk_response_bra_separated (src/ri_jk/hess_r.rs:82-186) with the
// RHF assembly of RHessRIJK::get_response_bra (hess_r.rs:1916-1953) and the UHF
// assembly of UHessRIJK::get_response_bra (src/ri_jk/hess_u.rs:270-313).
//
// The same sums are evaluated in an occupied-factored order that needs one pass
// over the dense cderi per K chunk and never forms AO-basis J or D matrices:
//   Z_P = B_P Cocc,  O_P = Cocc^T Z_P                      (once per preparation)
//   J:  d_P = sum_{mu nu} B_P,mu nu (D1 + D1^T)_mu nu = 2 sum_s <Z_P^s, bra_s>,
//       (J Cocc_s)_mu i = 2 sum_P Z^s_P,mu i d_P             (hess_r.rs:131-139, 1946)
//   K:  K_s = -sum_P [ B_P bra O_P + Z_P (Z_P^T bra)^T ]     (hess_r.rs:159-176)
// evaluated per chunk of aux functions as
//   T[(nu,P), (i,a)] = sum_j bra[nu,j,a] O_P[j,i]           (batched over P, a)
//   out += -scale_k * Bdense[mu, (nu,P)] T[(nu,P), (i,a)]    (one GEMM, K = nao * nchunk)
//   Wt[(j,P), (i,a)] = sum_nu Z_P[nu,i] bra[nu,j,a]          (batched over P, a)
//   out += -scale_k * Z[mu, (j,P)] Wt[(j,P), (i,a)]          (one GEMM, K = nocc * nchunk)
#include <algorithm>

#include "ctx.cuh"
#include "kernels.cuh"
#include "tc_ozaki.cuh"

namespace cphf {

const char* const kProfNames[PROF_NCLASS] = {"gemm_fp64_simt", "gemm_fp32_simt", "kterm_tcgen05_f16x3",
                                             "gemm_fp64_dfloat", "kterm_tcgen05_bf16x6_exact",
                                             "tgen_tcgen05_f16x3", "slice_scale_split",
                                             "krylov_mgs_lu", "xc_grouped_fp64", "xc_grouped_fp32",
                                             "wgen_tcgen05_f16x3", "term2_tcgen05_f16x3",
                                             "xc_tcgen05_f16x3", "xc_tcgen05_bf16x6_exact",
                                             "tgen_tcgen05_bf16x6_exact", "wgen_tcgen05_bf16x6_exact",
                                             "term2_tcgen05_bf16x6_exact", "kterm_tcgen05_bf16x4c_exact",
                                             "tgen_tcgen05_bf16x4c_exact", "wgen_tcgen05_bf16x4c_exact",
                                             "term2_tcgen05_bf16x4c_exact", "slice_exact",
                                             "kterm_tcgen05_bf16x3c_exact", "tgen_tcgen05_bf16x3c_exact",
                                             "wgen_tcgen05_bf16x3c_exact", "term2_tcgen05_bf16x3c_exact",
                                             "xc_tcgen05_bf16c_exact"};

static double gemm_flops(const GemmDesc& d) { return 2.0 * d.M * d.N * d.K * d.batch1 * d.batch2; }

void gemm64(cphf_ctx* c, const GemmDesc& d) {
  if (c->f32_correction) {
    // FP64 operands and result, FP32 arithmetic: the GEMMs of an operator applied to a small
    // correction, whose result is needed only to ~1e-7 of the correction itself
    gemm32x<double, double, double>(c, d);
    return;
  }
  const size_t need = gemm_workspace_bytes(d, 8, c->num_sms);
  if (need) c->ws_gemm.ensure(need, c->counter());
  if (c->f64_emulate) {
    ProfScope ps(c, PROF_GEMM_F64E, gemm_flops(d), 8.0 * (d.M * d.K + d.K * d.N + d.M * d.N) * d.batch1 * d.batch2);
    CPHF_CUDA(gemm_f64_emulated(d, c->stream, c->ws_gemm.p, c->ws_gemm.bytes, c->num_sms));
    return;
  }
  ProfScope ps(c, PROF_GEMM_F64, gemm_flops(d), 8.0 * (d.M * d.K + d.K * d.N + d.M * d.N) * d.batch1 * d.batch2);
  CPHF_CUDA((gemm<double, double, double, double>(d, c->stream, c->ws_gemm.p, c->ws_gemm.bytes, c->num_sms)));
}

void gemm32(cphf_ctx* c, const GemmDesc& d) { gemm32x<float, float, float>(c, d); }

template <typename TA, typename TB, typename TC>
void gemm32x(cphf_ctx* c, const GemmDesc& d) {
  const size_t need = gemm_workspace_bytes(d, 4, c->num_sms);
  if (need) c->ws_gemm.ensure(need, c->counter());
  ProfScope ps(c, PROF_GEMM_F32, gemm_flops(d), 4.0 * (d.M * d.K + d.K * d.N + d.M * d.N) * d.batch1 * d.batch2);
  CPHF_CUDA((gemm<float, TA, TB, TC>(d, c->stream, c->ws_gemm.p, c->ws_gemm.bytes, c->num_sms)));
}
template void gemm32x<float, float, float>(cphf_ctx*, const GemmDesc&);
template void gemm32x<float, float, double>(cphf_ctx*, const GemmDesc&);
template void gemm32x<float, double, float>(cphf_ctx*, const GemmDesc&);
template void gemm32x<double, float, float>(cphf_ctx*, const GemmDesc&);
template void gemm32x<float, double, double>(cphf_ctx*, const GemmDesc&);
template void gemm32x<double, double, float>(cphf_ctx*, const GemmDesc&);
template void gemm32x<double, float, double>(cphf_ctx*, const GemmDesc&);
template void gemm32x<double, double, double>(cphf_ctx*, const GemmDesc&);

void rijk_prepare(cphf_ctx* c) {
  const int64_t nao = c->nao, naux = c->naux;
  for (int s = 0; s < c->nspin; ++s) {
    SpinState& sp = c->spin[s];
    const int64_t no = sp.nocc;
    sp.Z.ensure((size_t)nao * no * naux * 8, c->counter());
    sp.O.ensure((size_t)no * no * naux * 8, c->counter());
    if (no == 0) continue;
    // Z_P = B_P Cocc  (batched over P)
    GemmDesc z;
    z.M = nao; z.N = no; z.K = nao; z.batch1 = naux;
    z.A = c->Bd.p; z.a_m = 1; z.a_k = nao; z.a_b1 = nao * nao;
    z.B = sp.C.p; z.b_k = 1; z.b_n = nao; z.b_b1 = 0;
    z.C = sp.Z.p; z.c_m = 1; z.c_n = nao; z.c_b1 = nao * no;
    gemm64(c, z);
    // O_P = Cocc^T Z_P
    GemmDesc o;
    o.M = no; o.N = no; o.K = nao; o.batch1 = naux;
    o.A = sp.C.p; o.a_m = nao; o.a_k = 1; o.a_b1 = 0;
    o.B = sp.Z.p; o.b_k = 1; o.b_n = nao; o.b_b1 = nao * no;
    o.C = sp.O.p; o.c_m = 1; o.c_n = no; o.c_b1 = no * no;
    gemm64(c, o);
  }
}

// aux functions per K chunk: T/Wt scratch bounded by ~1 GiB and the batched launches
// by the grid limit.
static int64_t k_chunk(const cphf_ctx* c, int64_t no, int64_t nb) {
  if (c->cfg.aux_chunk > 0) return std::min<int64_t>(c->cfg.aux_chunk, c->naux);
  const int64_t per = c->nao * no * nb * 8;
  int64_t np = std::max<int64_t>(1, (int64_t(1) << 30) / std::max<int64_t>(per, 1));
  np = std::min<int64_t>(np, std::max<int64_t>(1, 65535 / std::max<int64_t>(nb, 1)));
  return std::min<int64_t>(np, c->naux);
}

void rijk_response_fp64(cphf_ctx* c, const double* const* bra, int64_t nb, double* const* out,
                        bool accumulate) {
  const int64_t nao = c->nao, naux = c->naux;
  const int ns = c->nspin;
  bool written[2] = {accumulate, accumulate};
  if (c->scale_j != 0.0) {
    c->s_d.ensure((size_t)naux * nb * 8, c->counter());
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      GemmDesc d;
      d.M = naux; d.N = nb; d.K = nao * no;
      d.A = c->spin[s].Z.p; d.a_m = nao * no; d.a_k = 1;
      d.B = bra[s]; d.b_k = 1; d.b_n = nao * no;
      d.C = c->s_d.p; d.c_m = 1; d.c_n = naux;
      d.alpha = 2.0; d.beta = s == 0 ? 0.0 : 1.0;
      if (no > 0) gemm64(c, d);
      else if (s == 0) CPHF_CUDA(cudaMemsetAsync(c->s_d.p, 0, (size_t)naux * nb * 8, c->stream));
    }
    const double jfac = ns == 1 ? c->scale_j : 0.5 * c->scale_j;
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      if (no == 0) continue;
      GemmDesc j;
      j.M = nao * no; j.N = nb; j.K = naux;
      j.A = c->spin[s].Z.p; j.a_m = 1; j.a_k = nao * no;
      j.B = c->s_d.p; j.b_k = 1; j.b_n = naux;
      j.C = out[s]; j.c_m = 1; j.c_n = nao * no;
      j.alpha = 2.0 * jfac; j.beta = written[s] ? 1.0 : 0.0;
      gemm64(c, j);
      written[s] = true;
    }
  }
  if (c->scale_k != 0.0) {
    for (int s = 0; s < ns; ++s) {
      const SpinState& sp = c->spin[s];
      const int64_t no = sp.nocc;
      if (no == 0) continue;
      // the whole K term on the tensor cores with exact BF16 slices (FP64-accurate residual of
      // the mixed solve)
      if (c->oz_kterm && c->lowp) {
        if (!written[s]) CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * no * nb * 8, c->stream));
        written[s] = true;
        oz_k_terms(c, c->lowp->oz, s, bra[s], nb, -c->scale_k, out[s], c->oz_correction);
        continue;
      }
      const int64_t np_max = k_chunk(c, no, nb);
      c->s_T.ensure((size_t)nao * np_max * no * nb * 8, c->counter());
      c->s_W.ensure((size_t)no * np_max * no * nb * 8, c->counter());
      for (int64_t P0 = 0; P0 < naux; P0 += np_max) {
        const int64_t np = std::min<int64_t>(np_max, naux - P0);
        GemmDesc t;  // T[(nu,Pl),(i,a)] = sum_j bra[nu,j,a] O_P[j,i]
        t.M = nao; t.N = no; t.K = no; t.batch1 = np; t.batch2 = nb;
        t.A = bra[s]; t.a_m = 1; t.a_k = nao; t.a_b1 = 0; t.a_b2 = nao * no;
        t.B = sp.O.as<double>() + P0 * no * no; t.b_k = 1; t.b_n = no; t.b_b1 = no * no; t.b_b2 = 0;
        t.C = c->s_T.p; t.c_m = 1; t.c_n = nao * np; t.c_b1 = nao; t.c_b2 = nao * np * no;
        gemm64(c, t);
        GemmDesc k1;  // out += -scale_k Bdense[mu,(nu,P)] T[(nu,P),(i,a)]
        k1.M = nao; k1.N = no * nb; k1.K = nao * np;
        k1.A = c->Bd.as<double>() + P0 * nao * nao; k1.a_m = 1; k1.a_k = nao;
        k1.B = c->s_T.p; k1.b_k = 1; k1.b_n = nao * np;
        k1.C = out[s]; k1.c_m = 1; k1.c_n = nao;
        k1.alpha = -c->scale_k; k1.beta = written[s] ? 1.0 : 0.0;
        gemm64(c, k1);
        written[s] = true;
        GemmDesc w;  // Wt[(j,Pl),(i,a)] = sum_nu Z_P[nu,i] bra[nu,j,a]
        w.M = no; w.N = no; w.K = nao; w.batch1 = np; w.batch2 = nb;
        w.A = sp.Z.as<double>() + P0 * nao * no; w.a_m = nao; w.a_k = 1; w.a_b1 = nao * no; w.a_b2 = 0;
        w.B = bra[s]; w.b_k = 1; w.b_n = nao; w.b_b1 = 0; w.b_b2 = nao * no;
        w.C = c->s_W.p; w.c_m = no * np; w.c_n = 1; w.c_b1 = no; w.c_b2 = no * np * no;
        gemm64(c, w);
        GemmDesc k2;  // out += -scale_k Z[mu,(j,P)] Wt[(j,P),(i,a)]
        k2.M = nao; k2.N = no * nb; k2.K = no * np;
        k2.A = sp.Z.as<double>() + P0 * nao * no; k2.a_m = 1; k2.a_k = nao;
        k2.B = c->s_W.p; k2.b_k = 1; k2.b_n = no * np;
        k2.C = out[s]; k2.c_m = 1; k2.c_n = nao;
        k2.alpha = -c->scale_k; k2.beta = written[s] ? 1.0 : 0.0;
        gemm64(c, k2);
        written[s] = true;
      }
    }
  }
  for (int s = 0; s < ns; ++s) {
    if (!written[s] && c->spin[s].nocc > 0)
      CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * 8, c->stream));
  }
}

}  // namespace cphf
