// XC (fxc) response in bra form for gradient-dependent functionals: the SIGMA (GGA) and TAU
// (meta-GGA) branches of the reference's matrix-multiply numerical integration.
//
// Reference: get_rho_from_one_bra_mult_ket_with_output (src/numint_matmul/pure_eval_rho.rs:
// 216-334; SIGMA terms 289-296, TAU terms 309-315), contract_ao_wv_bra (pure_xcpot.rs:285-352;
// SIGMA 335-343, TAU 345-351), rks_fxc_pot_with_eff_bra_trans_with_output (pure_xcpot.rs:370-465,
// wv[g, y] = w_g sum_x fxc_eff[g, x, y] rho1[g, x]), uks_fxc_pot_with_eff_bra_trans_with_output
// (pure_xcpot.rs:921-1028, wv_t[g, y] = w_g sum_{x,s} fxc_eff[g, x, s, y, t] rho1_s[g, x]);
// get_rks_response_bra (hess_rks.rs:570-605, x4) / get_uks_response_bra (hess_uks.rs:390-441, x2).
//
// Per chunk of grid points (components c = 0 value, 1-3 gradient of the AO values phi_c):
//   ket_c[g, (i,a)] = sum_mu phi_c[g, mu] bra[mu, (i,a)]                    4 GEMMs per spin
//   rho1[g, x, a]  from aobra_c = phi_c Cocc (once per preparation) and ket_c   (one kernel)
//   wv[g, y, a]    = w_g sum_x fxc_eff[g, x, y] rho1[g, x, a]  (UKS: and over the input spin)
//   Q_0 = wv_0 aobra_0 + sum_t wv_t aobra_t,  Q_t = wv_t aobra_0 + 1/2 wv_4 aobra_t (TAU)
//   out[mu, (i,a)] += fac sum_c sum_g phi_c[g, mu] Q_c[g, (i,a)]                  4 GEMMs
// which is contract_ao_wv_bra's sum regrouped by the AO component that multiplies it.  The AO
// values are dense [ngrids, nao, 4]; the GEMMs run on the CUDA cores in FP64 (plain path; the
// double-float kernel inside the mixed solve's FP64-accurate residual) or FP32 (the mixed
// solve's inner operator).
#include <algorithm>

#include "ctx.cuh"
#include "kernels.cuh"
#include "xc_gga.cuh"

namespace cphf {
namespace {

constexpr int kThreads = 256;

unsigned blocks(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(n, kThreads), 1 << 20)); }

// rho1[g + ng (x + nvar a)] of one spin over a chunk of ng points: aob component c of point g
// and orbital i at aob[g + ldg i + ldc c]; ket component c at ket[c ncol ng + g + ng (i + no a)].
template <typename T>
__global__ void gga_rho_kernel(const T* __restrict__ aob, int64_t ldg, int64_t ldc, const T* __restrict__ ket,
                               int64_t ng, int64_t no, int64_t nb, int nvar, T* __restrict__ rho) {
  const int64_t total = ng * nb;
  const int64_t cs = ng * no * nb;  // component stride of ket
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t % ng, a = t / ng;
    double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0, tau = 0.0;
    for (int64_t i = 0; i < no; ++i) {
      const int64_t ka = g + ng * (i + no * a);
      const double a0 = aob[g + ldg * i], a1 = aob[g + ldg * i + ldc], a2 = aob[g + ldg * i + 2 * ldc],
                   a3 = aob[g + ldg * i + 3 * ldc];
      const double k0 = ket[ka], k1 = ket[ka + cs], k2 = ket[ka + 2 * cs], k3 = ket[ka + 3 * cs];
      r0 += a0 * k0;
      r1 += a0 * k1 + a1 * k0;   // pure_eval_rho.rs:289-296
      r2 += a0 * k2 + a2 * k0;
      r3 += a0 * k3 + a3 * k0;
      tau += a1 * k1 + a2 * k2 + a3 * k3;  // pure_eval_rho.rs:309-315
    }
    T* out = rho + g + ng * nvar * a;
    out[0] = (T)r0;
    out[ng] = (T)r1;
    out[2 * ng] = (T)r2;
    out[3 * ng] = (T)r3;
    if (nvar == 5) out[4 * ng] = (T)(0.5 * tau);
  }
}

// Q_c of output spin `so` into q[c ng no nb + g + ng (i + no a)]: wv from fxc_eff and rho1 of
// every input spin (rho1 of spin s at rho + s rho_ss), then contract_ao_wv_bra's components.
// fxc_eff element (x, s_in, y, s_out) of global point G at fxc[G + NG (x + nvar (s_in + 2 (y +
// nvar s_out)))] (UKS), (x, y) at fxc[G + NG (x + nvar y)] (RKS).
template <typename T>
__global__ void gga_q_kernel(const T* __restrict__ aob, int64_t ldg, int64_t ldc, const double* __restrict__ w,
                             const double* __restrict__ fxc, int64_t NG, int64_t g0, int nspin, int so,
                             const T* __restrict__ rho, int64_t rho_ss, int64_t ng, int64_t no, int64_t nb, int nvar,
                             T* __restrict__ q) {
  const int64_t total = ng * nb;
  const int64_t cs = ng * no * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t % ng, a = t / ng;
    const int64_t G = g0 + g;
    double wv[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int si = 0; si < nspin; ++si) {
      const T* r = rho + si * rho_ss + g + ng * nvar * a;
      for (int y = 0; y < nvar; ++y) {
        double acc = 0.0;
        for (int x = 0; x < nvar; ++x) {
          const int64_t idx = nspin == 1 ? x + nvar * y : x + nvar * (si + 2 * (y + nvar * so));
          acc += fxc[G + NG * idx] * (double)r[ng * x];
        }
        wv[y] += acc;
      }
    }
    const double wg = w[G];
    for (int y = 0; y < nvar; ++y) wv[y] *= wg;
    const double half_tau = nvar == 5 ? 0.5 * wv[4] : 0.0;
    for (int64_t i = 0; i < no; ++i) {
      const double a0 = aob[g + ldg * i], a1 = aob[g + ldg * i + ldc], a2 = aob[g + ldg * i + 2 * ldc],
                   a3 = aob[g + ldg * i + 3 * ldc];
      const int64_t qa = g + ng * (i + no * a);
      q[qa] = (T)(wv[0] * a0 + wv[1] * a1 + wv[2] * a2 + wv[3] * a3);   // pure_xcpot.rs:331-333, 336-339
      q[qa + cs] = (T)(wv[1] * a0 + half_tau * a1);                       // 340-342, 345-351
      q[qa + 2 * cs] = (T)(wv[2] * a0 + half_tau * a2);
      q[qa + 3 * cs] = (T)(wv[3] * a0 + half_tau * a3);
    }
  }
}

template <typename T>
void gemm_t(cphf_ctx* c, const GemmDesc& d) {
  if constexpr (sizeof(T) == 8) gemm64(c, d);
  else gemm32(c, d);
}

}  // namespace

void xc_gga_prepare(cphf_ctx* c) {
  const int64_t NG = c->ngrids, nao = c->nao;
  for (int s = 0; s < c->nspin; ++s) {
    SpinState& sp = c->spin[s];
    const int64_t no = sp.nocc;
    sp.aobG.ensure((size_t)std::max<int64_t>(NG * no * 4, 1) * 8, c->counter());
    if (no == 0 || NG == 0) continue;
    for (int comp = 0; comp < 4; ++comp) {
      GemmDesc d;  // aobra_c = phi_c Cocc  (pure_xcpot.rs:403-406)
      d.M = NG; d.N = no; d.K = nao;
      d.A = c->phiG.as<double>() + NG * nao * comp; d.a_m = 1; d.a_k = NG;
      d.B = sp.C.p; d.b_k = 1; d.b_n = nao;
      d.C = sp.aobG.as<double>() + NG * no * comp; d.c_m = 1; d.c_n = NG;
      gemm64(c, d);
    }
  }
}

template <typename T>
void xc_response_gga(cphf_ctx* c, const T* const* bra, int64_t nb, T* const* out, bool accumulate, const T* phi,
                     const T* const* aob, DevBuf& ket_buf, DevBuf& rho_buf) {
  const int64_t NG = c->ngrids, nao = c->nao;
  const int ns = c->nspin;
  const int nvar = c->xc_nvar;
  const double fac = ns == 1 ? 4.0 : 2.0;  // hess_rks.rs:603 / hess_uks.rs:438-439
  int64_t no_max = 0;
  for (int s = 0; s < ns; ++s) no_max = std::max(no_max, c->spin[s].nocc);
  bool written[2] = {accumulate, accumulate};
  if (NG > 0 && no_max > 0 && nb > 0) {
    // chunk of points: the four ket / Q planes within ~4 GiB
    const int64_t per_point = 4 * no_max * nb * (int64_t)sizeof(T);
    int64_t chunk = std::max<int64_t>(32, (int64_t(4) << 30) / std::max<int64_t>(per_point, 1));
    if (c->cfg.xc_chunk_points > 0) chunk = c->cfg.xc_chunk_points;
    chunk = std::min<int64_t>(chunk, NG);
    ket_buf.ensure((size_t)4 * chunk * no_max * nb * sizeof(T), c->counter());
    rho_buf.ensure((size_t)ns * chunk * nvar * nb * sizeof(T), c->counter());
    T* ket = ket_buf.as<T>();
    T* rho = rho_buf.as<T>();
    for (int64_t g0 = 0; g0 < NG; g0 += chunk) {
      const int64_t ng = std::min<int64_t>(chunk, NG - g0);
      const int64_t rho_ss = ng * nvar * nb;
      // rho1 of every spin (the ket planes are reused spin after spin)
      for (int s = 0; s < ns; ++s) {
        const int64_t no = c->spin[s].nocc, N = no * nb;
        if (no == 0) {
          CPHF_CUDA(cudaMemsetAsync(rho + s * rho_ss, 0, (size_t)rho_ss * sizeof(T), c->stream));
          continue;
        }
        for (int comp = 0; comp < 4; ++comp) {
          GemmDesc d;  // ket_c = phi_c bra  (pure_eval_rho.rs:283-296)
          d.M = ng; d.N = N; d.K = nao;
          d.A = phi + g0 + NG * nao * comp; d.a_m = 1; d.a_k = NG;
          d.B = bra[s]; d.b_k = 1; d.b_n = nao;
          d.C = ket + comp * ng * N; d.c_m = 1; d.c_n = ng;
          gemm_t<T>(c, d);
        }
        gga_rho_kernel<T><<<blocks(ng * nb), kThreads, 0, c->stream>>>(aob[s] + g0, NG, NG * no, ket, ng, no, nb,
                                                                        nvar, rho + s * rho_ss);
        count_launch();
      }
      // Q planes and the output contraction per output spin
      for (int so = 0; so < ns; ++so) {
        const int64_t no = c->spin[so].nocc, N = no * nb;
        if (no == 0) continue;
        gga_q_kernel<T><<<blocks(ng * nb), kThreads, 0, c->stream>>>(
            aob[so] + g0, NG, NG * no, c->weights.as<double>(), c->fxcG.as<double>(), NG, g0, ns, so, rho, rho_ss, ng,
            no, nb, nvar, ket);
        count_launch();
        for (int comp = 0; comp < 4; ++comp) {
          GemmDesc d;  // out += fac phi_c^T Q_c  (pure_xcpot.rs:331-351)
          d.M = nao; d.N = N; d.K = ng;
          d.A = phi + g0 + NG * nao * comp; d.a_m = NG; d.a_k = 1;
          d.B = ket + comp * ng * N; d.b_k = 1; d.b_n = ng;
          d.C = out[so]; d.c_m = 1; d.c_n = nao;
          d.alpha = fac;
          d.beta = written[so] ? 1.0 : 0.0;
          gemm_t<T>(c, d);
          written[so] = true;
        }
      }
    }
  }
  for (int s = 0; s < ns; ++s)
    if (!written[s] && c->spin[s].nocc > 0)
      CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * sizeof(T), c->stream));
  CPHF_CUDA(cudaGetLastError());
}

template void xc_response_gga<double>(cphf_ctx*, const double* const*, int64_t, double* const*, bool, const double*,
                                      const double* const*, DevBuf&, DevBuf&);
template void xc_response_gga<float>(cphf_ctx*, const float* const*, int64_t, float* const*, bool, const float*,
                                     const float* const*, DevBuf&, DevBuf&);

}  // namespace cphf
