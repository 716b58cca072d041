// XC response of the split-precision operator on the tensor cores (split FP16, tcgen05).
//
//   ket[p, (i,a)]  = sum_mu phi[p, mu] bra[mu, (i,a)]                  (GEMM 1, rows p, K = mu)
//   out[mu, (i,a)] += fac sum_p phi[p, mu] q[p, (i,a)]                  (GEMM 2, rows mu, K = p)
//
// (the contractions over the grid of get_rho_from_one_bra_mult_ket, pure_eval_rho.rs:283-287,
// and contract_ao_wv_bra, pure_xcpot.rs:331-333), with phi made dense over the AO index
// (zeros outside each grid batch's AO window).  The dense products do nao / nwin times the
// work of the block-sparse ones but run on the tensor cores:
//   * GEMM 1's A is the whole grid's phi as FP16 hi / lo planes [p][mu], one power-of-two
//     scale per point, built once per grid; a chunk of points is a row offset into it (rows
//     need no TMA alignment);
//   * GEMM 2 contracts over the points of a chunk, so its A (phi^T, rows mu) and B (q, rows
//     (i,a)) are sliced per chunk with K starting at 0 (the TMA K coordinate stays aligned).
// The rho1 and weighted-kernel steps between the GEMMs are the FP32 kernels of the SIMT path.
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"
#include "tc_ozaki.cuh"
#include "xc_grouped.cuh"
#include "xc_tc.cuh"

namespace cphf {
namespace {

struct BatchDev {
  int64_t g0, npts, lo, nwin, phi_off;
};

constexpr int EOFF = 14;  // FP16 planes hold x 2^(14 - e) for |x| < 2^e

__device__ __forceinline__ int exp_of(float m) {
  if (!(m > 0.f) || !isfinite(m)) return 0;
  int e;
  frexpf(m, &e);
  return e;
}

__device__ __forceinline__ void put16(float x, int e, __half* dst, int64_t plane) {
  const float v = ldexpf(x, EOFF - e);
  const __half h = __float2half_rn(v);
  dst[0] = h;
  dst[plane] = __float2half_rn(v - __half2float(h));
}

// phi[p, mu] of grid point p (0 outside its batch's AO window and for points of no batch)
__device__ __forceinline__ float phi_at(const float* __restrict__ phi, const BatchDev* __restrict__ batches,
                                        int bi, int64_t p, int64_t mu) {
  if (bi < 0) return 0.f;
  const BatchDev& b = batches[bi];
  const int64_t w = mu - b.lo;
  return (w >= 0 && w < b.nwin) ? phi[b.phi_off + (p - b.g0) + b.npts * w] : 0.f;
}

// dense planes [t][p][ldk] of every grid point, one warp per point, scale 2^(e_p - 14) per row
__global__ void phi_rows_kernel(const float* __restrict__ phi, const BatchDev* __restrict__ batches,
                                const int* __restrict__ pt_batch, int64_t ngrids, int64_t nao, int64_t ldk,
                                __half* __restrict__ dst, int64_t plane, double* __restrict__ rowscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = w0; p < ngrids; p += nw) {
    const int bi = pt_batch[p];
    float m = 0.f;
    if (bi >= 0) {
      const BatchDev& b = batches[bi];
      for (int64_t w = lane; w < b.nwin; w += 32) m = fmaxf(m, fabsf(phi[b.phi_off + (p - b.g0) + b.npts * w]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = exp_of(m);
    for (int64_t mu = lane; mu < nao; mu += 32) put16(phi_at(phi, batches, bi, p, mu), e, dst + p * ldk + mu, plane);
    if (lane == 0) rowscale[p] = ldexp(1.0, e - EOFF);
  }
}

// dense phi^T planes [t][mu][ldq] of the chunk's points [g0, g0 + npts), one warp per AO mu
__global__ void phi_cols_kernel(const float* __restrict__ phi, const BatchDev* __restrict__ batches,
                                const int* __restrict__ pt_batch, int64_t g0, int64_t npts, int64_t nao, int64_t ldq,
                                __half* __restrict__ dst, int64_t plane, double* __restrict__ rowscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t mu = w0; mu < nao; mu += nw) {
    float m = 0.f;
    for (int64_t p = lane; p < npts; p += 32) m = fmaxf(m, fabsf(phi_at(phi, batches, pt_batch[g0 + p], g0 + p, mu)));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = exp_of(m);
    for (int64_t p = lane; p < npts; p += 32)
      put16(phi_at(phi, batches, pt_batch[g0 + p], g0 + p, mu), e, dst + mu * ldq + p, plane);
    if (lane == 0) rowscale[mu] = ldexp(1.0, e - EOFF);
  }
}

// out[i] = mult 2^(e[i] - 14): the column scale of split-FP16 rows with exponents e
__global__ void col_scale_kernel(const int* __restrict__ e, int64_t n, double mult, double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = mult * ldexp(1.0, e[i] - EOFF);
}

unsigned blocks_for(int64_t threads) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(threads, 256), 1 << 20)); }

}  // namespace

void xc_response_tc(cphf_ctx* c, const float* const* bra, int64_t nb, float* const* out, bool accumulate) {
  LowpState& L = *c->lowp;
  XcTcState& X = L.xctc;
  OzState& z = L.lp;
  const int ns = c->nspin;
  const int64_t nao = c->nao, ngrids = c->ngrids, ldk = (nao + 7) / 8 * 8;
  if (!accumulate)
    for (int s = 0; s < ns; ++s)
      if (c->spin[s].nocc > 0)
        CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * 4, c->stream));
  if (nb <= 0 || c->xc_batches.empty()) return;
  cudaStream_t st = c->stream;
  if (!X.ready) {
    // batch records, point -> batch index and the dense phi planes of the whole grid
    std::vector<BatchDev> bh;
    std::vector<int> pb((size_t)ngrids, -1);
    for (size_t b = 0; b < c->xc_batches.size(); ++b) {
      const XcBatch& x = c->xc_batches[b];
      bh.push_back(BatchDev{x.g0, x.npts, x.lo, x.nwin, x.phi_off});
      for (int64_t p = x.g0; p < x.g0 + x.npts; ++p) pb[(size_t)p] = (int)b;
    }
    X.batches.ensure(bh.size() * sizeof(BatchDev), c->counter());
    X.pt_batch.ensure((size_t)std::max<int64_t>(ngrids, 1) * 4, c->counter());
    CPHF_CUDA(cudaMemcpyAsync(X.batches.p, bh.data(), bh.size() * sizeof(BatchDev), cudaMemcpyHostToDevice, st));
    CPHF_CUDA(cudaMemcpyAsync(X.pt_batch.p, pb.data(), pb.size() * 4, cudaMemcpyHostToDevice, st));
    X.phiA.ensure((size_t)2 * ngrids * ldk * 2, c->counter());
    X.phiA_scale.ensure((size_t)ngrids * 8, c->counter());
    phi_rows_kernel<<<blocks_for(ngrids * 32), 256, 0, st>>>(L.phi32.as<float>(), X.batches.as<BatchDev>(),
                                                              X.pt_batch.as<int>(), ngrids, nao, ldk,
                                                              X.phiA.as<__half>(), ngrids * ldk,
                                                              X.phiA_scale.as<double>());
    count_launch();
    CPHF_CUDA(cudaGetLastError());
    CPHF_CUDA(cudaStreamSynchronize(st));  // the host staging vectors go out of scope
    X.ready = true;
  }
  const XcPlan& pl = xc_plan(c, 4, nb);
  int64_t ket_spin[2] = {0, 0};
  for (int s = 0; s < ns; ++s) ket_spin[s] = pl.max_pts * c->spin[s].nocc * nb;
  L.s_ket.ensure((size_t)std::max<int64_t>(1, ket_spin[0] + ket_spin[1]) * 4, c->counter());
  L.s_rho.ensure((size_t)std::max<int64_t>(1, pl.max_pts * nb * 2) * 4, c->counter());
  const int64_t ldq_max = (pl.max_pts + 7) / 8 * 8;
  int64_t nmax = 1;
  for (int s = 0; s < ns; ++s) nmax = std::max<int64_t>(nmax, c->spin[s].nocc * nb);
  X.phiT.ensure((size_t)2 * nao * ldq_max * 2, c->counter());
  X.phiT_scale.ensure((size_t)nao * 8, c->counter());
  X.qpl.ensure((size_t)2 * nmax * ldq_max * 2, c->counter());
  X.eq.ensure((size_t)nmax * 4, c->counter());
  X.qscale.ensure((size_t)nmax * 8, c->counter());
  const double fac = ns == 1 ? 4.0 : 2.0;  // hess_rks.rs:603, hess_uks.rs:438-439
  int* err = L.err.as<int>();
  double nnz = 0.0;
  for (const XcBatch& x : c->xc_batches) nnz += (double)x.npts * (double)x.nwin;
  int64_t occ = 0;
  for (int s = 0; s < ns; ++s) occ += c->spin[s].nocc;
  ProfScope ps(c, PROF_XC32, 4.0 * nnz * occ * nb, 0.0);
  // GEMM 1's B: split planes of bra rows (i, a) over mu, once per application
  for (int s = 0; s < ns; ++s) {
    const int64_t N = c->spin[s].nocc * nb;
    if (N == 0) continue;
    X.bpl[s].ensure((size_t)2 * N * ldk * 2, c->counter());
    X.eb[s].ensure((size_t)N * 4, c->counter());
    X.bscale[s].ensure((size_t)N * 8, c->counter());
    lp_slice_rows(c, bra[s], N, nao, nao, X.bpl[s].as<__half>(), ldk, X.eb[s].as<int>());
    col_scale_kernel<<<blocks_for(N), 256, 0, st>>>(X.eb[s].as<int>(), N, 1.0, X.bscale[s].as<double>());
    count_launch();
  }
  for (const XcChunk& ch : pl.chunks) {
    const int64_t npts = ch.npts, g0 = ch.g0, ldq = (npts + 7) / 8 * 8;
    float* ket[2] = {L.s_ket.as<float>(), L.s_ket.as<float>() + ket_spin[0]};
    float* rho = L.s_rho.as<float>();
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc, N = no * nb;
      float* rho_s = rho + s * npts * nb;
      if (no == 0) {
        CPHF_CUDA(cudaMemsetAsync(rho_s, 0, (size_t)npts * nb * 4, st));
        continue;
      }
      // GEMM 1: ket = phi[g0:g0+npts, :] bra
      CPHF_CUDA(cudaMemsetAsync(ket[s], 0, (size_t)npts * N * 4, st));
      lp_gemm(c, z, X.phiA.as<__half>(), ngrids, ldk, g0, X.bpl[s].as<__half>(), N, ldk, npts, N, nao,
              X.phiA_scale.as<double>() + g0, X.bscale[s].as<double>(), ket[s], npts, err);
      launch_xc_rho<float>(c->spin[s].aobra32.as<float>() + g0, ngrids, ket[s], npts, no, nb, rho_s, npts, st);
    }
    // GEMM 2's A: phi^T of the chunk
    phi_cols_kernel<<<blocks_for(nao * 32), 256, 0, st>>>(L.phi32.as<float>(), X.batches.as<BatchDev>(),
                                                           X.pt_batch.as<int>(), g0, npts, nao, ldq,
                                                           X.phiT.as<__half>(), nao * ldq, X.phiT_scale.as<double>());
    count_launch();
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc, N = no * nb;
      if (no == 0) continue;
      launch_xc_q<float>(c->spin[s].aobra32.as<float>() + g0, ngrids, c->weights.as<double>() + g0,
                         c->fxc.as<double>() + g0, ngrids, ns, s, rho, npts, npts * nb, npts, no, nb, ket[s], st);
      // GEMM 2: out += fac phi^T q over the chunk's points
      lp_slice_rows(c, ket[s], N, npts, npts, X.qpl.as<__half>(), ldq, X.eq.as<int>());
      col_scale_kernel<<<blocks_for(N), 256, 0, st>>>(X.eq.as<int>(), N, fac, X.qscale.as<double>());
      count_launch();
      lp_gemm(c, z, X.phiT.as<__half>(), nao, ldq, 0, X.qpl.as<__half>(), N, ldq, nao, N, npts,
              X.phiT_scale.as<double>(), X.qscale.as<double>(), out[s], nao, err);
    }
  }
  CPHF_CUDA(cudaGetLastError());
}

}  // namespace cphf
