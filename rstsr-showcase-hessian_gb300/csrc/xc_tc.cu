// XC response on the tensor cores (tcgen05), over a dense-AO form of phi:
//
//   ket[p, (i,a)]  = sum_mu phi[p, mu] bra[mu, (i,a)]                  (GEMM 1, rows p, K = mu)
//   out[mu, (i,a)] += fac sum_p phi[p, mu] q[p, (i,a)]                  (GEMM 2, rows mu, K = p)
//
// (the contractions over the grid of get_rho_from_one_bra_mult_ket, pure_eval_rho.rs:283-287,
// and contract_ao_wv_bra, pure_xcpot.rs:331-333), with phi zero outside each grid batch's AO
// window.  The dense products do nao / nwin times the work of the block-sparse ones but run
// on the tensor cores, in one of two operand representations:
//   * split FP16 (Split2: hi / lo planes, three products, FP32 accumulation, ~1e-7 relative):
//     the operator of the mixed solve's inner iterations;
//   * exact BF16 slices (Exact6: six planes, 21 products, exact FP32 accumulation of the
//     leading groups, FP64 outputs, ~2^-34 relative to the row maxima): the FP64-accurate
//     residual of the mixed solve.
// GEMM 1's A is the whole grid's phi as planes [p][mu], one power-of-two scale per point, built
// once per grid; a chunk of points is a row offset into it (rows need no TMA alignment).
// GEMM 2 contracts over the points of a chunk, so its A (phi^T, rows mu) and B (q, rows
// (i,a)) are sliced per chunk with K starting at 0 (the TMA K coordinate stays aligned).
// The rho1 and weighted-kernel steps between the GEMMs are the kernels of the SIMT path.
#include <algorithm>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"
#include "slices.cuh"
#include "tc_ozaki.cuh"
#include "xc_grouped.cuh"
#include "xc_tc.cuh"

namespace cphf {
namespace {

struct BatchDev {
  int64_t g0, npts, lo, nwin, phi_off;
};

// phi[p, mu] of grid point p (0 outside its batch's AO window and for points of no batch)
template <class T>
__device__ __forceinline__ T phi_at(const T* __restrict__ phi, const BatchDev* __restrict__ batches, int bi,
                                    int64_t p, int64_t mu) {
  if (bi < 0) return T(0);
  const BatchDev& b = batches[bi];
  const int64_t w = mu - b.lo;
  return (w >= 0 && w < b.nwin) ? phi[b.phi_off + (p - b.g0) + b.npts * w] : T(0);
}

// dense planes [t][p][ldk] of every grid point, one warp per point; row scale 2^(e_p - EOFF)
template <class PR, class T>
__global__ void phi_rows_kernel(const T* __restrict__ phi, const BatchDev* __restrict__ batches,
                                const int* __restrict__ pt_batch, int64_t ngrids, int64_t nao, int64_t ldk,
                                typename PR::Elem* __restrict__ dst, int64_t plane, double* __restrict__ rowscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = w0; p < ngrids; p += nw) {
    const int bi = pt_batch[p];
    unsigned long long m = 0;
    if (bi >= 0) {
      const BatchDev& b = batches[bi];
      for (int64_t w = lane; w < b.nwin; w += 32) m = max(m, abs_key(phi[b.phi_off + (p - b.g0) + b.npts * w]));
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = key_exp(m, float_key<T>());
    for (int64_t mu = lane; mu < nao; mu += 32)
      Put<PR>::put(phi_at(phi, batches, bi, p, mu), e, dst + p * ldk + mu, plane);
    if (lane == 0) rowscale[p] = ldexp(1.0, e - PR::EOFF);
  }
}

// dense phi^T planes [t][mu][ldq] of the chunk's points [g0, g0 + npts), one warp per AO mu
template <class PR, class T>
__global__ void phi_cols_kernel(const T* __restrict__ phi, const BatchDev* __restrict__ batches,
                                const int* __restrict__ pt_batch, int64_t g0, int64_t npts, int64_t nao, int64_t ldq,
                                typename PR::Elem* __restrict__ dst, int64_t plane, double* __restrict__ rowscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t mu = w0; mu < nao; mu += nw) {
    unsigned long long m = 0;
    for (int64_t p = lane; p < npts; p += 32)
      m = max(m, abs_key(phi_at(phi, batches, pt_batch[g0 + p], g0 + p, mu)));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = key_exp(m, float_key<T>());
    for (int64_t p = lane; p < npts; p += 32)
      Put<PR>::put(phi_at(phi, batches, pt_batch[g0 + p], g0 + p, mu), e, dst + mu * ldq + p, plane);
    if (lane == 0) rowscale[mu] = ldexp(1.0, e - PR::EOFF);
  }
}

// out[i] = mult 2^(e[i] - eoff): the column scale of sliced rows with exponents e
__global__ void col_scale_kernel(const int* __restrict__ e, int64_t n, double mult, int eoff,
                                 double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = mult * ldexp(1.0, e[i] - eoff);
}

unsigned blocks_for(int64_t threads) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(threads, 256), 1 << 20));
}

// per representation: element type, profiler class, the contraction and the row slicer
template <class PR>
struct XcOps;
template <>
struct XcOps<Split2> {
  using T = float;
  static constexpr int PROF = PROF_XC_TC32;
  static void gemm(cphf_ctx* c, OzState& z, const __half* A, int64_t a_rows, int64_t a_ld, int64_t a_row0,
                   const __half* B, int64_t b_rows, int64_t b_ld, int64_t M, int64_t N, int64_t K, const double* rs,
                   const double* cs, float* out, int64_t ld_out, int* err) {
    lp_gemm(c, z, A, a_rows, a_ld, a_row0, B, b_rows, b_ld, M, N, K, rs, cs, out, ld_out, err);
  }
  static void slice(cphf_ctx* c, const float* src, int64_t rows, int64_t K, int64_t rs, __half* dst, int64_t ld,
                    int* e) {
    lp_slice_rows(c, src, rows, K, rs, dst, ld, e);
  }
};
template <>
struct XcOps<Exact6> {
  using T = double;
  static constexpr int PROF = PROF_XC_TC64;
  static void gemm(cphf_ctx* c, OzState& z, const __nv_bfloat16* A, int64_t a_rows, int64_t a_ld, int64_t a_row0,
                   const __nv_bfloat16* B, int64_t b_rows, int64_t b_ld, int64_t M, int64_t N, int64_t K,
                   const double* rs, const double* cs, double* out, int64_t ld_out, int* err) {
    oz_gemm(c, z, A, a_rows, a_ld, a_row0, B, b_rows, b_ld, M, N, K, rs, cs, out, ld_out, err);
  }
  static void slice(cphf_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, __nv_bfloat16* dst,
                    int64_t ld, int* e) {
    oz_slice_rows(c, src, rows, K, rs, dst, ld, e);
  }
};

// The response of all chunks: X holds the planes, z the tuner scratch, ket_buf / rho_buf the
// intermediates; phi and aobra[s] are the grid values in the representation's input type.
template <class PR>
void xc_tc(cphf_ctx* c, XcTcState& X, OzState& z, const typename XcOps<PR>::T* phi,
           const typename XcOps<PR>::T* const* aobra, DevBuf& ket_buf, DevBuf& rho_buf,
           const typename XcOps<PR>::T* const* bra, int64_t nb, typename XcOps<PR>::T* const* out, bool accumulate,
           int* err) {
  using T = typename XcOps<PR>::T;
  using E = typename PR::Elem;
  constexpr int NP = PR::S;
  const int ns = c->nspin;
  const int64_t nao = c->nao, ngrids = c->ngrids, ldk = (nao + 7) / 8 * 8;
  cudaStream_t st = c->stream;
  if (!accumulate)
    for (int s = 0; s < ns; ++s)
      if (c->spin[s].nocc > 0)
        CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * sizeof(T), st));
  if (nb <= 0 || c->xc_batches.empty()) return;
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
    X.phiA.ensure((size_t)NP * ngrids * ldk * sizeof(E), c->counter());
    X.phiA_scale.ensure((size_t)ngrids * 8, c->counter());
    phi_rows_kernel<PR, T><<<blocks_for(ngrids * 32), 256, 0, st>>>(phi, X.batches.as<BatchDev>(),
                                                                     X.pt_batch.as<int>(), ngrids, nao, ldk,
                                                                     X.phiA.as<E>(), ngrids * ldk,
                                                                     X.phiA_scale.as<double>());
    count_launch();
    CPHF_CUDA(cudaGetLastError());
    CPHF_CUDA(cudaStreamSynchronize(st));  // the host staging vectors go out of scope
    X.ready = true;
  }
  const XcPlan& pl = xc_plan(c, sizeof(T), nb);
  int64_t ket_spin[2] = {0, 0};
  for (int s = 0; s < ns; ++s) ket_spin[s] = pl.max_pts * c->spin[s].nocc * nb;
  ket_buf.ensure((size_t)std::max<int64_t>(1, ket_spin[0] + ket_spin[1]) * sizeof(T), c->counter());
  rho_buf.ensure((size_t)std::max<int64_t>(1, pl.max_pts * nb * 2) * sizeof(T), c->counter());
  const int64_t ldq_max = (pl.max_pts + 7) / 8 * 8;
  int64_t nmax = 1;
  for (int s = 0; s < ns; ++s) nmax = std::max<int64_t>(nmax, c->spin[s].nocc * nb);
  X.phiT.ensure((size_t)NP * nao * ldq_max * sizeof(E), c->counter());
  X.phiT_scale.ensure((size_t)nao * 8, c->counter());
  X.qpl.ensure((size_t)NP * nmax * ldq_max * sizeof(E), c->counter());
  X.eq.ensure((size_t)nmax * 4, c->counter());
  X.qscale.ensure((size_t)nmax * 8, c->counter());
  const double fac = ns == 1 ? 4.0 : 2.0;  // hess_rks.rs:603, hess_uks.rs:438-439
  double nnz = 0.0;
  for (const XcBatch& x : c->xc_batches) nnz += (double)x.npts * (double)x.nwin;
  int64_t occ = 0;
  for (int s = 0; s < ns; ++s) occ += c->spin[s].nocc;
  ProfScope ps(c, XcOps<PR>::PROF, 4.0 * nnz * occ * nb, 0.0);
  // GEMM 1's B: planes of bra rows (i, a) over mu, once per application
  for (int s = 0; s < ns; ++s) {
    const int64_t N = c->spin[s].nocc * nb;
    if (N == 0) continue;
    X.bpl[s].ensure((size_t)NP * N * ldk * sizeof(E), c->counter());
    X.eb[s].ensure((size_t)N * 4, c->counter());
    X.bscale[s].ensure((size_t)N * 8, c->counter());
    XcOps<PR>::slice(c, bra[s], N, nao, nao, X.bpl[s].as<E>(), ldk, X.eb[s].as<int>());
    col_scale_kernel<<<blocks_for(N), 256, 0, st>>>(X.eb[s].as<int>(), N, 1.0, PR::EOFF, X.bscale[s].as<double>());
    count_launch();
  }
  for (const XcChunk& ch : pl.chunks) {
    const int64_t npts = ch.npts, g0 = ch.g0, ldq = (npts + 7) / 8 * 8;
    T* ket[2] = {ket_buf.as<T>(), ket_buf.as<T>() + ket_spin[0]};
    T* rho = rho_buf.as<T>();
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc, N = no * nb;
      T* rho_s = rho + s * npts * nb;
      if (no == 0) {
        CPHF_CUDA(cudaMemsetAsync(rho_s, 0, (size_t)npts * nb * sizeof(T), st));
        continue;
      }
      // GEMM 1: ket = phi[g0:g0+npts, :] bra
      CPHF_CUDA(cudaMemsetAsync(ket[s], 0, (size_t)npts * N * sizeof(T), st));
      XcOps<PR>::gemm(c, z, X.phiA.as<E>(), ngrids, ldk, g0, X.bpl[s].as<E>(), N, ldk, npts, N, nao,
                      X.phiA_scale.as<double>() + g0, X.bscale[s].as<double>(), ket[s], npts, err);
      launch_xc_rho<T>(aobra[s] + g0, ngrids, ket[s], npts, no, nb, rho_s, npts, st);
    }
    // GEMM 2's A: phi^T of the chunk
    phi_cols_kernel<PR, T><<<blocks_for(nao * 32), 256, 0, st>>>(phi, X.batches.as<BatchDev>(), X.pt_batch.as<int>(),
                                                                  g0, npts, nao, ldq, X.phiT.as<E>(), nao * ldq,
                                                                  X.phiT_scale.as<double>());
    count_launch();
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc, N = no * nb;
      if (no == 0) continue;
      launch_xc_q<T>(aobra[s] + g0, ngrids, c->weights.as<double>() + g0, c->fxc.as<double>() + g0, ngrids, ns, s,
                     rho, npts, npts * nb, npts, no, nb, ket[s], st);
      // GEMM 2: out += fac phi^T q over the chunk's points
      XcOps<PR>::slice(c, ket[s], N, npts, npts, X.qpl.as<E>(), ldq, X.eq.as<int>());
      col_scale_kernel<<<blocks_for(N), 256, 0, st>>>(X.eq.as<int>(), N, fac, PR::EOFF, X.qscale.as<double>());
      count_launch();
      XcOps<PR>::gemm(c, z, X.phiT.as<E>(), nao, ldq, 0, X.qpl.as<E>(), N, ldq, nao, N, npts,
                      X.phiT_scale.as<double>(), X.qscale.as<double>(), out[s], nao, err);
    }
  }
  CPHF_CUDA(cudaGetLastError());
}

}  // namespace

void xc_response_tc(cphf_ctx* c, const float* const* bra, int64_t nb, float* const* out, bool accumulate) {
  LowpState& L = *c->lowp;
  const float* aobra[2] = {c->spin[0].aobra32.as<float>(), c->nspin > 1 ? c->spin[1].aobra32.as<float>() : nullptr};
  xc_tc<Split2>(c, L.xctc, L.lp, L.phi32.as<float>(), aobra, L.s_ket, L.s_rho, bra, nb, out, accumulate,
                L.err.as<int>());
}

void xc_response_tc64(cphf_ctx* c, const double* const* bra, int64_t nb, double* const* out, bool accumulate) {
  LowpState& L = *c->lowp;
  OzState& z = L.oz;
  z.err.ensure(sizeof(int), c->counter());
  CPHF_CUDA(cudaMemsetAsync(z.err.p, 0, sizeof(int), c->stream));
  const double* aobra[2] = {c->spin[0].aobra.as<double>(), c->nspin > 1 ? c->spin[1].aobra.as<double>() : nullptr};
  xc_tc<Exact6>(c, L.xctc64, z, c->phi.as<double>(), aobra, c->s_ket, c->s_rho, bra, nb, out, accumulate,
                z.err.as<int>());
  int flag = 0;
  CPHF_CUDA(cudaMemcpyAsync(&flag, z.err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  if (flag) throw Error(CPHF_ERR_TIMEOUT, "tensor-core XC response: a bounded pipeline wait expired");
}

}  // namespace cphf
