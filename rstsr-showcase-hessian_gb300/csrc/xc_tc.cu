// XC response on the tensor cores (tcgen05), per grid batch over its AO window:
//
//   ket[p, (i,a)]  = sum_{mu in win} phi[p, mu] bra[mu, (i,a)]          (GEMM 1, rows p, K = mu)
//   out[mu, (i,a)] += fac sum_{p in batch} phi[p, mu] q[p, (i,a)]       (GEMM 2, rows mu in win, K = p)
//   q[p, (i,a)]    = v[p, a] aobra[p, i],  v = w f rho1               (generated as planes)
//
// (the contractions over the grid of get_rho_from_one_bra_mult_ket, pure_eval_rho.rs:283-287,
// and contract_ao_wv_bra, pure_xcpot.rs:331-333), in one of two operand representations:
//   * split FP16 (Split2: hi / lo planes, three products, FP32 accumulation, ~1e-7 relative):
//     the operator of the mixed solve's inner iterations;
//   * exact BF16 slices (Exact6: six planes, 21 products, exact FP32 accumulation of the
//     leading groups, FP64 outputs, ~2^-34 relative to the row maxima): the FP64-accurate
//     residual of the mixed solve.
// Operand layouts (built once per grid):
//   * GEMM 1's A: for every point p, phi[p, lo8 + k] over its batch's window (ldw columns,
//     zero outside the window), one power-of-two scale per point; a batch is a row offset
//     (rows need no TMA alignment) and bra's K offset is lo8, a multiple of 8 AOs;
//   * GEMM 2's A: per batch, rows m of the window holding phi[g0 + k, lo + m] over the batch's
//     points, zero-padded to ldpT, one scale per row;
//   * GEMM 2's B: q is generated per chunk and spin straight from v and aobra into planes over
//     8-padded batch segments, so that each batch's K offset is 16-byte aligned.
// Split FP16 reduces GEMM 1 to rho1[p, a] = sum_i aobra[p, i] ket[p, (i, a)] in its epilogue (ket
// is never written) and generates q's planes in one pass from column-maximum bounds; the exact
// slices store ket, take rho1 from the SIMT path's kernel and slice q with its exact row maxima
// (fixed-point slices are relative to the row scale, so a loose bound would cost accuracy).
#include <algorithm>
#include <type_traits>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"
#include "slices.cuh"
#include "tc_ozaki.cuh"
#include "xc_grouped.cuh"
#include "xc_tc.cuh"

namespace cphf {
namespace {

// A-operand planes of GEMM 1: one warp per grid point; row scale 2^(e_p - EOFF)
template <class PR, class T>
__global__ void phi_win_kernel(const T* __restrict__ phi, const XcTcBatch* __restrict__ batches,
                               const int* __restrict__ pt_batch, int64_t ngrids, int64_t ldw,
                               typename PR::Elem* __restrict__ dst, int64_t plane, double* __restrict__ rowscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = w0; p < ngrids; p += nw) {
    const int bi = pt_batch[p];
    XcTcBatch b{};
    if (bi >= 0) b = batches[bi];
    const T* row = phi + b.phi_off + (p - b.g0);
    unsigned long long m = 0;
    for (int64_t w = lane; w < b.nwin; w += 32) m = max(m, abs_key(row[b.npts * w]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = key_exp(m, float_key<T>());
    for (int64_t k = lane; k < ldw; k += 32) {
      const int64_t w = b.lo8 + k - b.lo;
      Put<PR>::put((w >= 0 && w < b.nwin) ? row[b.npts * w] : T(0), e, dst + p * ldw + k, plane);
    }
    if (lane == 0) rowscale[p] = ldexp(1.0, e - PR::EOFF);
  }
}

// A-operand planes of GEMM 2: one warp per (batch, window AO) row; row scale 2^(e_r - EOFF)
template <class PR, class T>
__global__ void phi_t_kernel(const T* __restrict__ phi, const XcTcBatch* __restrict__ batches,
                             const int* __restrict__ rowmap, int64_t nrow, int64_t ldp,
                             typename PR::Elem* __restrict__ dst, int64_t plane, double* __restrict__ rowscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < nrow; r += nw) {
    const XcTcBatch b = batches[rowmap[r]];
    const T* col = phi + b.phi_off + b.npts * (r - b.rT);
    unsigned long long m = 0;
    for (int64_t k = lane; k < b.npts; k += 32) m = max(m, abs_key(col[k]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = key_exp(m, float_key<T>());
    for (int64_t k = lane; k < ldp; k += 32) Put<PR>::put(k < b.npts ? col[k] : T(0), e, dst + r * ldp + k, plane);
    if (lane == 0) rowscale[r] = ldexp(1.0, e - PR::EOFF);
  }
}

// v[g + npts a] = w[g] sum_s' f[g, s', sout] rho1_s'[g, a] over a chunk's points (the weighted
// kernel of the SIMT path's q, without its aobra factor)
template <class T>
__global__ void xc_v_kernel(const double* __restrict__ w, const double* __restrict__ fxc, int64_t fxc_ld, int nspin,
                            int sout, const T* __restrict__ rho, int64_t ld_rho_spin, int64_t npts, int64_t nb,
                            T* __restrict__ v) {
  const int64_t total = npts * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t % npts;
    double f;
    if (nspin == 1) {
      f = fxc[g] * (double)rho[t];
    } else {
      f = fxc[g + fxc_ld * (0 + 2 * sout)] * (double)rho[t] + fxc[g + fxc_ld * (1 + 2 * sout)] * (double)rho[t + ld_rho_spin];
    }
    v[t] = (T)(w[g] * f);
  }
}

// B-operand planes of GEMM 2: row n = (i, a) over the chunk's 8-padded point columns j,
// q = v[p, a] aobra[p, i] (0 in the padding); one warp per row; column scale fac 2^(e_n - EOFF)
template <class PR, class T>
__global__ void q_planes_kernel(const T* __restrict__ v, const T* __restrict__ aobra, int64_t ngrids,
                                const int* __restrict__ colmap, int64_t g0, int64_t npts, int64_t ncol, int64_t nocc,
                                int64_t nrows, double fac, typename PR::Elem* __restrict__ dst, int64_t plane,
                                double* __restrict__ colscale) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t n = w0; n < nrows; n += nw) {
    const int64_t i = n % nocc, a = n / nocc;
    const T* va = v + npts * a;
    const T* ai = aobra + ngrids * i;
    auto q = [&](int64_t j) -> T {
      const int gp = colmap[j];
      return gp >= 0 ? va[gp - g0] * ai[gp] : T(0);
    };
    unsigned long long m = 0;
    for (int64_t j = lane; j < ncol; j += 32) m = max(m, abs_key(q(j)));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = key_exp(m, float_key<T>());
    for (int64_t j = lane; j < ncol; j += 32) Put<PR>::put(q(j), e, dst + n * ncol + j, plane);
    if (lane == 0) colscale[n] = fac * ldexp(1.0, e - PR::EOFF);
  }
}

// mx[c] = max_r |x[r + ld c]| as ordered keys (r < nr, c = blockIdx.y); mx zeroed first
template <class T>
__global__ void colmax_key_kernel(const T* __restrict__ x, int64_t ld, int64_t nr, unsigned long long* __restrict__ mx) {
  const T* col = x + ld * (int64_t)blockIdx.y;
  unsigned long long m = 0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x)
    m = max(m, abs_key(col[r]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(mx + blockIdx.y, m);
}

// Split-FP16 planes of q[(i, a), j] = v[p, a] aobra[p, i] over the chunk's 8-padded point
// columns j (p = colmap[j], 0 in the padding): one thread per column j and group of QA
// right-hand sides, whose v values stay in registers across the occupied orbitals.  Row
// (i, a) is scaled by 2^(e_v[a] + e_ao[i]), the exponents of the column maxima of v and aobra
// over the chunk: an upper bound of |q| that keeps every element in FP16 range, and the hi /
// lo split keeps ~22 bits of each element relative to itself.
constexpr int QA = 8;
template <class T>
__global__ void q_split_kernel(const T* __restrict__ v, const T* __restrict__ aobra, int64_t ngrids,
                               const int* __restrict__ colmap, int64_t g0, int64_t npts, int64_t ncol, int64_t nocc,
                               int64_t nb, const unsigned long long* __restrict__ mxv,
                               const unsigned long long* __restrict__ mxa, __half* __restrict__ dst, int64_t plane) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= ncol) return;
  const int64_t a0 = (int64_t)blockIdx.y * QA;
  const int na = (int)(nb - a0 < QA ? nb - a0 : QA);
  const int gp = colmap[j];
  float vv[QA];
  int ev[QA];
#pragma unroll
  for (int t = 0; t < QA; ++t) {
    vv[t] = (t < na && gp >= 0) ? (float)v[(gp - g0) + npts * (a0 + t)] : 0.f;
    ev[t] = t < na ? key_exp(mxv[a0 + t], float_key<T>()) : 0;
  }
  for (int64_t i = 0; i < nocc; ++i) {
    const float ao = gp >= 0 ? (float)aobra[gp + ngrids * i] : 0.f;
    const int ea = key_exp(mxa[i], float_key<T>());
#pragma unroll
    for (int t = 0; t < QA; ++t)
      if (t < na) Put<Split2>::put(vv[t] * ao, ev[t] + ea, dst + (i + nocc * (a0 + t)) * ncol + j, plane);
  }
}

// colscale[(i, a)] = fac 2^(e_v[a] + e_ao[i] - EOFF), the scales of q_split_kernel's rows
template <class T>
__global__ void q_split_scale_kernel(const unsigned long long* __restrict__ mxv,
                                     const unsigned long long* __restrict__ mxa, int64_t nocc, int64_t nrows,
                                     double fac, double* __restrict__ colscale) {
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nrows) return;
  const int e = key_exp(mxv[n / nocc], float_key<T>()) + key_exp(mxa[n % nocc], float_key<T>());
  colscale[n] = fac * ldexp(1.0, e - Split2::EOFF);
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
  static void gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0,
                   int64_t M, int64_t N, int64_t K, const double* rs, const double* cs, float* out, int64_t ld_out,
                   int* err, int kb_per_cta, bool store) {
    lp_gemm(c, z, A, a_row0, B, b_k0, M, N, K, rs, cs, out, ld_out, err, kb_per_cta, store);
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
  static void gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0,
                   int64_t M, int64_t N, int64_t K, const double* rs, const double* cs, double* out, int64_t ld_out,
                   int* err, int kb_per_cta, bool store) {
    oz_gemm(c, z, A, a_row0, B, b_k0, M, N, K, rs, cs, out, ld_out, err, kb_per_cta, store);
  }
  static void slice(cphf_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, __nv_bfloat16* dst,
                    int64_t ld, int* e) {
    oz_slice_rows(c, src, rows, K, rs, dst, ld, e);
  }
};

template <int NS>
struct XcOps<ExactC<NS>> {  // correction precision: the leading NS planes of the exact slices
  using T = double;
  static constexpr int PROF = PROF_XC_TC64C;
  static void gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0,
                   int64_t M, int64_t N, int64_t K, const double* rs, const double* cs, double* out, int64_t ld_out,
                   int* err, int kb_per_cta, bool store) {
    oz_gemm_corr(c, z, NS, A, a_row0, B, b_k0, M, N, K, rs, cs, out, ld_out, err, kb_per_cta, store);
  }
  static void slice(cphf_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, __nv_bfloat16* dst,
                    int64_t ld, int* e) {
    oz_slice_rows_corr(c, NS, src, rows, K, rs, dst, ld, e);
  }
};

// Batch records and the phi planes of the grid (once per grid).
template <class PR, class T>
void xc_tc_prepare(cphf_ctx* c, XcTcState& X, const T* phi) {
  using E = typename PR::Elem;
  constexpr int NP = PR::S;
  const int64_t ngrids = c->ngrids;
  cudaStream_t st = c->stream;
  X.hb.clear();
  std::vector<int> pb((size_t)ngrids, -1), rowmap, colmap;
  int64_t ldw = 8, ldp = 8, rT = 0, gofs = 0;
  for (size_t b = 0; b < c->xc_batches.size(); ++b) {
    const XcBatch& x = c->xc_batches[b];
    const int64_t lo8 = x.lo / 8 * 8, kw = x.nwin > 0 ? x.lo + x.nwin - lo8 : 0;
    X.hb.push_back(XcTcBatch{x.g0, x.npts, x.lo, x.nwin, x.phi_off, lo8, kw, rT, gofs});
    for (int64_t p = x.g0; p < x.g0 + x.npts; ++p) pb[(size_t)p] = (int)b;
    for (int64_t m = 0; m < x.nwin; ++m) rowmap.push_back((int)b);
    for (int64_t j = 0; j < (x.npts + 7) / 8 * 8; ++j) colmap.push_back(j < x.npts ? (int)(x.g0 + j) : -1);
    ldw = std::max(ldw, (kw + 7) / 8 * 8);
    ldp = std::max(ldp, (x.npts + 7) / 8 * 8);
    rT += x.nwin;
    gofs += (x.npts + 7) / 8 * 8;
  }
  X.hb.push_back(XcTcBatch{ngrids, 0, 0, 0, 0, 0, 0, rT, gofs});  // end sentinel
  X.ldw = ldw;
  X.ldpT = ldp;
  X.nrowT = rT;
  X.batches.ensure(X.hb.size() * sizeof(XcTcBatch), c->counter());
  X.pt_batch.ensure((size_t)std::max<int64_t>(ngrids, 1) * 4, c->counter());
  X.rowmap.ensure((size_t)std::max<int64_t>(rT, 1) * 4, c->counter());
  X.colmap.ensure((size_t)std::max<int64_t>(gofs, 1) * 4, c->counter());
  CPHF_CUDA(cudaMemcpyAsync(X.batches.p, X.hb.data(), X.hb.size() * sizeof(XcTcBatch), cudaMemcpyHostToDevice, st));
  CPHF_CUDA(cudaMemcpyAsync(X.pt_batch.p, pb.data(), pb.size() * 4, cudaMemcpyHostToDevice, st));
  if (rT > 0) CPHF_CUDA(cudaMemcpyAsync(X.rowmap.p, rowmap.data(), rowmap.size() * 4, cudaMemcpyHostToDevice, st));
  if (gofs > 0) CPHF_CUDA(cudaMemcpyAsync(X.colmap.p, colmap.data(), colmap.size() * 4, cudaMemcpyHostToDevice, st));
  X.phiB.ensure((size_t)NP * ngrids * ldw * sizeof(E), c->counter());
  X.phiB_scale.ensure((size_t)std::max<int64_t>(ngrids, 1) * 8, c->counter());
  X.phiT.ensure((size_t)NP * std::max<int64_t>(rT, 1) * ldp * sizeof(E), c->counter());
  X.phiT_scale.ensure((size_t)std::max<int64_t>(rT, 1) * 8, c->counter());
  phi_win_kernel<PR, T><<<blocks_for(ngrids * 32), 256, 0, st>>>(phi, X.batches.as<XcTcBatch>(), X.pt_batch.as<int>(),
                                                                  ngrids, ldw, X.phiB.as<E>(), ngrids * ldw,
                                                                  X.phiB_scale.as<double>());
  count_launch();
  if (rT > 0) {
    phi_t_kernel<PR, T><<<blocks_for(rT * 32), 256, 0, st>>>(phi, X.batches.as<XcTcBatch>(), X.rowmap.as<int>(), rT,
                                                              ldp, X.phiT.as<E>(), rT * ldp, X.phiT_scale.as<double>());
    count_launch();
  }
  CPHF_CUDA(cudaGetLastError());
  CPHF_CUDA(cudaStreamSynchronize(st));  // the host staging vectors go out of scope
  X.ready = true;
}

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
  // correction precision reads the leading planes of the exact slices' phi planes
  using PREP = std::conditional_t<(PR::NACC == 4 && PR::S < 6), Exact6, PR>;
  if (!X.ready) xc_tc_prepare<PREP, T>(c, X, phi);
  const XcPlan& pl = xc_plan(c, sizeof(T), nb);
  int64_t ket_spin[2] = {0, 0};
  for (int s = 0; s < ns; ++s) ket_spin[s] = pl.max_pts * c->spin[s].nocc * nb;
  constexpr bool fused_rho = std::is_same<PR, Split2>::value;  // rho1 reduced in GEMM 1's epilogue
  if constexpr (!fused_rho)
    ket_buf.ensure((size_t)std::max<int64_t>(1, ket_spin[0] + ket_spin[1]) * sizeof(T), c->counter());
  rho_buf.ensure((size_t)std::max<int64_t>(1, pl.max_pts * nb * 2) * sizeof(T), c->counter());
  int64_t ncol_max = 8, nmax = 1;
  for (const XcChunk& ch : pl.chunks) ncol_max = std::max(ncol_max, X.hb[ch.b1].gofs - X.hb[ch.b0].gofs);
  for (int s = 0; s < ns; ++s) nmax = std::max<int64_t>(nmax, c->spin[s].nocc * nb);
  X.v.ensure((size_t)std::max<int64_t>(1, pl.max_pts * nb) * sizeof(T), c->counter());
  X.qpl.ensure((size_t)NP * nmax * ncol_max * sizeof(E), c->counter());
  X.qscale.ensure((size_t)nmax * 8, c->counter());
  int64_t omax = 1;
  for (int s = 0; s < ns; ++s) omax = std::max<int64_t>(omax, c->spin[s].nocc);
  X.qmax.ensure((size_t)(nb + omax) * 8, c->counter());
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
  const PlaneMat phiB{X.phiB.p, ngrids, X.ldw, X.ldw};
  const PlaneMat phiT{X.phiT.p, std::max<int64_t>(X.nrowT, 1), X.ldpT, X.ldpT};
  for (const XcChunk& ch : pl.chunks) {
    const int64_t npts = ch.npts, g0 = ch.g0;
    const int64_t gofs0 = X.hb[ch.b0].gofs, ncol = X.hb[ch.b1].gofs - gofs0;
    T* ket[2] = {ket_buf.as<T>(), ket_buf.as<T>() + ket_spin[0]};
    T* rho = rho_buf.as<T>();
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc, N = no * nb;
      T* rho_s = rho + s * npts * nb;
      if (no == 0) {
        CPHF_CUDA(cudaMemsetAsync(rho_s, 0, (size_t)npts * nb * sizeof(T), st));
        continue;
      }
      const PlaneMat B{X.bpl[s].p, N, ldk, nao};
      if constexpr (fused_rho) {
        // GEMM 1 per batch reduced to rho1[p, a] = sum_i aobra[p, i] (phi[p, win] bra[win, (i, a)])
        CPHF_CUDA(cudaMemsetAsync(rho_s, 0, (size_t)npts * nb * sizeof(T), st));
        for (int64_t b = ch.b0; b < ch.b1; ++b) {
          const XcTcBatch& x = X.hb[b];
          if (x.npts == 0 || x.nwin == 0) continue;
          const RhoEpilogue re{rho_s + (x.g0 - g0), aobra[s] + x.g0, npts, ngrids, no};
          lp_gemm_rho(c, z, phiB, x.g0, B, x.lo8, x.npts, N, x.kw, X.phiB_scale.as<double>() + x.g0,
                      X.bscale[s].as<double>(), re, err, (int)div_up(x.kw, 32));
        }
      } else {
        // GEMM 1 per batch: ket[p - g0, :] = phi[p, win] bra[win, :] (one K range: stored)
        for (int64_t b = ch.b0; b < ch.b1; ++b) {
          const XcTcBatch& x = X.hb[b];
          if (x.npts == 0) continue;
          if (x.nwin == 0) {
            CPHF_CUDA(cudaMemset2DAsync(ket[s] + (x.g0 - g0), npts * sizeof(T), 0, x.npts * sizeof(T), N, st));
            continue;
          }
          XcOps<PR>::gemm(c, z, phiB, x.g0, B, x.lo8, x.npts, N, x.kw, X.phiB_scale.as<double>() + x.g0,
                          X.bscale[s].as<double>(), ket[s] + (x.g0 - g0), npts, err, (int)div_up(x.kw, 32), true);
        }
        launch_xc_rho<T>(aobra[s] + g0, ngrids, ket[s], npts, no, nb, rho_s, npts, st);
      }
    }
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc, N = no * nb;
      if (no == 0) continue;
      xc_v_kernel<T><<<blocks_for(npts * nb), 256, 0, st>>>(c->weights.as<double>() + g0, c->fxc.as<double>() + g0,
                                                            ngrids, ns, s, rho, npts * nb, npts, nb, X.v.as<T>());
      count_launch();
      if constexpr (std::is_same<PR, Split2>::value) {
        // one pass, scales from the column maxima of v and aobra over the chunk
        unsigned long long* mxv = X.qmax.as<unsigned long long>();
        unsigned long long* mxa = mxv + nb;
        CPHF_CUDA(cudaMemsetAsync(mxv, 0, (size_t)(nb + no) * 8, st));
        const unsigned gx = (unsigned)std::min<int64_t>(div_up(npts, 256), 64);
        colmax_key_kernel<T><<<dim3(gx, (unsigned)nb), 256, 0, st>>>(X.v.as<T>(), npts, npts, mxv);
        colmax_key_kernel<T><<<dim3(gx, (unsigned)no), 256, 0, st>>>(aobra[s] + g0, ngrids, npts, mxa);
        q_split_scale_kernel<T><<<blocks_for(N), 256, 0, st>>>(mxv, mxa, no, N, fac, X.qscale.as<double>());
        q_split_kernel<T><<<dim3((unsigned)div_up(ncol, 128), (unsigned)div_up(nb, QA)), 128, 0, st>>>(
            X.v.as<T>(), aobra[s], ngrids, X.colmap.as<int>() + gofs0, g0, npts, ncol, no, nb, mxv, mxa,
            X.qpl.as<__half>(), N * ncol);
        count_launch(4);
      } else {
        q_planes_kernel<PR, T><<<blocks_for(N * 32), 256, 0, st>>>(X.v.as<T>(), aobra[s], ngrids,
                                                                   X.colmap.as<int>() + gofs0, g0, npts, ncol, no, N,
                                                                   fac, X.qpl.as<E>(), N * ncol, X.qscale.as<double>());
        count_launch();
      }
      // GEMM 2 per batch: out[win, :] += fac phi[batch, win]^T q[batch, :]
      const PlaneMat Q{X.qpl.p, N, ncol, ncol};
      const int64_t n_tiles = div_up(N, 128);
      for (int64_t b = ch.b0; b < ch.b1; ++b) {
        const XcTcBatch& x = X.hb[b];
        if (x.nwin == 0 || x.npts == 0) continue;
        const int64_t nkb = div_up(x.npts, 32), tiles = div_up(x.nwin, 128) * n_tiles;
        const int64_t ranges = std::min<int64_t>(nkb, div_up(2 * (int64_t)c->num_sms, tiles));
        XcOps<PR>::gemm(c, z, phiT, x.rT, Q, x.gofs - gofs0, x.nwin, N, x.npts, X.phiT_scale.as<double>() + x.rT,
                        X.qscale.as<double>(), out[s] + x.lo, nao, err, (int)div_up(nkb, ranges), false);
      }
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
  // a correction-precision application (3 or 4 slices) shares the exact slices' grid planes
  if (c->oz_correction == 3)
    xc_tc<Exact6c3>(c, L.xctc64, z, c->phi.as<double>(), aobra, c->s_ket, c->s_rho, bra, nb, out, accumulate,
                    z.err.as<int>());
  else if (c->oz_correction == 4)
    xc_tc<Exact6c>(c, L.xctc64, z, c->phi.as<double>(), aobra, c->s_ket, c->s_rho, bra, nb, out, accumulate,
                   z.err.as<int>());
  else
    xc_tc<Exact6>(c, L.xctc64, z, c->phi.as<double>(), aobra, c->s_ket, c->s_rho, bra, nb, out, accumulate,
                  z.err.as<int>());
  int flag = 0;
  CPHF_CUDA(cudaMemcpyAsync(&flag, z.err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  if (flag) throw Error(CPHF_ERR_TIMEOUT, "tensor-core XC response: a bounded pipeline wait expired");
}

}  // namespace cphf
