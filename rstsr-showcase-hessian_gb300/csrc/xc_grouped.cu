// Persistent grouped GEMMs for the XC response over uneven per-atom grid batches.
//
// One chunk of grid batches (e.g. a run of atoms) is processed by two launches, whatever
// the batch sizes:
//   ket[p, n]  = sum_mu phi_g[p - p_g, mu] bra[lo_g + mu, n]        (rows p of batch g)
//   out[mu, n] = beta out[mu, n] + alpha sum_g sum_p phi_g[p - p_g, mu - lo_g] q[p, n]
// ket / q are [P_chunk, N] with the chunk's points stacked, so the rho1 and weighted-kernel
// steps between the two launches run over the whole chunk at once.  The first launch walks
// a flat list of (batch, row tile, column tile) work items; the second gives every output
// tile the batches whose AO window meets it and sums them in a fixed order (deterministic,
// no atomics).  Reference: contract over the grid of get_rho_from_one_bra_mult_ket
// (pure_eval_rho.rs:283-287) and contract_ao_wv_bra (pure_xcpot.rs:331-333).
#include <algorithm>
#include <vector>

#include "ctx.cuh"
#include "dfloat.cuh"
#include "kernels.cuh"
#include "xc_grouped.cuh"

namespace cphf {
namespace {

template <typename T>
struct XcCfg;
template <>
struct XcCfg<double> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};
template <>
struct XcCfg<float> {
  static constexpr int BM = 128, BN = 128, BK = 16, TM = 8, TN = 8;
};

// Register-tiled product over one K range; loadA(m, k) / loadB(k, n) return 0 outside.
// Operands are stored as T and converted to the compute type TC when staged (TC = dfloat:
// FP64-accurate products on the FP32 pipes for the mixed solve's residual).  The next K tile
// is fetched into registers while the current one is multiplied out of shared memory (FP32
// compute; for FP64 / double-float the extra registers cost more occupancy than they save).
template <typename TC, typename Cfg, typename LA_, typename LB_>
__device__ __forceinline__ void tile_accumulate(TC (&acc)[Cfg::TM][Cfg::TN], int64_t K, LA_ loadA, LB_ loadB,
                                                TC (*As)[Cfg::BM], TC (*Bs)[Cfg::BN]) {
  constexpr int BM = Cfg::BM, BN = Cfg::BN, BK = Cfg::BK, TM = Cfg::TM, TN = Cfg::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  constexpr int RA = BM * BK / NT, RB = BK * BN / NT;
  static_assert(BM * BK % NT == 0 && BK * BN % NT == 0, "tile / thread count");
  const int tid = threadIdx.x, tx = tid % NTX, ty = tid / NTX;
  if (K <= 0) return;
  TC ra[RA], rb[RB];
  auto fetch = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < RA; ++r) {
      const int e = tid + r * NT, mm = e % BM, kk = e / BM;
      ra[r] = (k0 + kk < K) ? TC(loadA(mm, k0 + kk)) : TC(0);
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      const int e = tid + r * NT, kk = e % BK, nn = e / BK;
      rb[r] = (k0 + kk < K) ? TC(loadB(k0 + kk, nn)) : TC(0);
    }
  };
  constexpr bool PREFETCH = sizeof(TC) == 4;
  if (PREFETCH) fetch(0);
  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    if (PREFETCH) {
#pragma unroll
      for (int r = 0; r < RA; ++r) {
        const int e = tid + r * NT;
        As[e / BM][e % BM] = ra[r];
      }
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        const int e = tid + r * NT;
        Bs[e % BK][e / BK] = rb[r];
      }
    } else {
      for (int e = tid; e < BM * BK; e += NT) {
        const int mm = e % BM, kk = e / BM;
        As[kk][mm] = (k0 + kk < K) ? TC(loadA(mm, k0 + kk)) : TC(0);
      }
      for (int e = tid; e < BK * BN; e += NT) {
        const int kk = e % BK, nn = e / BK;
        Bs[kk][nn] = (k0 + kk < K) ? TC(loadB(k0 + kk, nn)) : TC(0);
      }
    }
    __syncthreads();
    if (PREFETCH && k0 + BK < K) fetch(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      TC a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + i * NTY];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + j * NTX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = madd(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
}

template <typename T, typename TC>
__global__ void __launch_bounds__(256, sizeof(TC) == 4 ? 2 : 3) xc_gemm1_kernel(const XcGroupDev* __restrict__ groups, int ngroups,
                                                       const T* __restrict__ phi, const T* __restrict__ bra,
                                                       int64_t nao, int64_t N, int64_t pchunk, T* __restrict__ ket,
                                                       int64_t total_tiles, int64_t tiles_n) {
  using Cfg = XcCfg<T>;
  constexpr int BM = Cfg::BM, BN = Cfg::BN, BK = Cfg::BK, TM = Cfg::TM, TN = Cfg::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM;
  __shared__ TC As[BK][BM];
  __shared__ TC Bs[BK][BN];
  const int tid = threadIdx.x, tx = tid % NTX, ty = tid / NTX;
  for (int64_t w = blockIdx.x; w < total_tiles; w += gridDim.x) {
    int g = 0;
    while (g + 1 < ngroups && groups[g + 1].tile_begin <= w) ++g;  // groups are few (atoms)
    const XcGroupDev G = groups[g];
    const int64_t local = w - G.tile_begin;
    const int64_t tm = local / tiles_n, tn = local % tiles_n;
    const int64_t m0 = tm * BM, n0 = tn * BN;
    TC acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = TC(0);
    const T* A = phi + G.phi_off;
    auto la = [&](int mm, int64_t k) -> T {
      const int64_t m = m0 + mm;
      return m < G.npts ? A[m + G.npts * k] : (T)0;
    };
    auto lb = [&](int64_t k, int nn) -> T {
      const int64_t n = n0 + nn;
      return n < N ? bra[G.lo + k + nao * n] : (T)0;
    };
    tile_accumulate<TC, Cfg>(acc, G.nwin, la, lb, As, Bs);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t m = m0 + ty + i * NTY;
      if (m >= G.npts) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int64_t n = n0 + tx + j * NTX;
        if (n < N) ket[G.p_local + m + pchunk * n] = static_cast<T>(acc[i][j]);
      }
    }
  }
}

template <typename T, typename TC>
__global__ void __launch_bounds__(256, sizeof(TC) == 4 ? 2 : 3) xc_gemm2_kernel(const XcGroupDev* __restrict__ groups, int ngroups,
                                                       const T* __restrict__ phi, const T* __restrict__ q,
                                                       int64_t nao, int64_t N, int64_t pchunk, T* __restrict__ out,
                                                       double alpha, double beta, int64_t tiles_m, int64_t tiles_n) {
  using Cfg = XcCfg<T>;
  constexpr int BM = Cfg::BM, BN = Cfg::BN, BK = Cfg::BK, TM = Cfg::TM, TN = Cfg::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM;
  __shared__ TC As[BK][BM];
  __shared__ TC Bs[BK][BN];
  const int tid = threadIdx.x, tx = tid % NTX, ty = tid / NTX;
  for (int64_t w = blockIdx.x; w < tiles_m * tiles_n; w += gridDim.x) {
    const int64_t tm = w % tiles_m, tn = w / tiles_m;
    const int64_t m0 = tm * BM, n0 = tn * BN;
    TC acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = TC(0);
    for (int g = 0; g < ngroups; ++g) {
      const XcGroupDev G = groups[g];
      if (G.nwin == 0 || G.lo >= m0 + BM || G.lo + G.nwin <= m0) continue;  // window misses the tile
      const T* A = phi + G.phi_off;
      auto la = [&](int mm, int64_t k) -> T {  // A(mu, p) = phi_g[p, mu - lo]
        const int64_t mu = m0 + mm - G.lo;
        return (mu >= 0 && mu < G.nwin) ? A[k + G.npts * mu] : (T)0;
      };
      auto lb = [&](int64_t k, int nn) -> T {
        const int64_t n = n0 + nn;
        return n < N ? q[G.p_local + k + pchunk * n] : (T)0;
      };
      tile_accumulate<TC, Cfg>(acc, G.npts, la, lb, As, Bs);
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t m = m0 + ty + i * NTY;
      if (m >= nao) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int64_t n = n0 + tx + j * NTX;
        if (n >= N) continue;
        T* p = out + m + nao * n;
        T v = (T)alpha * static_cast<T>(acc[i][j]);
        if (beta != 0.0) v = fma((T)beta, *p, v);
        *p = v;
      }
    }
  }
}

}  // namespace

template <typename T>
void xc_grouped_gemm1(cphf_ctx* c, const XcGroupDev* groups_dev, int ngroups, int64_t total_tiles, const T* phi,
                      const T* bra, int64_t N, int64_t pchunk, T* ket) {
  using Cfg = XcCfg<T>;
  const int64_t tiles_n = div_up(N, Cfg::BN);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(total_tiles, 8 * (int64_t)c->num_sms));
  bool launched = false;
  if constexpr (sizeof(T) == 8) {
    if (c->f64_emulate) {
      xc_gemm1_kernel<T, dfloat><<<grid, 256, 0, c->stream>>>(groups_dev, ngroups, phi, bra, c->nao, N, pchunk, ket,
                                                              total_tiles, tiles_n);
      launched = true;
    }
  }
  if (!launched)
    xc_gemm1_kernel<T, T><<<grid, 256, 0, c->stream>>>(groups_dev, ngroups, phi, bra, c->nao, N, pchunk, ket,
                                                       total_tiles, tiles_n);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

template <typename T>
void xc_grouped_gemm2(cphf_ctx* c, const XcGroupDev* groups_dev, int ngroups, const T* phi, const T* q, int64_t N,
                      int64_t pchunk, T* out, double alpha, double beta) {
  using Cfg = XcCfg<T>;
  const int64_t tiles_m = div_up(c->nao, Cfg::BM), tiles_n = div_up(N, Cfg::BN);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tiles_m * tiles_n, 8 * (int64_t)c->num_sms));
  bool launched = false;
  if constexpr (sizeof(T) == 8) {
    if (c->f64_emulate) {
      xc_gemm2_kernel<T, dfloat><<<grid, 256, 0, c->stream>>>(groups_dev, ngroups, phi, q, c->nao, N, pchunk, out,
                                                              alpha, beta, tiles_m, tiles_n);
      launched = true;
    }
  }
  if (!launched)
    xc_gemm2_kernel<T, T><<<grid, 256, 0, c->stream>>>(groups_dev, ngroups, phi, q, c->nao, N, pchunk, out, alpha,
                                                       beta, tiles_m, tiles_n);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

int64_t xc_tiles_m(int64_t npts, bool f64) { return div_up(npts, f64 ? XcCfg<double>::BM : XcCfg<float>::BM); }
int64_t xc_tiles_n(int64_t N, bool f64) { return div_up(N, f64 ? XcCfg<double>::BN : XcCfg<float>::BN); }

// Chunks of consecutive batches whose intermediates (ket of every spin) fit the budget; one
// cached plan per (precision, chunk cap, nb, nocc) so that the block widths of a Krylov solve
// each keep theirs (captured operator graphs read the plan's device records).
XcPlan& xc_plan(cphf_ctx* c, size_t esize, int64_t nb) {
  const bool f64 = esize == 8;
  const int ns = c->nspin;
  const int64_t key[4] = {(int64_t)esize * 1000003 + c->cfg.xc_chunk_points, nb, c->spin[0].nocc,
                          ns > 1 ? c->spin[1].nocc : -1};
  for (auto& p : c->xc_plans)
    if (std::equal(key, key + 4, p->key) && !p->chunks.empty()) return *p;
  if (c->xc_plans.size() >= 64) c->xc_plans.erase(c->xc_plans.begin());  // frees its records
  c->xc_plans.emplace_back(new XcPlan());
  XcPlan& pl = *c->xc_plans.back();
  const int64_t budget = int64_t(8) << 30;  // bytes of ket intermediates per chunk
  int64_t per_point = 0;
  for (int s = 0; s < ns; ++s) per_point += c->spin[s].nocc * nb * (int64_t)esize;
  per_point = std::max<int64_t>(per_point, 1);
  const int64_t cap = c->cfg.xc_chunk_points > 0 ? c->cfg.xc_chunk_points : std::max<int64_t>(1, budget / per_point);
  pl.chunks.clear();
  std::vector<XcGroupDev> recs;
  const int64_t nbatch = (int64_t)c->xc_batches.size();
  int64_t b = 0;
  pl.max_pts = 0;
  while (b < nbatch) {
    XcChunk ch{};
    ch.b0 = b;
    ch.g0 = c->xc_batches[b].g0;
    int64_t pts = 0;
    while (b < nbatch && (pts == 0 || pts + c->xc_batches[b].npts <= cap)) pts += c->xc_batches[b++].npts;
    ch.b1 = b;
    ch.npts = pts;
    ch.group_off = (int64_t)recs.size();
    for (int s = 0; s < 2; ++s) {
      const int64_t N = s < ns ? c->spin[s].nocc * nb : 0;
      const int64_t tn = xc_tiles_n(std::max<int64_t>(N, 1), f64);
      int64_t tiles = 0;
      for (int64_t k = ch.b0; k < ch.b1; ++k) {
        const XcBatch& x = c->xc_batches[k];
        XcGroupDev g{x.g0 - ch.g0, x.npts, x.lo, x.nwin, x.phi_off, tiles};
        if (x.nwin > 0) tiles += xc_tiles_m(x.npts, f64) * tn;
        recs.push_back(g);
      }
      ch.tiles[s] = tiles;
    }
    pl.max_pts = std::max(pl.max_pts, pts);
    pl.chunks.push_back(ch);
  }
  pl.groups.ensure(std::max<size_t>(recs.size(), 1) * sizeof(XcGroupDev), c->counter());
  CPHF_CUDA(cudaMemcpyAsync(pl.groups.p, recs.data(), recs.size() * sizeof(XcGroupDev), cudaMemcpyHostToDevice,
                            c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  std::copy(key, key + 4, pl.key);
  return pl;
}

template <typename T>
void xc_response_grouped(cphf_ctx* c, const T* const* bra, int64_t nb, T* const* out, bool accumulate, const T* phi,
                         const T* const* aobra, DevBuf& ket_buf, DevBuf& rho_buf) {
  const int ns = c->nspin;
  const int64_t nao = c->nao;
  if (!accumulate)
    for (int s = 0; s < ns; ++s)
      if (c->spin[s].nocc > 0) CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * sizeof(T), c->stream));
  if (nb <= 0 || c->xc_batches.empty()) return;
  XcPlan& pl = xc_plan(c, sizeof(T), nb);
  int64_t ket_spin[2] = {0, 0};
  for (int s = 0; s < ns; ++s) ket_spin[s] = pl.max_pts * c->spin[s].nocc * nb;
  ket_buf.ensure((size_t)std::max<int64_t>(1, ket_spin[0] + ket_spin[1]) * sizeof(T), c->counter());
  rho_buf.ensure((size_t)std::max<int64_t>(1, pl.max_pts * nb * 2) * sizeof(T), c->counter());
  const double fac = ns == 1 ? 4.0 : 2.0;  // hess_rks.rs:603, hess_uks.rs:438-439
  const XcGroupDev* gdev = pl.groups.as<XcGroupDev>();
  double nnz = 0.0;  // stored AO values of the grid batches
  for (const XcBatch& x : c->xc_batches) nnz += (double)x.npts * (double)x.nwin;
  int64_t occ = 0;
  for (int s = 0; s < ns; ++s) occ += c->spin[s].nocc;
  ProfScope ps(c, sizeof(T) == 8 ? PROF_XC64 : PROF_XC32, 4.0 * nnz * occ * nb, 0.0);
  for (const XcChunk& ch : pl.chunks) {
    const int ng = (int)(ch.b1 - ch.b0);
    T* ket[2] = {ket_buf.as<T>(), ket_buf.as<T>() + ket_spin[0]};
    T* rho = rho_buf.as<T>();
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      T* rho_s = rho + s * ch.npts * nb;
      if (no == 0) {
        CPHF_CUDA(cudaMemsetAsync(rho_s, 0, (size_t)ch.npts * nb * sizeof(T), c->stream));
        continue;
      }
      // rows of batches with an empty AO window are never written: clear them first
      CPHF_CUDA(cudaMemsetAsync(ket[s], 0, (size_t)ch.npts * no * nb * sizeof(T), c->stream));
      xc_grouped_gemm1<T>(c, gdev + ch.group_off + s * ng, ng, ch.tiles[s], phi, bra[s], no * nb, ch.npts, ket[s]);
      launch_xc_rho<T>(aobra[s] + ch.g0, c->ngrids, ket[s], ch.npts, no, nb, rho_s, ch.npts, c->stream);
    }
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      if (no == 0) continue;
      launch_xc_q<T>(aobra[s] + ch.g0, c->ngrids, c->weights.as<double>() + ch.g0, c->fxc.as<double>() + ch.g0,
                     c->ngrids, ns, s, rho, ch.npts, ch.npts * nb, ch.npts, no, nb, ket[s], c->stream);
      xc_grouped_gemm2<T>(c, gdev + ch.group_off + s * ng, ng, phi, ket[s], no * nb, ch.npts, out[s], fac, 1.0);
    }
  }
}

template void xc_response_grouped<double>(cphf_ctx*, const double* const*, int64_t, double* const*, bool,
                                          const double*, const double* const*, DevBuf&, DevBuf&);
template void xc_response_grouped<float>(cphf_ctx*, const float* const*, int64_t, float* const*, bool, const float*,
                                         const float* const*, DevBuf&, DevBuf&);

template void xc_grouped_gemm1<double>(cphf_ctx*, const XcGroupDev*, int, int64_t, const double*, const double*,
                                       int64_t, int64_t, double*);
template void xc_grouped_gemm1<float>(cphf_ctx*, const XcGroupDev*, int, int64_t, const float*, const float*,
                                      int64_t, int64_t, float*);
template void xc_grouped_gemm2<double>(cphf_ctx*, const XcGroupDev*, int, const double*, const double*, int64_t,
                                       int64_t, double*, double, double);
template void xc_grouped_gemm2<float>(cphf_ctx*, const XcGroupDev*, int, const float*, const float*, int64_t,
                                      int64_t, float*, double, double);

}  // namespace cphf
