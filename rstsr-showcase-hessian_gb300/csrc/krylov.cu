// Block Krylov solver for (I + A) x = b on the device.
//
// Follows krylov_block (src/util/krylov_block.rs:39-197) step by step:
//   - residual of the accumulated solution at each (re)start (86-87),
//   - orth_block: serial modified Gram-Schmidt of the block, non-normalized, dropping
//     ||v||^2 <= lindep (225-253) -- run right-looking on the device, same update order,
//   - per cycle: aop on the surviving block, append to the xs / ax slabs (111-116),
//     project the image off the whole subspace at once (119-122), MGS the new
//     directions, convergence on the unfiltered max ||v||^2 (130, 157), keep only
//     directions above max(lindep, tol^2) (134-142),
//   - hard restart into x_accum (170-175) and the final projected solve (178-184),
//   - projected_solve: h = xs^T ax + diag(ip), g = xs^T b, LU solve, xs c (204-215).
// The Galerkin matrix h is assembled block by block as the subspace grows (its new
// columns are exactly the xs^T axt product of the projection step), so each entry is
// the same dot product the reference evaluates at solve time.
// All arithmetic here is FP64.  The only host synchronisation per cycle is the read
// of the MGS keep flags / squared norms (the reference's Vec<f64>).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"

namespace cphf {

namespace {

struct KrylovWork {
  double *xs, *ax, *h, *hw, *gw, *bres, *xacc, *x1, *coef, *ip_dev, *part;
  int *keep, *idx, *info;
};

// MGS on V [n, m]; returns kept flags and squared norms (host), synchronizing once.
void orth_block(cphf_ctx* c, const KrylovWork& w, double* V, int64_t n, int64_t m, double lindep,
                std::vector<int>& keep, std::vector<double>& ip) {
  keep.assign(m, 0);
  ip.assign(m, 0.0);
  if (m == 0) return;
  double* ipd = w.part + mgs_partials_size(n, m) + m;  // after partials + coef
  {
    // algorithmic work of the right-looking MGS: m(m-1)/2 dot + axpy pairs of length n
    // (~2 n m^2 FLOPs), each step re-reading and re-writing the trailing columns (~8 n m^2 bytes)
    ProfScope ps(c, PROF_KRYLOV, 2.0 * n * m * m, 8.0 * n * m * m);
    launch_mgs(V, n, m, lindep, ipd, w.keep, w.part, c->stream);
  }
  CPHF_CUDA(cudaMemcpyAsync(keep.data(), w.keep, m * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaMemcpyAsync(ip.data(), ipd, m * 8, cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  for (int64_t i = 0; i < m; ++i)
    if (!std::isfinite(ip[i])) throw Error(CPHF_ERR_NONFINITE, "non-finite vector in the Krylov subspace");
}

// Copy the selected columns of V [n, m] to dst (ld n).
void select_cols(cphf_ctx* c, const KrylovWork& w, const double* V, int64_t n,
                 const std::vector<int>& sel, double* dst) {
  if (sel.empty()) return;
  CPHF_CUDA(cudaMemcpyAsync(w.idx, sel.data(), sel.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  launch_gather_cols(V, n, w.idx, (int64_t)sel.size(), dst, n, c->stream);
}

// x_out (+)= xs c with h c = g, h = xs^T ax + diag(ip), g = xs^T b   (krylov_block.rs:204-215)
void projected_solve(cphf_ctx* c, const KrylovWork& w, int64_t n, int64_t nd, int64_t maxb,
                     int64_t nset, const double* b, double* x_out, bool accumulate) {
  // hw = h[:nd, :nd] + diag(ip)
  CPHF_CUDA(cudaMemcpy2DAsync(w.hw, nd * 8, w.h, maxb * 8, nd * 8, nd, cudaMemcpyDeviceToDevice, c->stream));
  launch_add_diag(w.hw, nd, w.ip_dev, nd, c->stream);
  GemmDesc g;  // gw = xs^T b
  g.M = nd; g.N = nset; g.K = n;
  g.A = w.xs; g.a_m = n; g.a_k = 1;
  g.B = b; g.b_k = 1; g.b_n = n;
  g.C = w.gw; g.c_m = 1; g.c_n = nd;
  gemm64(c, g);
  {
    // LU with partial pivoting (2/3 nd^3) and the forward / back substitutions (2 nd^2 nset)
    ProfScope ps(c, PROF_KRYLOV, (2.0 / 3.0) * nd * nd * nd + 2.0 * nd * nd * nset, 8.0 * nd * (nd + nset));
    launch_lu_solve(w.hw, nd, w.gw, nd, nd, nset, w.info, c->stream);
  }
  int info = 0;
  CPHF_CUDA(cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GemmDesc x;  // x_out (+)= xs c
  x.M = n; x.N = nset; x.K = nd;
  x.A = w.xs; x.a_m = 1; x.a_k = n;
  x.B = w.gw; x.b_k = 1; x.b_n = nd;
  x.C = x_out; x.c_m = 1; x.c_n = n;
  x.beta = accumulate ? 1.0 : 0.0;
  gemm64(c, x);
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  if (info != 0) throw Error(CPHF_ERR_NONFINITE, "singular projected Krylov system (zero pivot " + std::to_string(info) + ")");
}

}  // namespace

bool krylov_device(cphf_ctx* c, const DeviceOp& aop, const double* b, const double* x0, int64_t n,
                   int64_t nset, const KrylovParams& p, double* x, cphf_stats* st) {
  const int64_t maxb = nset * (p.max_space + 1);
  c->k_xs.ensure((size_t)n * maxb * 8, c->counter());
  c->k_ax.ensure((size_t)n * maxb * 8, c->counter());
  c->k_h.ensure((size_t)maxb * maxb * 8, c->counter());
  c->k_hw.ensure((size_t)maxb * maxb * 8 + (size_t)maxb * nset * 8, c->counter());
  c->k_b.ensure((size_t)n * nset * 8, c->counter());
  c->k_xacc.ensure((size_t)n * nset * 8, c->counter());
  c->k_x1.ensure((size_t)n * nset * 8, c->counter());
  c->k_coef.ensure((size_t)maxb * nset * 8, c->counter());
  c->k_ip.ensure((size_t)maxb * 8, c->counter());
  c->k_part.ensure((size_t)(mgs_partials_size(n, nset) + 2 * nset + 8) * 8, c->counter());
  c->k_keep.ensure((size_t)std::max<int64_t>(nset, 1) * sizeof(int), c->counter());
  c->k_idx.ensure((size_t)std::max<int64_t>(nset, 1) * sizeof(int), c->counter());
  c->k_info.ensure(sizeof(int), c->counter());
  KrylovWork w;
  w.xs = c->k_xs.as<double>();
  w.ax = c->k_ax.as<double>();
  w.h = c->k_h.as<double>();
  w.hw = c->k_hw.as<double>();
  w.gw = w.hw + maxb * maxb;
  w.bres = c->k_b.as<double>();
  w.xacc = c->k_xacc.as<double>();
  w.x1 = c->k_x1.as<double>();
  w.coef = c->k_coef.as<double>();
  w.ip_dev = c->k_ip.as<double>();
  w.part = c->k_part.as<double>();
  w.keep = c->k_keep.as<int>();
  w.idx = c->k_idx.as<int>();
  w.info = c->k_info.as<int>();
  cudaStream_t s = c->stream;

  int64_t calls = 0, cols = 0;
  auto apply = [&](const double* xin, int64_t nb, double* yout) {
    ++calls;
    cols += nb;
    aop(xin, nb, yout);
  };

  if (x0) CPHF_CUDA(cudaMemcpyAsync(w.xacc, x0, n * nset * 8, cudaMemcpyDeviceToDevice, s));
  else CPHF_CUDA(cudaMemsetAsync(w.xacc, 0, n * nset * 8, s));

  const double conv_thresh = std::max(p.lindep, p.tol * p.tol);
  int64_t total_cycles = 0, restart_idx = 0, last_nd = 0, nd = 0;
  double last_max_ip = 0.0;
  std::vector<double> all_ip;
  std::vector<int> keep;
  std::vector<double> ip;
  std::vector<int> sel;
  std::vector<double> cur_ip;  // squared norms of the block about to be applied

  while (total_cycles < p.max_cycle) {
    // krylov_block.rs:86-87
    if (restart_idx == 0 && x0 == nullptr) {
      CPHF_CUDA(cudaMemcpyAsync(w.bres, b, n * nset * 8, cudaMemcpyDeviceToDevice, s));
    } else {
      apply(w.xacc, nset, w.x1);
      c->k_norm.ensure((size_t)(nset + residual_partials_size(n, nset)) * 8, c->counter());
      launch_residual_norms(b, w.xacc, w.x1, w.bres, n, nset, c->k_norm.as<double>(),
                            c->k_norm.as<double>() + nset, s);
    }
    // orth_block(b_residual) -> x1 (krylov_block.rs:90); works on a copy in ax scratch
    CPHF_CUDA(cudaMemcpyAsync(w.x1, w.bres, n * nset * 8, cudaMemcpyDeviceToDevice, s));
    orth_block(c, w, w.x1, n, nset, p.lindep, keep, ip);
    sel.clear();
    cur_ip.clear();
    for (int64_t i = 0; i < nset; ++i)
      if (keep[i]) { sel.push_back((int)i); cur_ip.push_back(ip[i]); }
    if (sel.empty()) {
      last_nd = 0;
      break;
    }
    select_cols(c, w, w.x1, n, sel, w.xs);  // block lives at xs[:, 0:nblock]
    all_ip.clear();
    nd = 0;
    bool converged = false;
    for (int64_t inner = 0; inner < p.max_space; ++inner) {
      if (total_cycles >= p.max_cycle) break;
      ++total_cycles;
      const int64_t nblock = (int64_t)cur_ip.size();
      double* xnew = w.xs + n * nd;
      double* axnew = w.ax + n * nd;
      apply(xnew, nblock, axnew);  // krylov_block.rs:111-114
      all_ip.insert(all_ip.end(), cur_ip.begin(), cur_ip.end());
      CPHF_CUDA(cudaMemcpyAsync(w.ip_dev + nd, cur_ip.data(), nblock * 8, cudaMemcpyHostToDevice, s));
      const int64_t nd_old = nd;
      nd += nblock;
      // h[:nd, nd_old:nd] = xs^T axt  (also the unscaled projection coefficients)
      GemmDesc g;
      g.M = nd; g.N = nblock; g.K = n;
      g.A = w.xs; g.a_m = n; g.a_k = 1;
      g.B = axnew; g.b_k = 1; g.b_n = n;
      g.C = w.h + maxb * nd_old; g.c_m = 1; g.c_n = maxb;
      gemm64(c, g);
      if (nd_old > 0) {  // h[nd_old:nd, :nd_old] = xs_new^T ax_old
        GemmDesc r;
        r.M = nblock; r.N = nd_old; r.K = n;
        r.A = xnew; r.a_m = n; r.a_k = 1;
        r.B = w.ax; r.b_k = 1; r.b_n = n;
        r.C = w.h + nd_old; r.c_m = 1; r.c_n = maxb;
        gemm64(c, r);
      }
      // coeffs = (xs^T axt) / ip ; x1_new = axt - xs coeffs   (krylov_block.rs:119-122)
      CPHF_CUDA(cudaMemcpy2DAsync(w.coef, nd * 8, w.h + maxb * nd_old, maxb * 8, nd * 8, nblock,
                                  cudaMemcpyDeviceToDevice, s));
      launch_scale_rows(w.coef, nd, w.ip_dev, nd, nblock, s);
      CPHF_CUDA(cudaMemcpyAsync(w.x1, axnew, n * nblock * 8, cudaMemcpyDeviceToDevice, s));
      GemmDesc pr;
      pr.M = n; pr.N = nblock; pr.K = nd;
      pr.A = w.xs; pr.a_m = 1; pr.a_k = n;
      pr.B = w.coef; pr.b_k = 1; pr.b_n = nd;
      pr.C = w.x1; pr.c_m = 1; pr.c_n = n;
      pr.alpha = -1.0; pr.beta = 1.0;
      gemm64(c, pr);
      // MGS of the new directions; convergence on the unfiltered max (krylov_block.rs:127-131)
      orth_block(c, w, w.x1, n, nblock, p.lindep, keep, ip);
      double max_ip = 0.0;
      sel.clear();
      cur_ip.clear();
      for (int64_t i = 0; i < nblock; ++i) {
        if (!keep[i]) continue;
        max_ip = std::max(max_ip, ip[i]);
        if (ip[i] > conv_thresh) { sel.push_back((int)i); cur_ip.push_back(ip[i]); }
      }
      if (p.verbose)
        std::printf("restart %lld inner %lld (total cycle %lld): max(||v||^2) = %.3e, max(||v||) = %.3e, per-elem L2 = %.3e\n",
                    (long long)restart_idx, (long long)inner + 1, (long long)total_cycles, max_ip,
                    std::sqrt(max_ip), std::sqrt(max_ip / (double)n));
      last_max_ip = max_ip;
      if (max_ip < conv_thresh) {
        converged = true;
        break;
      }
      if (nd + (int64_t)sel.size() > maxb) throw Error(CPHF_ERR_STATE, "Krylov slab overflow");
      select_cols(c, w, w.x1, n, sel, w.xs + n * nd);
    }
    last_nd = nd;
    if (converged || total_cycles >= p.max_cycle) break;
    // hard restart (krylov_block.rs:170-175)
    projected_solve(c, w, n, nd, maxb, nset, w.bres, w.xacc, true);
    ++restart_idx;
    if (p.verbose) std::printf("---- restart %lld: x_accum refined, subspace reset ----\n", (long long)restart_idx);
  }

  // final projected solve (krylov_block.rs:179-184)
  CPHF_CUDA(cudaMemcpyAsync(x, w.xacc, n * nset * 8, cudaMemcpyDeviceToDevice, s));
  if (last_nd > 0) projected_solve(c, w, n, last_nd, maxb, nset, w.bres, x, true);
  CPHF_CUDA(cudaStreamSynchronize(s));
  if (st) {
    st->aop_calls += calls;
    st->aop_columns += cols;
    st->cycles += total_cycles;
    st->restarts += restart_idx;
    st->max_innerprod = last_max_ip;
  }
  return last_max_ip < conv_thresh;
}

}  // namespace cphf
