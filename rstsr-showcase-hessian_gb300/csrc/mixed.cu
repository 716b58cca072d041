// Split-precision CPHF operator and the FP64 defect-correction solve.
//
// The operator is the same sequence of contractions as the FP64 path (rijk.cu, xc.cu,
// operator.cu) with FP32 operands and accumulation; the dominant K-term contraction
// B_P bra O_P runs on the tensor cores as a three-product split-FP16 GEMM with FP32
// accumulation in TMEM (tc_gemm.cu).  Its error (~1e-6 relative) is removed by defect
// correction: each step solves (I + A_lowp) d = r with the device Krylov solver (FP64
// basis, orthogonalisation and projected solve), then recomputes r = b - (I + A) x with
// an FP64-accurate operator (exact BF16 slice products on the tensor cores plus
// double-float GEMMs by default, or native FP64), until max_j ||r_j||_2 < residual_tol.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "tc_gemm.cuh"
#include "tc_ozaki.cuh"
#include "xc_gga.cuh"
#include "xc_grouped.cuh"
#include "xc_tc.cuh"

namespace cphf {


void lowp_release(cphf_ctx* c) { c->lowp.reset(); }

void lowp_prepare(cphf_ctx* c) {
  if (!c->lowp) c->lowp.reset(new LowpState());
  LowpState& L = *c->lowp;
  const int64_t nao = c->nao, naux = c->naux;
  L.err.ensure(sizeof(int), c->counter());
  CPHF_CUDA(cudaMemsetAsync(L.err.p, 0, sizeof(int), c->stream));
  if (c->has_rijk) {
    // tc_available / oz_available also set the kernels' shared-memory limits
    L.use_tc = c->cfg.tensor_cores != 0 && tc_available(c) && oz_available(c);
    if (L.use_tc) {
      tc_prepare_cderi(c, L.Bhi, L.Blo, L.ldk);
    } else {
      L.Bd32.ensure((size_t)nao * nao * naux * 4, c->counter());
      launch_to_f32(c->Bd.as<double>(), nao * nao * naux, L.Bd32.as<float>(), c->stream);
    }
  }
  for (int s = 0; s < c->nspin; ++s) {
    SpinState& sp = c->spin[s];
    sp.C32.ensure((size_t)nao * sp.nmo * 4, c->counter());
    launch_to_f32(sp.C.as<double>(), nao * sp.nmo, sp.C32.as<float>(), c->stream);
    if (c->has_rijk) {
      sp.Z32.ensure((size_t)nao * sp.nocc * naux * 4, c->counter());
      launch_to_f32(sp.Z.as<double>(), nao * sp.nocc * naux, sp.Z32.as<float>(), c->stream);
      sp.O32.ensure((size_t)sp.nocc * sp.nocc * naux * 4, c->counter());
      launch_to_f32(sp.O.as<double>(), sp.nocc * sp.nocc * naux, sp.O32.as<float>(), c->stream);
    }
    if (c->has_xc && c->xc_den == 0) {
      sp.aobra32.ensure((size_t)c->ngrids * std::max<int64_t>(sp.nocc, 1) * 4, c->counter());
      launch_to_f32(sp.aobra.as<double>(), c->ngrids * sp.nocc, sp.aobra32.as<float>(), c->stream);
    }
  }
  if (c->has_xc && c->xc_den == 0) {
    const int64_t tot = c->phi.bytes / 8;
    L.phi32.ensure((size_t)std::max<int64_t>(tot, 1) * 4, c->counter());
    launch_to_f32(c->phi.as<double>(), tot, L.phi32.as<float>(), c->stream);
  }
  if (c->has_xc && c->xc_den != 0) {  // GGA / meta-GGA: FP32 copies of phi and phi_c Cocc
    const int64_t tot = c->ngrids * c->nao * 4;
    L.phiG32.ensure((size_t)std::max<int64_t>(tot, 1) * 4, c->counter());
    launch_to_f32(c->phiG.as<double>(), tot, L.phiG32.as<float>(), c->stream);
    for (int s = 0; s < c->nspin; ++s) {
      SpinState& sp = c->spin[s];
      const int64_t n4 = c->ngrids * sp.nocc * 4;
      sp.aobG32.ensure((size_t)std::max<int64_t>(n4, 1) * 4, c->counter());
      launch_to_f32(sp.aobG.as<double>(), n4, sp.aobG32.as<float>(), c->stream);
    }
  }
  // Chunk budget of the K term's T / W intermediates: up to 8 GiB, at most a quarter of the
  // memory still free once the resident operand planes are in place (fewer, longer launches).
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
    L.budget = std::max<int64_t>(int64_t(256) << 20, std::min<int64_t>(int64_t(8) << 30, (int64_t)(free_b / 4)));
  else
    cudaGetLastError();
}

static int64_t k_chunk_lowp(const cphf_ctx* c, int64_t no, int64_t nb) {
  if (c->cfg.aux_chunk > 0) return std::min<int64_t>(c->cfg.aux_chunk, c->naux);
  const int64_t per = c->nao * no * nb * 4;
  int64_t np = std::max<int64_t>(1, (int64_t(1) << 30) / std::max<int64_t>(per, 1));
  np = std::min<int64_t>(np, std::max<int64_t>(1, 65535 / std::max<int64_t>(nb, 1)));
  return std::min<int64_t>(np, c->naux);
}

static void rijk_response_lowp(cphf_ctx* c, float* const* bra, int64_t nb, float* const* out) {
  LowpState& L = *c->lowp;
  const int64_t nao = c->nao, naux = c->naux;
  const int ns = c->nspin;
  bool written[2] = {false, false};
  if (c->scale_j != 0.0) {
    L.s_d.ensure((size_t)naux * nb * 4, c->counter());
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      if (no == 0) {
        if (s == 0) CPHF_CUDA(cudaMemsetAsync(L.s_d.p, 0, (size_t)naux * nb * 4, c->stream));
        continue;
      }
      GemmDesc d;
      d.M = naux; d.N = nb; d.K = nao * no;
      d.A = c->spin[s].Z32.p; d.a_m = nao * no; d.a_k = 1;
      d.B = bra[s]; d.b_k = 1; d.b_n = nao * no;
      d.C = L.s_d.p; d.c_m = 1; d.c_n = naux;
      d.alpha = 2.0; d.beta = s == 0 ? 0.0 : 1.0;
      gemm32(c, d);
    }
    const double jfac = ns == 1 ? c->scale_j : 0.5 * c->scale_j;
    for (int s = 0; s < ns; ++s) {
      const int64_t no = c->spin[s].nocc;
      if (no == 0) continue;
      GemmDesc j;
      j.M = nao * no; j.N = nb; j.K = naux;
      j.A = c->spin[s].Z32.p; j.a_m = 1; j.a_k = nao * no;
      j.B = L.s_d.p; j.b_k = 1; j.b_n = naux;
      j.C = out[s]; j.c_m = 1; j.c_n = nao * no;
      j.alpha = 2.0 * jfac; j.beta = 0.0;
      gemm32(c, j);
      written[s] = true;
    }
  }
  if (c->scale_k != 0.0) {
    for (int s = 0; s < ns; ++s) {
      const SpinState& sp = c->spin[s];
      const int64_t no = sp.nocc;
      if (no == 0) continue;
      if (!written[s]) {
        CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * no * nb * 4, c->stream));
        written[s] = true;
      }
      const int64_t np_max = k_chunk_lowp(c, no, nb);
      if (L.use_tc) {
        // the whole K term on the tensor cores (split FP16): term 1 with T made by the batched
        // T-generation kernel, then W-generation and term 2 per chunk
        int* err = L.err.as<int>();
        lp_begin(c, L.lp, s, bra[s], nb);
        tc_k_term1(c, L.Bhi, L.Blo, L.ldk, no, nb, out[s], L.s_Thi, L.s_Tlo,
                   [&](int64_t P0, int64_t npc, __half* hi, __half* lo, unsigned* mx, float* scale) {
                     lp_tgen_planes(c, L.lp, s, P0, npc, nb, L.ldk, hi, lo, mx, scale, (float)L.sA,
                                    (float)-c->scale_k, err);
                   });
        // W / term-2 chunk: W's two FP16 planes, nocc-wide rows, within the budget and with
        // 32-bit plane offsets
        const int64_t ldj = (no + 7) / 8 * 8;
        int64_t np_w = std::max<int64_t>(1, std::min<int64_t>(naux, L.budget / std::max<int64_t>(4 * no * nb * ldj, 1)));
        np_w = std::max<int64_t>(1, std::min<int64_t>(np_w, ((int64_t)INT32_MAX - 1) / std::max<int64_t>(no * nb * ldj, 1)));
        for (int64_t P0 = 0; P0 < naux; P0 += np_w)
          lp_w_term2(c, L.lp, s, P0, std::min<int64_t>(np_w, naux - P0), nb, -c->scale_k, out[s], err);
        continue;
      }
      L.s_T.ensure((size_t)nao * np_max * no * nb * 4, c->counter());
      L.s_W.ensure((size_t)no * np_max * no * nb * 4, c->counter());
      for (int64_t P0 = 0; P0 < naux; P0 += np_max) {
        const int64_t np = std::min<int64_t>(np_max, naux - P0);
        {
          // T[(nu,Pl),(i,a)]: rows (nu, a) two-level, columns i, batch over P
          GemmDesc t;
          t.M = nao * nb; t.N = no; t.K = no; t.batch1 = np;
          t.A = bra[s]; t.a_m = 1; t.m_div = nao; t.a_m2 = nao * no; t.a_k = nao; t.a_b1 = 0;
          t.B = sp.O32.as<float>() + P0 * no * no; t.b_k = 1; t.b_n = no; t.b_b1 = no * no;
          t.C = L.s_T.p; t.c_m = 1; t.c_m2 = nao * np * no; t.c_n = nao * np; t.c_b1 = nao;
          gemm32(c, t);
          GemmDesc k1;
          k1.M = nao; k1.N = no * nb; k1.K = nao * np;
          k1.A = L.Bd32.as<float>() + P0 * nao * nao; k1.a_m = 1; k1.a_k = nao;
          k1.B = L.s_T.p; k1.b_k = 1; k1.b_n = nao * np;
          k1.C = out[s]; k1.c_m = 1; k1.c_n = nao;
          k1.alpha = -c->scale_k; k1.beta = 1.0;
          gemm32(c, k1);
        }
        // Wt[(j,Pl),(i,a)] = sum_nu bra[nu, (j,a)] Z_P[nu, i]: rows (j, a) two-level in the
        // output, columns i, K = nu, batch over P
        GemmDesc w;
        w.M = no * nb; w.N = no; w.K = nao; w.batch1 = np;
        w.A = bra[s]; w.a_m = nao; w.a_k = 1; w.a_b1 = 0;
        w.B = sp.Z32.as<float>() + P0 * nao * no; w.b_k = 1; w.b_n = nao; w.b_b1 = nao * no;
        w.C = L.s_W.p; w.m_div = no; w.a_m2 = nao * no; w.c_m = 1; w.c_m2 = no * np * no; w.c_n = no * np;
        w.c_b1 = no;
        gemm32(c, w);
        GemmDesc k2;
        k2.M = nao; k2.N = no * nb; k2.K = no * np;
        k2.A = sp.Z32.as<float>() + P0 * nao * no; k2.a_m = 1; k2.a_k = nao;
        k2.B = L.s_W.p; k2.b_k = 1; k2.b_n = no * np;
        k2.C = out[s]; k2.c_m = 1; k2.c_n = nao;
        k2.alpha = -c->scale_k; k2.beta = 1.0;
        gemm32(c, k2);
      }
    }
  }
  for (int s = 0; s < ns; ++s)
    if (!written[s] && c->spin[s].nocc > 0)
      CPHF_CUDA(cudaMemsetAsync(out[s], 0, (size_t)nao * c->spin[s].nocc * nb * 4, c->stream));
}

static void xc_response_lowp(cphf_ctx* c, float* const* bra, int64_t nb, float* const* out, bool accumulate) {
  LowpState& L = *c->lowp;
  if (c->xc_den != 0) {  // GGA / meta-GGA on the CUDA cores in FP32
    const float* aob[2] = {c->spin[0].aobG32.as<float>(), c->nspin > 1 ? c->spin[1].aobG32.as<float>() : nullptr};
    xc_response_gga<float>(c, bra, nb, out, accumulate, L.phiG32.as<float>(), aob, L.s_gket, L.s_grho);
    return;
  }
  if (L.use_tc) {
    xc_response_tc(c, bra, nb, out, accumulate);
    return;
  }
  const float* aobra[2] = {c->spin[0].aobra32.as<float>(), c->nspin > 1 ? c->spin[1].aobra32.as<float>() : nullptr};
  xc_response_grouped<float>(c, bra, nb, out, accumulate, L.phi32.as<float>(), aobra, L.s_ket, L.s_rho);
}

void response_mo_lowp(cphf_ctx* c, const double* x, int64_t nb, double* y, bool check) {
  LowpState& L = *c->lowp;
  const int ns = c->nspin;
  const int64_t nao = c->nao, n = krylov_n(c);
  int64_t tot_occ = 0, max_occ = 0, max_nmo = 0;
  for (int s = 0; s < ns; ++s) {
    tot_occ += c->spin[s].nocc;
    max_occ = std::max(max_occ, c->spin[s].nocc);
    max_nmo = std::max(max_nmo, c->spin[s].nmo);
  }
  L.s_c1.ensure((size_t)nao * tot_occ * nb * 4, c->counter());
  L.s_resp.ensure((size_t)nao * tot_occ * nb * 4, c->counter());
  L.s_y.ensure((size_t)max_nmo * max_occ * nb * 4, c->counter());
  if (ns == 2) L.s_x.ensure((size_t)n * nb * 8, c->counter());
  float* c1[2] = {nullptr, nullptr};
  float* rb[2] = {nullptr, nullptr};
  const double* xs[2] = {nullptr, nullptr};
  int64_t off_occ = 0, off_x = 0;
  for (int s = 0; s < ns; ++s) {
    const SpinState& sp = c->spin[s];
    c1[s] = L.s_c1.as<float>() + nao * off_occ * nb;
    rb[s] = L.s_resp.as<float>() + nao * off_occ * nb;
    off_occ += sp.nocc;
    const int64_t len = sp.nmo * sp.nocc;
    if (ns == 1) {
      xs[s] = x;
    } else {
      double* dst = L.s_x.as<double>() + off_x * nb;
      if (len > 0)
        CPHF_CUDA(cudaMemcpy2DAsync(dst, len * 8, x + off_x, n * 8, len * 8, nb, cudaMemcpyDeviceToDevice, c->stream));
      xs[s] = dst;
    }
    off_x += len;
    if (sp.nocc == 0) continue;
    GemmDesc d;
    d.M = nao; d.N = sp.nocc * nb; d.K = sp.nmo;
    d.A = sp.C32.p; d.a_m = 1; d.a_k = nao;
    d.B = xs[s]; d.b_k = 1; d.b_n = sp.nmo;
    d.C = c1[s]; d.c_m = 1; d.c_n = nao;
    gemm32x<float, double, float>(c, d);
  }
  bool acc = false;
  if (c->has_rijk) { rijk_response_lowp(c, c1, nb, rb); acc = true; }
  if (c->has_xc) { xc_response_lowp(c, c1, nb, rb, acc); acc = true; }
  off_x = 0;
  for (int s = 0; s < ns; ++s) {
    const SpinState& sp = c->spin[s];
    const int64_t no = sp.nocc, nmo = sp.nmo, nvir = nmo - no;
    double* yo = y + off_x;
    off_x += nmo * no;
    if (no == 0) continue;
    if (nvir > 0) {
      GemmDesc d;
      d.M = nvir; d.N = no * nb; d.K = nao;
      d.A = sp.C32.as<float>() + no * nao; d.a_m = nao; d.a_k = 1;
      d.B = rb[s]; d.b_k = 1; d.b_n = nao;
      d.C = L.s_y.p; d.c_m = 1; d.c_n = nvir;
      gemm32(c, d);
    }
    launch_dimless_f32(L.s_y.as<float>(), xs[s], ns == 1 ? n : nmo * no, sp.e.as<double>(), nmo, no, nb,
                       c->cfg.level_shift, yo, n, c->stream);
  }
  if (check) lowp_check(c);
}

void lowp_check(cphf_ctx* c) {
  LowpState& L = *c->lowp;
  if (L.use_tc && c->has_rijk) {
    int flag = 0;
    CPHF_CUDA(cudaMemcpyAsync(&flag, L.err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    if (flag) throw Error(CPHF_ERR_TIMEOUT, "tensor-core K-term kernel: a bounded pipeline wait expired");
  }
}

// The split-precision operator as the inner solves apply it.  With cfg.cuda_graphs each block
// width nb is captured once into a CUDA graph that reads the staging buffer g_x and writes
// g_y; later applications copy x in, replay the graph and copy y out.  A graph is replayed
// only while the buffer / plan generation it was captured at is current (it bakes in
// pointers and plan contents); the first application of a width, and any application after
// the generation moved, runs eagerly (warming every buffer and plan) and then captures.
void lowp_apply(cphf_ctx* c, const double* x, int64_t nb, double* y) {
  LowpState& L = *c->lowp;
  if (!c->cfg.cuda_graphs || L.graphs_off || c->prof.on) {
    response_mo_lowp(c, x, nb, y);
    return;
  }
  const int64_t n = krylov_n(c);
  const size_t bytes = (size_t)n * nb * 8;
  L.g_x.ensure(bytes, c->counter());
  L.g_y.ensure(bytes, c->counter());
  const int64_t gen = state_generation();
  for (auto& g : L.graphs) {
    if (g.nb != nb || g.gen != gen) continue;
    CPHF_CUDA(cudaMemcpyAsync(L.g_x.p, x, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CPHF_CUDA(cudaGraphLaunch(g.exec, c->stream));
    CPHF_CUDA(cudaMemcpyAsync(y, L.g_y.p, bytes, cudaMemcpyDeviceToDevice, c->stream));
    count_launch(g.nodes);
    lowp_check(c);
    return;
  }
  // stale or missing: drop graphs of older generations, run eagerly, then capture this width
  std::vector<OpGraph> keep;
  for (auto& g : L.graphs) {
    if (g.gen == gen) keep.push_back(g);
    else if (g.exec) cudaGraphExecDestroy(g.exec);
  }
  L.graphs.swap(keep);
  response_mo_lowp(c, x, nb, y);
  const int64_t gen0 = state_generation();
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    try {
      response_mo_lowp(c, L.g_x.as<double>(), nb, L.g_y.as<double>(), false);
    } catch (...) {
      ok = false;
    }
    const bool ended = cudaStreamEndCapture(c->stream, &graph) == cudaSuccess;
    ok = ok && ended && graph && state_generation() == gen0;
  }
  size_t nodes = 0, kernels = 0;
  if (ok) ok = cudaGraphGetNodes(graph, nullptr, &nodes) == cudaSuccess;
  if (ok && nodes > 0) {
    std::vector<cudaGraphNode_t> list(nodes);
    ok = cudaGraphGetNodes(graph, list.data(), &nodes) == cudaSuccess;
    for (size_t i = 0; ok && i < nodes; ++i) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(list[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  if (!ok) {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    L.graphs_off = true;  // run eagerly from now on
    return;
  }
  OpGraph g;
  g.nb = nb;
  g.gen = gen0;
  g.nodes = (int64_t)kernels;
  g.exec = exec;
  L.graphs.push_back(g);
}

AccurateScope::AccurateScope(cphf_ctx* ctx, int mode, int correction_slices) : c(ctx) {
  const bool tc = c->lowp && c->lowp->use_tc && oz_available(c);
  c->f64_emulate = mode != 0;
  c->oz_kterm = mode == 2 && c->has_rijk && tc && oz_supported(c);
  c->oz_xc = mode == 2 && c->has_xc && c->xc_den == 0 && tc;  // the tensor-core XC covers LDA
  c->oz_correction = (c->oz_kterm || c->oz_xc) ? correction_slices : 0;
  c->f32_correction = c->oz_correction != 0;  // the correction's J, C x and C^T r GEMMs to ~1e-7 of it
  // mode 2 without any tensor-core contraction available is the double-float operator
  used = mode == 2 && !(c->oz_kterm || c->oz_xc) ? 1 : mode;
}

AccurateScope::~AccurateScope() {
  c->f64_emulate = false;
  c->oz_kterm = false;
  c->oz_xc = false;
  c->oz_correction = 0;
  c->f32_correction = false;
}

bool solve_mixed(cphf_ctx* c, const double* b, const double* x0, int64_t nset, double* x, cphf_stats* st,
                 const double* m) {
  if (!c->lowp) lowp_prepare(c);
  const int64_t n = krylov_n(c);
  // refinement vectors r, rr (scaled residual), d (correction), FP64
  DevBuf& buf = c->k_r;
  buf.ensure((size_t)n * nset * 8 * 4, c->counter());
  double* r = buf.as<double>();
  double* rr = r + n * nset;
  double* dlt = rr + n * nset;
  double* adl = dlt + n * nset;
  // a learned left preconditioner m acts on the inner solves only: m (I + A_lowp) d = m r
  cudaStream_t s = c->stream;
  CPHF_CUDA(cudaMemsetAsync(x, 0, n * nset * 8, s));
  CPHF_CUDA(cudaMemcpyAsync(r, b, n * nset * 8, cudaMemcpyDeviceToDevice, s));
  // column norms of b
  c->k_norm.ensure((size_t)(nset + residual_partials_size(n, nset)) * 8, c->counter());
  std::vector<double> h(nset);
  {
    CPHF_CUDA(cudaMemsetAsync(dlt, 0, n * nset * 8, s));
    launch_residual_norms(b, dlt, dlt, rr, n, nset, c->k_norm.as<double>(), c->k_norm.as<double>() + nset, s);
    CPHF_CUDA(cudaMemcpyAsync(h.data(), c->k_norm.p, nset * 8, cudaMemcpyDeviceToHost, s));
    CPHF_CUDA(cudaStreamSynchronize(s));
  }
  double res = 0.0;
  for (double v : h) res = std::max(res, std::sqrt(v));
  const KrylovParams p{c->cfg.inner_tol, c->cfg.cphf_lindep, c->cfg.cphf_max_cycle, c->cfg.cphf_max_space,
                       c->cfg.verbose != 0};
  // The learned left preconditioner m acts on the first inner solve (step 0) only: the later
  // corrections solve the plain operator, so that their stopping test is on the residual
  // itself (a test on m r bounds the residual only up to max |m| / min |m|).
  bool use_m = m != nullptr;
  bool loosen = true, loosened = false;
  DeviceOp op = [&](const double* xin, int64_t nb, double* yout) {
    lowp_apply(c, xin, nb, yout);
    if (use_m) launch_apply_precond(m, xin, yout, n, nb, c->stream);
    st->lowp_matvec_columns += nb;
  };
  // Defect correction.  Step 0 solves with the full right-hand side; its residual is the one
  // that must be exact, so it is recomputed with the FP64-accurate operator (residual_dfloat):
  // r1 = b - (I + A) x1.  With verify_residual on (1 native FP64, 2 the residual_dfloat
  // operator) every later residual is recomputed the same way and convergence is decided only
  // on a recomputed residual, so the solve measures its own final ||b - (I+A)x||.  With it off,
  // later corrections d are O(|r1|) and the update r -= (I + A_lowp) d carries an error of
  // only eps_lowp |d| ~ eps_lowp^2 |b|, far below the tolerance.
  auto accurate_residual = [&](int mode) {
    AccurateScope scope(c, mode);
    res = fp64_residual(c, b, x, nset, r, st);
    st->residual_mode = scope.used;
  };
  const int first_mode = c->cfg.residual_dfloat;
  const int final_mode = c->cfg.verify_residual == 1 ? 0 : c->cfg.verify_residual == 2 ? first_mode : -1;
  const double update_margin = 0.5;
  bool done = res < c->cfg.residual_tol;
  st->residual_mode = 0;  // |b| itself is exact
  for (int64_t step = 0; step < c->cfg.max_refine && !done; ++step) {
    // solve (I + A_lowp) d' = r / |r|  (relative tolerances), d = |r| d'
    const double scale = res > 0.0 ? res : 1.0;
    launch_axpby(1.0 / scale, r, 0.0, rr, n * nset, s);
    use_m = m != nullptr && step == 0;
    if (use_m) launch_scale_rows_by(m, rr, rr, n, nset, s);
    const double* g0 = nullptr;
    if (step == 0 && x0) {
      launch_axpby(1.0 / scale, x0, 0.0, adl, n * nset, s);  // initial guess in scaled units
      g0 = adl;
    }
    // the inner solve's Gram / projection GEMMs in double-float (its operator is ~1e-6 accurate)
    c->f64_emulate = c->cfg.residual_dfloat != 0;
    try {
      // Later corrections need only bring the residual below the target: relative tolerance
      // 0.1 residual_tol / |r| (within [inner_tol, 1e-2]) instead of inner_tol.  At nao 600-800
      // this saves the second inner cycle of step 1 (one operator application of six); the
      // final residual then sits ~1e-10 instead of ~1e-11, still 100x below the target.  A
      // loosened step that does not reach the target turns the loosening off for the rest of
      // the solve.
      KrylovParams pk = p;
      loosened = step > 0 && res > 0.0 && loosen;
      if (loosened) pk.tol = std::max(c->cfg.inner_tol, std::min(1e-2, 0.1 * c->cfg.residual_tol / res));
      krylov_device(c, op, rr, g0, n, nset, pk, dlt, st);
    } catch (...) {
      c->f64_emulate = false;
      throw;
    }
    c->f64_emulate = false;
    launch_axpby(scale, dlt, 0.0, dlt, n * nset, s);
    launch_axpby(1.0, dlt, 1.0, x, n * nset, s);
    st->refine_steps += 1;
    const char* how;
    if (step > 0 && c->cfg.verify_residual == 2 && first_mode == 2 && !c->cfg.fp64_every_step &&
        st->residual_mode != 3) {
      // r -= (I + A) d with the exact-slice operator in correction precision: d solves
      // (I + A) d = r, so |(I + A) d| ~ |r|, and an operator accurate to eps relative to |A| |d|
      // adds ~eps |r| (with a margin of 4 for |A| |(I + A)^-1|; measured: ~2^-19 |r| with 3
      // slices).  The fewest slices whose error stays below a tenth of residual_tol: 3 (6
      // exact-accumulated products, eps ~2^-16), 4 (10, ~2^-22), else all six; r stays a
      // computed residual, not a split-precision estimate.
      const double tenth = 0.1 * c->cfg.residual_tol;
      const int slices = res * 0x1p-14 <= tenth ? 3 : res * 0x1p-20 <= tenth ? 4 : 0;
      int used = 0;
      {
        AccurateScope scope(c, 2, slices);
        response_mo_fp64(c, dlt, nset, adl, true);
        used = scope.used;
      }
      st->fp64_matvec_columns += nset;
      launch_residual_norms(r, dlt, adl, r, n, nset, c->k_norm.as<double>(), c->k_norm.as<double>() + nset, s);
      CPHF_CUDA(cudaMemcpyAsync(h.data(), c->k_norm.p, nset * 8, cudaMemcpyDeviceToHost, s));
      CPHF_CUDA(cudaStreamSynchronize(s));
      res = 0.0;
      for (double v : h) res = std::max(res, std::sqrt(v));
      if (!std::isfinite(res)) throw Error(CPHF_ERR_NONFINITE, "non-finite residual");
      st->residual_mode = used == 2 ? 4 : used;
      done = res < c->cfg.residual_tol;
      how = "exact-slice correction update";
    } else if (step == 0 || c->cfg.fp64_every_step || final_mode >= 0) {
      const int mode = (step == 0 || final_mode < 0) ? first_mode : final_mode;
      accurate_residual(mode);
      done = res < c->cfg.residual_tol;
      if (done && final_mode >= 0 && mode != final_mode) {
        // converged on the first correction's operator: confirm with the final-check operator
        accurate_residual(final_mode);
        done = res < c->cfg.residual_tol;
      }
      how = "recomputed";
    } else {
      lowp_apply(c, dlt, nset, adl);
      st->lowp_matvec_columns += nset;
      launch_residual_norms(r, dlt, adl, r, n, nset, c->k_norm.as<double>(), c->k_norm.as<double>() + nset, s);
      CPHF_CUDA(cudaMemcpyAsync(h.data(), c->k_norm.p, nset * 8, cudaMemcpyDeviceToHost, s));
      CPHF_CUDA(cudaStreamSynchronize(s));
      res = 0.0;
      for (double v : h) res = std::max(res, std::sqrt(v));
      if (!std::isfinite(res)) throw Error(CPHF_ERR_NONFINITE, "non-finite residual");
      st->residual_mode = 3;
      done = res < update_margin * c->cfg.residual_tol;
      how = "updated";
    }
    if (loosened && !done) loosen = false;
    if (c->cfg.verbose)
      std::printf("defect correction step %lld: max ||b - (I+A)x|| = %.3e (%s, mode %lld)\n", (long long)step + 1,
                  res, how, (long long)st->residual_mode);
  }
  st->residual_max = res;
  return done;
}

}  // namespace cphf
