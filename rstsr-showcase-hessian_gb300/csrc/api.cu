// C ABI of libcphf (include/cphf.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "decompose.cuh"
#include "kernels.cuh"
#include "mlp.cuh"

using namespace cphf;

namespace {

struct CounterScope {
  int64_t* prev;
  explicit CounterScope(cphf_ctx* c) : prev(g_launch_counter) { g_launch_counter = &c->launches; }
  ~CounterScope() { g_launch_counter = prev; }
};

template <typename F>
cphf_status guarded(cphf_ctx* c, F&& f) {
  if (!c) return CPHF_ERR_ARG;
  try {
    CPHF_CUDA(cudaSetDevice(c->device));
    CounterScope scope(c);
    f();
    c->last_error.clear();
    return CPHF_OK;
  } catch (const Error& e) {
    c->last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    c->last_error = e.what();
    return CPHF_ERR_CUDA;
  }
}

// Copy `bytes` from a host or device pointer into device memory (cudaMemcpyDefault / UVA).
void copy_in(cphf_ctx* c, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return;
  CPHF_CHECK_ARG(src != nullptr, "null input pointer");
  CPHF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
}
void copy_out(cphf_ctx* c, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return;
  CPHF_CHECK_ARG(dst != nullptr, "null output pointer");
  CPHF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
}
// Read a small array from host or device memory into a host vector.
template <typename T>
std::vector<T> read_small(cphf_ctx* c, const T* src, int64_t n) {
  std::vector<T> v(n);
  if (n == 0) return v;
  CPHF_CHECK_ARG(src != nullptr, "null input pointer");
  CPHF_CUDA(cudaMemcpyAsync(v.data(), src, n * sizeof(T), cudaMemcpyDefault, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  return v;
}

void require_prepared(cphf_ctx* c) {
  if (!c->prepared) throw Error(CPHF_ERR_STATE, "cphf_prepare (make_response_preparation) has not been called");
  if (!c->has_rijk && !c->has_xc) throw Error(CPHF_ERR_STATE, "no electron-interaction plugin is set");
}

int64_t bra_elems(cphf_ctx* c, int s, int64_t nprop) { return c->nao * c->spin[s].nocc * nprop; }
int64_t mo_elems(cphf_ctx* c, int s, int64_t nprop) { return c->spin[s].nmo * c->spin[s].nocc * nprop; }

// Staging of spin-resolved arrays into one device buffer; returns per-spin device pointers.
void stage_in(cphf_ctx* c, DevBuf& buf, const double* const* src, const std::vector<int64_t>& elems,
              double* dev[2]) {
  int64_t tot = 0;
  for (int64_t e : elems) tot += e;
  buf.ensure((size_t)std::max<int64_t>(tot, 1) * 8, c->counter());
  int64_t off = 0;
  for (size_t s = 0; s < elems.size(); ++s) {
    dev[s] = buf.as<double>() + off;
    if (src) copy_in(c, dev[s], src[s], elems[s] * 8);
    off += elems[s];
  }
}

// The packed Krylov vector [n, nprop] from per-spin [nmo, nocc_s, nprop] arrays (uscf.rs:292-304).
void pack_krylov(cphf_ctx* c, const double* const* src, int64_t nprop, double* dst) {
  const int64_t n = krylov_n(c);
  int64_t off = 0;
  for (int s = 0; s < c->nspin; ++s) {
    const int64_t len = c->spin[s].nmo * c->spin[s].nocc;
    if (len > 0 && nprop > 0) {
      CPHF_CHECK_ARG(src[s] != nullptr, "null input pointer");
      CPHF_CUDA(cudaMemcpy2DAsync(dst + off, n * 8, src[s], len * 8, len * 8, nprop, cudaMemcpyDefault, c->stream));
    }
    off += len;
  }
}
void unpack_krylov(cphf_ctx* c, const double* src, int64_t nprop, double* const* dst) {
  const int64_t n = krylov_n(c);
  int64_t off = 0;
  for (int s = 0; s < c->nspin; ++s) {
    const int64_t len = c->spin[s].nmo * c->spin[s].nocc;
    if (len > 0 && nprop > 0) {
      CPHF_CHECK_ARG(dst[s] != nullptr, "null output pointer");
      CPHF_CUDA(cudaMemcpy2DAsync(dst[s], len * 8, src + off, n * 8, len * 8, nprop, cudaMemcpyDefault, c->stream));
    }
    off += len;
  }
}

void check_finite(cphf_ctx* c, const double* dev, int64_t n, const char* what) {
  // context-owned counter: no allocation per call
  c->k_finite.ensure(sizeof(int), c->counter());
  CPHF_CUDA(cudaMemsetAsync(c->k_finite.p, 0, sizeof(int), c->stream));
  launch_count_nonfinite(dev, n, c->k_finite.as<int>(), c->stream);
  int bad = 0;
  CPHF_CUDA(cudaMemcpyAsync(&bad, c->k_finite.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  if (bad) throw Error(CPHF_ERR_NONFINITE, std::string("non-finite values in ") + what);
}

}  // namespace

namespace cphf {
// mixed-precision solve (defined in mixed.cu); m: optional left preconditioner of the inner solves
bool solve_mixed(cphf_ctx* c, const double* b, const double* x0, int64_t nset, double* x, cphf_stats* st,
                 const double* m);
}

extern "C" {

cphf_status cphf_config_default(cphf_config* cfg) {
  if (!cfg) return CPHF_ERR_ARG;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->level_shift = 0.0;
  cfg->cphf_tol = 1e-8;
  cfg->cphf_max_cycle = 42;
  cfg->cphf_max_space = 14;
  cfg->cphf_lindep = 1e-14;
  cfg->precision = CPHF_PRECISION_FP64;
  cfg->device = 0;
  cfg->residual_tol = 1e-8;
  cfg->inner_tol = 1e-6;
  cfg->max_refine = 6;
  cfg->use_learned_guess = 0;
  cfg->verbose = 0;
  cfg->aux_chunk = 0;
  cfg->tensor_cores = 1;
  cfg->verify_residual = 2;
  cfg->fp64_every_step = 0;
  cfg->xc_chunk_points = 0;
  cfg->residual_dfloat = 2;
  cfg->cuda_graphs = 1;
  return CPHF_OK;
}

const char* cphf_status_string(cphf_status s) {
  switch (s) {
    case CPHF_OK: return "ok";
    case CPHF_ERR_SHAPE: return "shape mismatch";
    case CPHF_ERR_NOT_CONVERGED: return "krylov_block failed to converge";
    case CPHF_ERR_NONFINITE: return "non-finite value";
    case CPHF_ERR_OOM: return "out of device memory";
    case CPHF_ERR_CUDA: return "CUDA error";
    case CPHF_ERR_TIMEOUT: return "device wait timed out";
    case CPHF_ERR_STATE: return "invalid call order";
    case CPHF_ERR_ARG: return "invalid argument";
  }
  return "unknown status";
}

cphf_status cphf_ctx_create(const cphf_config* cfg, cphf_ctx** out) {
  if (!out) return CPHF_ERR_ARG;
  *out = nullptr;
  cphf_ctx* c = new cphf_ctx();
  if (cfg) c->cfg = *cfg; else cphf_config_default(&c->cfg);
  c->device = c->cfg.device;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return CPHF_ERR_CUDA;
  }
  *out = c;
  return CPHF_OK;
}

cphf_status cphf_ctx_destroy(cphf_ctx* c) {
  if (!c) return CPHF_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  lowp_release(c);
  cudaStream_t s = c->stream;
  delete c;
  if (s) cudaStreamDestroy(s);
  return CPHF_OK;
}

cphf_status cphf_ctx_set_config(cphf_ctx* c, const cphf_config* cfg) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(cfg != nullptr, "null config");
    CPHF_CHECK_ARG(cfg->device == c->device, "the device of a context cannot change");
    const bool was_mixed = c->cfg.precision == CPHF_PRECISION_MIXED;
    c->cfg = *cfg;
    if (c->prepared && !was_mixed && cfg->precision == CPHF_PRECISION_MIXED) lowp_prepare(c);
  });
}

const char* cphf_last_error(const cphf_ctx* c) { return c ? c->last_error.c_str() : "null context"; }
void* cphf_ctx_stream(const cphf_ctx* c) { return c ? (void*)c->stream : nullptr; }
int64_t cphf_ctx_device_bytes(const cphf_ctx* c) { return c ? c->device_bytes : 0; }
int64_t cphf_ctx_kernel_launches(const cphf_ctx* c) { return c ? c->launches : 0; }

int32_t cphf_ctx_tensor_cores_active(const cphf_ctx* c) {
  return (c && c->lowp && c->lowp->use_tc && c->has_rijk) ? 1 : 0;
}

cphf_status cphf_ctx_profile(cphf_ctx* c, int32_t enable) {
  return guarded(c, [&] {
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& r : c->prof.recs) {
      c->prof.pool.push_back(r.start);
      c->prof.pool.push_back(r.stop);
    }
    c->prof.recs.clear();
    c->prof.on = enable != 0;
  });
}

int32_t cphf_ctx_profile_report(cphf_ctx* c, cphf_prof_entry* out, int32_t max) {
  if (!c) return -1;
  int32_t n = 0;
  cphf_status st = guarded(c, [&] {
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    cphf_prof_entry acc[PROF_NCLASS];
    std::memset(acc, 0, sizeof(acc));
    for (const auto& r : c->prof.recs) {
      float ms = 0.f;
      CPHF_CUDA(cudaEventElapsedTime(&ms, r.start, r.stop));
      cphf_prof_entry& e = acc[r.cls];
      e.launches += 1;
      e.ms += ms;
      e.max_ms = std::max(e.max_ms, (double)ms);
      e.flops += r.flops;
      e.bytes += r.bytes;
    }
    for (int k = 0; k < PROF_NCLASS && n < max; ++k) {
      if (acc[k].launches == 0) continue;
      std::strncpy(acc[k].name, kProfNames[k], sizeof(acc[k].name) - 1);
      if (out) out[n] = acc[k];
      ++n;
    }
  });
  return st == CPHF_OK ? n : -1;
}

cphf_status cphf_ctx_synchronize(cphf_ctx* c) {
  return guarded(c, [&] { CPHF_CUDA(cudaStreamSynchronize(c->stream)); });
}

cphf_status cphf_set_nao(cphf_ctx* c, int64_t nao) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(nao > 0, "nao must be positive");
    CPHF_CHECK_SHAPE(!c->has_rijk || c->nao == nao, "nao differs from the cderi's");
    c->nao = nao;
    c->prepared = false;
  });
}

// The packed cderi in c->cderi_tp becomes the RI-JK plugin's B (dense copy, state reset).
static void install_cderi(cphf_ctx* c, int64_t nao, int64_t naux, double scale_j, double scale_k) {
  const int64_t nao_tp = nao * (nao + 1) / 2;
  c->nao = nao;
  c->naux = naux;
  c->scale_j = scale_j;
  c->scale_k = scale_k;
  check_finite(c, c->cderi_tp.as<double>(), nao_tp * naux, "cderi");
  c->Bd.ensure((size_t)nao * nao * naux * 8, c->counter());
  launch_unpack_cderi(c->cderi_tp.as<double>(), nao, naux, c->Bd.as<double>(), c->stream);
  c->has_rijk = true;
  c->prepared = false;
  lowp_release(c);
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
}

cphf_status cphf_rijk_set_cderi(cphf_ctx* c, const double* cderi, int64_t nao, int64_t naux,
                                double scale_j, double scale_k) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(nao > 0 && naux > 0, "nao and naux must be positive");
    CPHF_CHECK_SHAPE(!c->has_xc || c->nao == nao, "nao differs from the XC grid's");
    const int64_t nao_tp = nao * (nao + 1) / 2;
    c->cderi_tp.ensure((size_t)nao_tp * naux * 8, c->counter());
    copy_in(c, c->cderi_tp.p, cderi, (size_t)nao_tp * naux * 8);
    install_cderi(c, nao, naux, scale_j, scale_k);
  });
}

static void fill_j2c_info(cphf_j2c_info* info, const J2cDecomp& d, double t_dec, double t_solve) {
  if (!info) return;
  info->eig_fallback = d.fallback ? 1 : 0;
  info->jacobi_sweeps = d.sweeps;
  info->min_diag = d.min_diag;
  info->seconds_decompose = t_dec;
  info->seconds_solve = t_solve;
}

cphf_status cphf_j2c_decompose(cphf_ctx* c, const double* j2c, int64_t naux, double threshold, double* j2c_u,
                               cphf_j2c_info* info) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(naux > 0, "naux must be positive");
    CPHF_CHECK_ARG(j2c_u != nullptr, "null output");
    DecompWork w;
    DevBuf m;
    m.ensure((size_t)naux * naux * 8, c->counter());
    copy_in(c, m.p, j2c, (size_t)naux * naux * 8);
    check_finite(c, m.as<double>(), naux * naux, "j2c");
    const auto t0 = std::chrono::steady_clock::now();
    const J2cDecomp d = j2c_cholesky(c, m.as<double>(), naux, threshold, w);
    const double t_dec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    copy_out(c, j2c_u, w.U.p, (size_t)naux * naux * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    fill_j2c_info(info, d, t_dec, 0.0);
  });
}

cphf_status cphf_rijk_set_j3c(cphf_ctx* c, const double* j3c, const double* j2c, int64_t nao, int64_t naux,
                              double scale_j, double scale_k, double threshold, cphf_j2c_info* info) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(nao > 0 && naux > 0, "nao and naux must be positive");
    CPHF_CHECK_SHAPE(!c->has_xc || c->nao == nao, "nao differs from the XC grid's");
    const int64_t nao_tp = nao * (nao + 1) / 2;
    c->cderi_tp.ensure((size_t)nao_tp * naux * 8, c->counter());
    copy_in(c, c->cderi_tp.p, j3c, (size_t)nao_tp * naux * 8);
    check_finite(c, c->cderi_tp.as<double>(), nao_tp * naux, "j3c");
    J2cDecomp d;
    double t_dec = 0.0, t_solve = 0.0;
    {
      DecompWork w;
      DevBuf m;
      m.ensure((size_t)naux * naux * 8, c->counter());
      copy_in(c, m.p, j2c, (size_t)naux * naux * 8);
      check_finite(c, m.as<double>(), naux * naux, "j2c");
      const auto t0 = std::chrono::steady_clock::now();
      d = j2c_cholesky(c, m.as<double>(), naux, threshold, w);
      const auto t1 = std::chrono::steady_clock::now();
      solve_by_j2c_right(c, c->cderi_tp.as<double>(), nao_tp, naux, w);
      CPHF_CUDA(cudaStreamSynchronize(c->stream));
      const auto t2 = std::chrono::steady_clock::now();
      t_dec = std::chrono::duration<double>(t1 - t0).count();
      t_solve = std::chrono::duration<double>(t2 - t1).count();
    }
    install_cderi(c, nao, naux, scale_j, scale_k);
    fill_j2c_info(info, d, t_dec, t_solve);
  });
}

cphf_status cphf_rijk_get_cderi(cphf_ctx* c, double* cderi) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(c->has_rijk, "RI-JK plugin not set");
    copy_out(c, cderi, c->cderi_tp.p, (size_t)c->nao * (c->nao + 1) / 2 * c->naux * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_xc_set_grid(cphf_ctx* c, const double* ao, const double* weights, const double* fxc,
                             int64_t ngrids, int32_t nspin, const int64_t* batch_offsets,
                             int64_t nbatch) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(c->nao > 0, "set cderi or nao before the XC grid");
    CPHF_CHECK_ARG(ngrids >= 0, "ngrids must be non-negative");
    CPHF_CHECK_ARG(nspin == 1 || nspin == 2, "nspin must be 1 or 2");
    const int64_t nao = c->nao;
    std::vector<int64_t> off;
    if (batch_offsets && nbatch > 0) {
      off = read_small(c, batch_offsets, nbatch + 1);
      CPHF_CHECK_SHAPE(off.front() == 0 && off.back() == ngrids, "batch offsets must span [0, ngrids]");
      for (int64_t b = 0; b < nbatch; ++b) CPHF_CHECK_SHAPE(off[b] <= off[b + 1], "batch offsets must be non-decreasing");
    } else {
      off = {0, ngrids};
    }
    const int64_t nb = (int64_t)off.size() - 1;
    // stage the dense AO block, find each batch's non-zero AO window, pack the windows
    DevBuf dense;
    dense.ensure((size_t)std::max<int64_t>(ngrids * nao, 1) * 8, nullptr);
    copy_in(c, dense.p, ao, (size_t)ngrids * nao * 8);
    // window detection on the host copy of per-(batch, column) non-zero flags
    std::vector<int> flags((size_t)nb * nao, 0);
    {
      DevBuf fl;
      fl.ensure((size_t)std::max<int64_t>(nb * nao, 1) * sizeof(int), nullptr);
      CPHF_CUDA(cudaMemsetAsync(fl.p, 0, (size_t)nb * nao * sizeof(int), c->stream));
      DevBuf doff;
      doff.ensure(off.size() * 8, nullptr);
      CPHF_CUDA(cudaMemcpyAsync(doff.p, off.data(), off.size() * 8, cudaMemcpyHostToDevice, c->stream));
      launch_nonzero_flags(dense.as<double>(), ngrids, nao, doff.as<int64_t>(), nb, fl.as<int>(), c->stream);
      CPHF_CUDA(cudaMemcpyAsync(flags.data(), fl.p, flags.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      CPHF_CUDA(cudaStreamSynchronize(c->stream));
    }
    std::vector<XcBatch> batches(nb);
    int64_t total = 0;
    for (int64_t b = 0; b < nb; ++b) {
      XcBatch& x = batches[b];
      x.g0 = off[b];
      x.npts = off[b + 1] - off[b];
      int64_t lo = nao, hi = -1;
      for (int64_t m = 0; m < nao; ++m)
        if (flags[b * nao + m]) { lo = std::min(lo, m); hi = std::max(hi, m); }
      if (hi < lo) { x.lo = 0; x.nwin = 0; }
      else { x.lo = lo; x.nwin = hi - lo + 1; }
      x.phi_off = total;
      total += x.npts * x.nwin;
    }
    c->phi.ensure((size_t)std::max<int64_t>(total, 1) * 8, c->counter());
    for (const XcBatch& x : batches) {
      if (x.npts == 0 || x.nwin == 0) continue;
      CPHF_CUDA(cudaMemcpy2DAsync(c->phi.as<double>() + x.phi_off, x.npts * 8,
                                  dense.as<double>() + x.g0 + ngrids * x.lo, ngrids * 8, x.npts * 8,
                                  x.nwin, cudaMemcpyDeviceToDevice, c->stream));
    }
    c->weights.ensure((size_t)std::max<int64_t>(ngrids, 1) * 8, c->counter());
    copy_in(c, c->weights.p, weights, (size_t)ngrids * 8);
    const int64_t nf = nspin == 1 ? ngrids : 4 * ngrids;
    c->fxc.ensure((size_t)std::max<int64_t>(nf, 1) * 8, c->counter());
    copy_in(c, c->fxc.p, fxc, (size_t)nf * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    c->xc_batches = batches;
    c->xc_plans.clear();  // chunk plans depend on the batches
    c->ngrids = ngrids;
    c->xc_nspin = nspin;
    c->xc_den = 0;
    c->xc_nvar = 1;
    c->phiG.release();
    c->fxcG.release();
    c->has_xc = true;
    c->prepared = false;
    lowp_release(c);
  });
}

cphf_status cphf_xc_set_grid_ex(cphf_ctx* c, int32_t den_type, const double* ao, int32_t ncomp, const double* weights,
                                const double* fxc_eff, int64_t ngrids, int32_t nspin, const int64_t* batch_offsets,
                                int64_t nbatch) {
  if (den_type == 0) {  // RHO: component 0 of ao, fxc_eff [ngrids, 1, 1] / [ngrids, 1, 2, 1, 2]
    if (!c) return CPHF_ERR_ARG;
    if (ncomp < 1) {
      c->last_error = "ncomp must be at least 1";
      return CPHF_ERR_ARG;
    }
    return cphf_xc_set_grid(c, ao, weights, fxc_eff, ngrids, nspin, batch_offsets, nbatch);
  }
  return guarded(c, [&] {
    CPHF_CHECK_ARG(c->nao > 0, "set cderi or nao before the XC grid");
    CPHF_CHECK_ARG(den_type == 1 || den_type == 2, "den_type must be 0 (RHO), 1 (SIGMA) or 2 (TAU)");
    CPHF_CHECK_ARG(ncomp >= 4, "SIGMA / TAU need the AO values and their three first derivatives (ncomp >= 4)");
    CPHF_CHECK_ARG(ngrids >= 0, "ngrids must be non-negative");
    CPHF_CHECK_ARG(nspin == 1 || nspin == 2, "nspin must be 1 or 2");
    const int64_t nao = c->nao, nvar = den_type == 1 ? 4 : 5;
    c->phiG.ensure((size_t)std::max<int64_t>(ngrids * nao * 4, 1) * 8, c->counter());
    copy_in(c, c->phiG.p, ao, (size_t)ngrids * nao * 4 * 8);  // components 0-3 of [ngrids, nao, ncomp]
    c->weights.ensure((size_t)std::max<int64_t>(ngrids, 1) * 8, c->counter());
    copy_in(c, c->weights.p, weights, (size_t)ngrids * 8);
    const int64_t nf = ngrids * nvar * nvar * (nspin == 1 ? 1 : 4);
    c->fxcG.ensure((size_t)std::max<int64_t>(nf, 1) * 8, c->counter());
    copy_in(c, c->fxcG.p, fxc_eff, (size_t)nf * 8);
    check_finite(c, c->phiG.as<double>(), ngrids * nao * 4, "ao");
    check_finite(c, c->fxcG.as<double>(), nf, "fxc_eff");
    (void)batch_offsets;
    (void)nbatch;  // the dense path chunks the points itself
    c->phi.release();
    c->xc_batches.clear();
    c->xc_plans.clear();
    c->ngrids = ngrids;
    c->xc_nspin = nspin;
    c->xc_den = den_type;
    c->xc_nvar = (int)nvar;
    c->has_xc = true;
    c->prepared = false;
    lowp_release(c);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_prepare(cphf_ctx* c, int32_t nspin, const double* const* mo_coeff,
                         const double* const* mo_occ, const double* const* mo_energy, int64_t nmo) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(nspin == 1 || nspin == 2, "nspin must be 1 or 2");
    CPHF_CHECK_ARG(c->nao > 0, "set cderi or nao before the preparation");
    CPHF_CHECK_ARG(mo_coeff && mo_occ && mo_energy, "null orbital arrays");
    CPHF_CHECK_SHAPE(nmo > 0 && nmo <= c->nao, "nmo must be in [1, nao]");
    CPHF_CHECK_SHAPE(!c->has_xc || c->xc_nspin == nspin, "XC grid spin count differs");
    const int64_t nao = c->nao;
    for (int s = 0; s < nspin; ++s) {
      std::vector<double> occ = read_small(c, mo_occ[s], nmo);
      int64_t nocc = 0;
      for (int64_t p = 0; p < nmo; ++p) nocc += occ[p] > 0.0 ? 1 : 0;
      for (int64_t p = 0; p < nmo; ++p)
        CPHF_CHECK_SHAPE((occ[p] > 0.0) == (p < nocc), "orbitals must be ordered occupied first");
      SpinState& sp = c->spin[s];
      sp.nmo = nmo;
      sp.nocc = nocc;
      sp.iaia.release();  // learned-guess features of the previous orbitals
      sp.C.ensure((size_t)nao * nmo * 8, c->counter());
      copy_in(c, sp.C.p, mo_coeff[s], (size_t)nao * nmo * 8);
      sp.e.ensure((size_t)nmo * 8, c->counter());
      copy_in(c, sp.e.p, mo_energy[s], (size_t)nmo * 8);
      check_finite(c, sp.C.as<double>(), nao * nmo, "mo_coeff");
      check_finite(c, sp.e.as<double>(), nmo, "mo_energy");
    }
    c->nspin = nspin;
    if (c->has_rijk) rijk_prepare(c);
    if (c->has_xc) xc_prepare(c);
    lowp_release(c);
    if (c->cfg.precision == CPHF_PRECISION_MIXED) lowp_prepare(c);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    c->prepared = true;
  });
}

static cphf_status response_common(cphf_ctx* c, int which, const double* const* bra, int64_t nprop,
                                   double* const* out) {
  return guarded(c, [&] {
    require_prepared(c);
    CPHF_CHECK_ARG(bra && out, "null bra/out arrays");
    CPHF_CHECK_SHAPE(nprop >= 0, "nprop must be non-negative");
    if (which == 0) CPHF_CHECK_ARG(c->has_rijk, "RI-JK plugin not set");
    if (which == 1) CPHF_CHECK_ARG(c->has_xc, "XC plugin not set");
    std::vector<int64_t> el;
    for (int s = 0; s < c->nspin; ++s) el.push_back(bra_elems(c, s, nprop));
    double* din[2];
    double* dout[2];
    stage_in(c, c->s_host_io, bra, el, din);
    stage_in(c, c->s_misc, nullptr, el, dout);
    if (nprop > 0) {
      bool acc = false;
      if (c->has_rijk && (which < 0 || which == 0)) { rijk_response_fp64(c, din, nprop, dout, acc); acc = true; }
      if (c->has_xc && (which < 0 || which == 1)) { xc_response_fp64(c, din, nprop, dout, acc); acc = true; }
    }
    for (int s = 0; s < c->nspin; ++s) copy_out(c, out[s], dout[s], el[s] * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_response_bra(cphf_ctx* c, const double* const* bra, int64_t nprop, double* const* out) {
  return response_common(c, -1, bra, nprop, out);
}

cphf_status cphf_plugin_response_bra(cphf_ctx* c, int32_t which, const double* const* bra, int64_t nprop,
                                     double* const* out) {
  if (which != 0 && which != 1) return CPHF_ERR_ARG;
  return response_common(c, which, bra, nprop, out);
}

static cphf_status response_mo_common(cphf_ctx* c, const double* const* mo1, int64_t nprop,
                                      double* const* resp, bool dimless, bool lowp = false) {
  return guarded(c, [&] {
    require_prepared(c);
    CPHF_CHECK_ARG(mo1 && resp, "null arrays");
    if (lowp) CPHF_CHECK_ARG(c->cfg.precision == CPHF_PRECISION_MIXED, "the context is not in mixed precision");
    const int64_t n = krylov_n(c);
    c->s_host_io.ensure((size_t)std::max<int64_t>(n * nprop, 1) * 8 * 2, c->counter());
    double* x = c->s_host_io.as<double>();
    double* y = x + n * nprop;
    pack_krylov(c, mo1, nprop, x);
    if (nprop > 0 && lowp) response_mo_lowp(c, x, nprop, y);
    else if (nprop > 0) response_mo_fp64(c, x, nprop, y, dimless);
    unpack_krylov(c, y, nprop, resp);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_response_mo(cphf_ctx* c, const double* const* mo1, int64_t nprop, double* const* resp) {
  return response_mo_common(c, mo1, nprop, resp, false);
}

cphf_status cphf_response_dimless(cphf_ctx* c, const double* const* mo1, int64_t nprop, double* const* resp) {
  return response_mo_common(c, mo1, nprop, resp, true);
}

cphf_status cphf_response_dimless_lowp(cphf_ctx* c, const double* const* mo1, int64_t nprop, double* const* resp) {
  return response_mo_common(c, mo1, nprop, resp, true, true);
}

cphf_status cphf_solve_dimless_cphf(cphf_ctx* c, const double* const* rhs, int64_t nprop,
                                    const double* const* x0, double* const* mo1, cphf_stats* stats) {
  bool converged = true;
  cphf_stats st{};
  const auto t0 = std::chrono::steady_clock::now();
  cphf_status rc = guarded(c, [&] {
    require_prepared(c);
    CPHF_CHECK_ARG(rhs && mo1, "null arrays");
    CPHF_CHECK_SHAPE(nprop > 0, "nprop must be positive");
    const int64_t n = krylov_n(c);
    c->s_host_io.ensure((size_t)n * nprop * 8 * 3, c->counter());
    double* b = c->s_host_io.as<double>();
    double* xg = b + n * nprop;
    double* x = xg + n * nprop;
    pack_krylov(c, rhs, nprop, b);
    check_finite(c, b, n * nprop, "rhs");
    if (x0) pack_krylov(c, x0, nprop, xg);
    const double* x0p = x0 ? xg : nullptr;
    // Learned initial guess / left preconditioner, in context-owned buffers (no allocation per
    // solve).  Mixed precision: the preconditioner m acts on the first inner solve only, whose
    // convergence the outer FP64-accurate residual decides; mode 2 also starts the first inner
    // solve from the guess (one more operator application for its residual).  FP64: the guess
    // is only the initial x0, so the Krylov iteration and its stopping test are the
    // reference's unmodified ones (krylov_block.rs:86-87, 130-157).
    double* m = nullptr;
    const bool mixed = c->cfg.precision == CPHF_PRECISION_MIXED;
    if (c->cfg.use_learned_guess) {
      mlp_require(c);
      if (c->spin[0].iaia.p == nullptr) mlp_prepare_iaia(c);
      c->k_pre.ensure((size_t)n * 8 * (1 + nprop), c->counter());
      double* mbuf = c->k_pre.as<double>();
      double* guess = mbuf + n;
      const bool want_guess = !mixed || c->cfg.use_learned_guess == 2;
      mlp_guess(c, b, nprop, guess, mixed ? mbuf : nullptr);
      if (mixed) m = mbuf;
      if (!x0p && want_guess) x0p = guess;
    }
    if (mixed) {
      converged = solve_mixed(c, b, x0p, nprop, x, &st, m);
    } else {
      KrylovParams p{c->cfg.cphf_tol, c->cfg.cphf_lindep, c->cfg.cphf_max_cycle, c->cfg.cphf_max_space,
                     c->cfg.verbose != 0};
      DeviceOp op = [&](const double* xin, int64_t nb, double* yout) {
        response_mo_fp64(c, xin, nb, yout, true);
        st.fp64_matvec_columns += nb;
      };
      converged = krylov_device(c, op, b, x0p, n, nprop, p, x, &st);
      st.residual_max = -1.0;  // not evaluated by the plain solver (the reference does not either)
      st.residual_mode = -1;
    }
    unpack_krylov(c, x, nprop, mo1);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
  st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  if (rc == CPHF_OK && !converged) {
    c->last_error = "krylov_block failed to converge";
    return CPHF_ERR_NOT_CONVERGED;
  }
  return rc;
}

cphf_status cphf_compute_dimless_cphf_rhs(cphf_ctx* c, const double* f1ao_core, const double* const* f1bra_el,
                                          const double* s1ao, int64_t natm, double* const* rhs, double* const* f1mo,
                                          double* const* s1mo) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(c->nspin == 1 || c->nspin == 2, "cphf_prepare has not been called");
    CPHF_CHECK_ARG(s1ao && rhs && f1mo && s1mo, "null arrays");
    CPHF_CHECK_SHAPE(natm > 0, "natm must be positive");
    const int64_t nao = c->nao, nprop = 3 * natm, nsq = nao * nao * nprop;
    // shared AO derivatives (core Fock and overlap are spin independent, uscf.rs:104-148)
    DevBuf ao;
    ao.ensure((size_t)2 * nsq * 8, c->counter());
    double* F = ao.as<double>();
    double* S1 = F + nsq;
    if (f1ao_core) copy_in(c, F, f1ao_core, (size_t)nsq * 8);
    copy_in(c, S1, s1ao, (size_t)nsq * 8);
    for (int s = 0; s < c->nspin; ++s) {
      const SpinState& sp = c->spin[s];
      const int64_t no = sp.nocc, nmo = sp.nmo, nb = nao * no * nprop, nm = nmo * no * nprop;
      DevBuf tmp;
      tmp.ensure((size_t)std::max<int64_t>(2 * nb + 3 * nm, 1) * 8, c->counter());
      double* fbra = tmp.as<double>();
      double* sbra = fbra + nb;
      double* f1 = sbra + nb;
      double* s1 = f1 + nm;
      double* r = s1 + nm;
      if (f1bra_el && f1bra_el[s]) copy_in(c, fbra, f1bra_el[s], (size_t)nb * 8);
      else CPHF_CUDA(cudaMemsetAsync(fbra, 0, (size_t)nb * 8, c->stream));
      if (no > 0) {
        GemmDesc g;  // f1bra = f1bra_el + f1ao_core Cocc   (rscf.rs:158), batched over the 3 natm derivatives
        g.M = nao; g.N = no; g.K = nao; g.batch1 = nprop;
        g.A = F; g.a_m = 1; g.a_k = nao; g.a_b1 = nao * nao;
        g.B = sp.C.p; g.b_k = 1; g.b_n = nao; g.b_b1 = 0;
        g.C = fbra; g.c_m = 1; g.c_n = nao; g.c_b1 = nao * no;
        g.beta = 1.0;
        if (f1ao_core) gemm64(c, g);
        g.A = S1; g.C = sbra; g.beta = 0.0;  // s1ao Cocc   (rscf.rs:169)
        gemm64(c, g);
        GemmDesc m;  // f1mo = C^T f1bra, s1mo = C^T (s1ao Cocc)   (rscf.rs:159, 169)
        m.M = nmo; m.N = no * nprop; m.K = nao;
        m.A = sp.C.p; m.a_m = nao; m.a_k = 1;
        m.B = fbra; m.b_k = 1; m.b_n = nao;
        m.C = f1; m.c_m = 1; m.c_n = nmo;
        gemm64(c, m);
        m.B = sbra; m.C = s1;
        gemm64(c, m);
        launch_cphf_rhs(f1, s1, sp.e.as<double>(), nmo, no, nprop, c->cfg.level_shift, r, c->stream);
      }
      copy_out(c, rhs[s], r, (size_t)nm * 8);
      copy_out(c, f1mo[s], f1, (size_t)nm * 8);
      copy_out(c, s1mo[s], s1, (size_t)nm * 8);
      CPHF_CUDA(cudaStreamSynchronize(c->stream));
    }
  });
}

cphf_status cphf_finalize_cphf(cphf_ctx* c, const double* const* f1mo, const double* const* s1mo,
                               int64_t natm, double* const* mo1, double* const* mo_e1) {
  return guarded(c, [&] {
    require_prepared(c);
    CPHF_CHECK_ARG(f1mo && s1mo && mo1 && mo_e1, "null arrays");
    CPHF_CHECK_SHAPE(natm > 0, "natm must be positive");
    const int64_t nprop = 3 * natm, n = krylov_n(c);
    // device layout: [mo1 | resp | f1 | s1] in Krylov packing, then per-spin mo_e1
    int64_t ne1 = 0;
    for (int s = 0; s < c->nspin; ++s) ne1 += c->spin[s].nocc * c->spin[s].nocc * nprop;
    c->s_host_io.ensure((size_t)(4 * n * nprop + ne1) * 8, c->counter());
    double* x = c->s_host_io.as<double>();
    double* resp = x + n * nprop;
    double* f1 = resp + n * nprop;
    double* s1 = f1 + n * nprop;
    double* e1 = s1 + n * nprop;
    pack_krylov(c, mo1, nprop, x);
    pack_krylov(c, f1mo, nprop, f1);
    pack_krylov(c, s1mo, nprop, s1);
    {
      // rscf.rs:342.  A mixed-precision context evaluates this response with its FP64-accurate
      // operator (residual_dfloat: exact-slice tensor cores + double-float by default), a
      // plain FP64 context with native FP64.
      const bool mixed = c->cfg.precision == CPHF_PRECISION_MIXED && c->lowp;
      AccurateScope scope(c, mixed ? c->cfg.residual_dfloat : 0);
      response_mo_fp64(c, x, nprop, resp, false);
    }
    int64_t off = 0, offe = 0;
    for (int s = 0; s < c->nspin; ++s) {
      const SpinState& sp = c->spin[s];
      const int64_t len = sp.nmo * sp.nocc;
      // per-spin contiguous views: copy out of the packed layout when nspin == 2
      if (c->nspin == 1) {
        launch_finalize(f1, s1, resp, sp.e.as<double>(), sp.nmo, sp.nocc, nprop, x, e1, c->stream);
      } else {
        DevBuf tmp;
        tmp.ensure((size_t)std::max<int64_t>(len * nprop, 1) * 8 * 4, c->counter());
        double* t0 = tmp.as<double>();
        double* arr[4] = {t0, t0 + len * nprop, t0 + 2 * len * nprop, t0 + 3 * len * nprop};
        const double* srcs[4] = {x, resp, f1, s1};
        for (int k = 0; k < 4; ++k)
          if (len > 0)
            CPHF_CUDA(cudaMemcpy2DAsync(arr[k], len * 8, srcs[k] + off, n * 8, len * 8, nprop, cudaMemcpyDeviceToDevice, c->stream));
        launch_finalize(arr[2], arr[3], arr[1], sp.e.as<double>(), sp.nmo, sp.nocc, nprop, arr[0], e1 + offe, c->stream);
        if (len > 0)
          CPHF_CUDA(cudaMemcpy2DAsync(x + off, n * 8, arr[0], len * 8, len * 8, nprop, cudaMemcpyDeviceToDevice, c->stream));
        CPHF_CUDA(cudaStreamSynchronize(c->stream));
      }
      copy_out(c, mo_e1[s], e1 + offe, (size_t)sp.nocc * sp.nocc * nprop * 8);
      off += len;
      offe += sp.nocc * sp.nocc * nprop;
    }
    unpack_krylov(c, x, nprop, mo1);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_get_cphf_hess(cphf_ctx* c, const double* const* f1mo, const double* const* s1mo,
                               const double* const* mo1, const double* const* mo_e1, int64_t natm,
                               double* de) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(c->nspin == 1 || c->nspin == 2, "cphf_prepare has not been called");
    CPHF_CHECK_ARG(f1mo && s1mo && mo1 && mo_e1 && de, "null arrays");
    CPHF_CHECK_SHAPE(natm > 0, "natm must be positive");
    const int64_t nprop = 3 * natm;
    DevBuf G;
    G.ensure((size_t)nprop * nprop * 8 + (size_t)9 * natm * natm * 8, c->counter());
    double* Gd = G.as<double>();
    double* ded = Gd + nprop * nprop;
    CPHF_CUDA(cudaMemsetAsync(Gd, 0, (size_t)nprop * nprop * 8, c->stream));
    const double f0 = c->nspin == 1 ? 4.0 : 2.0, fs = f0, fe = c->nspin == 1 ? 2.0 : 1.0;
    for (int s = 0; s < c->nspin; ++s) {
      const SpinState& sp = c->spin[s];
      const int64_t len = sp.nmo * sp.nocc * nprop, le = sp.nocc * sp.nocc * nprop;
      DevBuf tmp;
      tmp.ensure((size_t)std::max<int64_t>(3 * len + le, 1) * 8, c->counter());
      double* f1 = tmp.as<double>();
      double* s1 = f1 + len;
      double* m1 = s1 + len;
      double* e1 = m1 + len;
      copy_in(c, f1, f1mo[s], len * 8);
      copy_in(c, s1, s1mo[s], len * 8);
      copy_in(c, m1, mo1[s], len * 8);
      copy_in(c, e1, mo_e1[s], le * 8);
      launch_hess_pairs(f1, s1, m1, e1, sp.e.as<double>(), sp.nmo, sp.nocc, nprop, f0, fs, fe, Gd, c->stream);
      CPHF_CUDA(cudaStreamSynchronize(c->stream));
    }
    launch_hess_assemble(Gd, natm, ded, c->stream);
    copy_out(c, de, ded, (size_t)9 * natm * natm * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_krylov_block(cphf_ctx* c, cphf_aop_fn aop, void* user, const double* b, const double* x0,
                              int64_t n, int64_t nset, double tol, int64_t max_cycle, int64_t max_space,
                              double lindep, double* x, cphf_stats* stats) {
  bool converged = true;
  cphf_stats st{};
  const auto t0 = std::chrono::steady_clock::now();
  cphf_status rc = guarded(c, [&] {
    CPHF_CHECK_ARG(aop != nullptr, "null operator");
    CPHF_CHECK_SHAPE(n > 0 && nset > 0, "n and nset must be positive");
    CPHF_CHECK_ARG(max_space > 0 && max_cycle >= 0, "max_space must be positive");
    c->s_misc.ensure((size_t)n * nset * 8 * 3, c->counter());
    double* db = c->s_misc.as<double>();
    double* dx0 = db + n * nset;
    double* dx = dx0 + n * nset;
    copy_in(c, db, b, (size_t)n * nset * 8);
    if (x0) copy_in(c, dx0, x0, (size_t)n * nset * 8);
    KrylovParams p{tol, lindep, max_cycle, max_space, c->cfg.verbose != 0};
    DeviceOp op = [&](const double* xin, int64_t nb, double* yout) {
      const int r = aop(user, xin, n, nb, yout, (void*)c->stream);
      if (r != 0) throw Error(CPHF_ERR_ARG, "operator callback returned " + std::to_string(r));
    };
    converged = krylov_device(c, op, db, x0 ? dx0 : nullptr, n, nset, p, dx, &st);
    copy_out(c, x, dx, (size_t)n * nset * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
  st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  if (rc == CPHF_OK && !converged) {
    c->last_error = "krylov_block failed to converge";
    return CPHF_ERR_NOT_CONVERGED;
  }
  return rc;
}

struct cphf_dense_op {
  cphf_ctx* ctx;
  DevBuf A;
  int64_t n;
};

cphf_status cphf_dense_op_create(cphf_ctx* c, const double* A, int64_t n, cphf_dense_op** out) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(out != nullptr && n > 0, "invalid dense operator arguments");
    auto* op = new cphf_dense_op();
    op->ctx = c;
    op->n = n;
    op->A.ensure((size_t)n * n * 8, nullptr);
    copy_in(c, op->A.p, A, (size_t)n * n * 8);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
    *out = op;
  });
}

int cphf_dense_op_apply(void* user, const double* x, int64_t n, int64_t nblock, double* y, void*) {
  auto* op = static_cast<cphf_dense_op*>(user);
  if (!op || n != op->n) return 1;
  try {
    GemmDesc d;
    d.M = n; d.N = nblock; d.K = n;
    d.A = op->A.p; d.a_m = 1; d.a_k = n;
    d.B = x; d.b_k = 1; d.b_n = n;
    d.C = y; d.c_m = 1; d.c_n = n;
    gemm64(op->ctx, d);
  } catch (const std::exception&) {
    return 2;
  }
  return 0;
}

cphf_status cphf_dense_op_destroy(cphf_dense_op* op) {
  delete op;
  return CPHF_OK;
}

cphf_status cphf_copy(cphf_ctx* c, void* dst, const void* src, int64_t bytes) {
  return guarded(c, [&] {
    CPHF_CHECK_ARG(bytes >= 0, "negative size");
    copy_out(c, dst, src, (size_t)bytes);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

}  // extern "C"
