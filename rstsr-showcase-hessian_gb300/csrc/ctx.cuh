// Context of libcphf: device-resident plugin state, scratch and the operator entry points.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "gemm_simt.cuh"

struct cphf_ctx;

namespace cphf {

// Per-spin slice copies of the FP64-accurate tensor-core K term (tc_ozaki.cu); every slice
// array holds 6 BF16 planes, rows scaled by a power of two (exponents alongside).
struct OzSpin {
  DevBuf O, eO;        // [6][naux][nocc(i)][ldj] of O_P[j, i], K = j; exponent per (P, i)
  DevBuf Z, eZ;        // [6][naux][nocc(i)][ldk] of Z_P[nu, i], K = nu; exponent per (P, i)
  DevBuf Zt, sZt, eZt; // [6][naux][nao(mu)][ldj] of Z_P[mu, j], K = j; scale per mu over (j, P)
  DevBuf Omax, Zmax;   // split FP16: max |O_P|, max |Z_P| per aux function (float bits), for the T / W bounds
  int64_t ldj = 0;     // padded K = nocc rows
  bool ready = false;
};
struct OzState {
  DevBuf A;                    // [6][naux][nao][ldk] slices of the row-scaled cderi
  DevBuf rowscale, e_row, mx;  // per-row power-of-two scales of A
  OzSpin spin[2];
  // per-call scratch: bra slices (both K orders), T / Wt staging (FP32 pairs) and slices
  DevBuf braw, ebraw, brat, ebrat, T, B, W, Ws, braS, braWS, wsc;
  DevBuf colscale, e_col, mxc, err, tune_out;
  int64_t ldk = 0;
  bool ready = false;
};

// Dense split-FP16 forms of phi for the tensor-core XC response (xc_tc.cu).
// One grid batch of the tensor-core XC response: its points [g0, g0 + npts) and AO window
// [lo, lo + nwin), the window start rounded down to 8 AOs (lo8, so that the TMA K offset of bra
// is 16-byte aligned) and its length from there (kw), its first row of the phi^T planes (rT)
// and its first column in the 8-padded point layout of the q planes (gofs).
struct XcTcBatch {
  int64_t g0, npts, lo, nwin, phi_off, lo8, kw, rT, gofs;
};

// Block-sparse operand planes of phi for the tensor-core XC response (xc_tc.cu).
struct XcTcState {
  std::vector<XcTcBatch> hb;  // host copy of the batch records (one more entry: gofs of the end)
  int64_t ldw = 0, ldpT = 0, nrowT = 0;
  DevBuf batches, pt_batch, rowmap, colmap;  // records, point -> batch, phi^T row -> batch, q column -> point
  DevBuf phiB, phiB_scale;    // [t][p][ldw]: phi[p, lo8 + k] over the window of p's batch, scale per point
  DevBuf phiT, phiT_scale;    // [t][rT + m][ldpT]: phi[g0 + k, lo + m] per batch, scale per row
  DevBuf bpl[2], eb[2], bscale[2];  // planes of bra rows (i, a) per spin, their exponents and scales
  DevBuf v, qpl, qscale;      // w f rho1 of a chunk and spin, planes of q rows (i, a), their scales
  DevBuf qmax;                // column maxima of v and aobra (the split-FP16 q scales)
  bool ready = false;
};

// One captured application of the split-precision operator for block width nb, reading and
// writing the staging buffers of LowpState (g_x, g_y).
struct OpGraph {
  int64_t nb = 0, gen = -1, nodes = 0;
  cudaGraphExec_t exec = nullptr;
};

// State of the split-precision operator (mixed.cu).
struct LowpState {
  DevBuf Bd32;                 // [nao, nao, naux] FP32 (SIMT fallback of the K term)
  DevBuf Bhi, Blo;             // FP16 hi / lo split of the dense cderi for the tensor-core K term
  int64_t ldk = 0;             // padded row length of the FP16 copies
  OzState oz;                  // FP64-accurate tensor-core K term of the residual
  OzState lp;                  // split-FP16 planes of O, Z and bra for the K term's other contractions
  XcTcState xctc;              // dense split-FP16 phi for the tensor-core XC response
  XcTcState xctc64;            // dense exact-slice phi for the FP64-accurate XC residual
  DevBuf phi32;
  DevBuf phiG32, s_gket, s_grho;  // GGA / meta-GGA XC in FP32
  DevBuf s_c1, s_resp, s_T, s_W, s_d, s_ket, s_rho, s_y, s_x, s_Thi, s_Tlo, s_acc;
  DevBuf err;                  // device error flag of the tensor-core kernels (bounded waits)
  double sA = 1.0;             // power-of-two scale of the FP16 cderi planes
  int64_t budget = int64_t(1) << 30;  // bytes per chunk of T / W intermediates (set at preparation)
  bool use_tc = true;
  // captured operator applications (cfg.cuda_graphs)
  std::vector<OpGraph> graphs;
  DevBuf g_x, g_y;
  bool graphs_off = false;     // capture failed once: run the operator eagerly from then on
  void drop_graphs() {
    for (auto& g : graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    graphs.clear();
  }
  ~LowpState() { drop_graphs(); }
};

// Learned initial guess / preconditioner (mlp.cu): weights, Adam moments, scratch.
struct MlpState {
  DevBuf w, m, v, g, part, idx, feat, out;
  int64_t step = 0;
};

struct SpinState {
  int64_t nmo = 0, nocc = 0;
  DevBuf C;       // [nao, nmo] FP64 (occupied columns first)
  DevBuf e;       // [nmo] FP64
  DevBuf Z;       // [nao, nocc, naux] FP64: Z_P = B_P Cocc
  DevBuf O;       // [nocc, nocc, naux] FP64: O_P = Cocc^T B_P Cocc
  DevBuf aobra;   // [ngrids, nocc] FP64: phi Cocc (XC)
  // split-precision copies (mixed path)
  DevBuf C32, Z32, O32, aobra32;
  DevBuf iaia;    // [nvir, nocc] FP32: RI diagonal (ia|ia), feature of the learned guess
  DevBuf aobG, aobG32;  // [ngrids, nocc, 4] phi_c Cocc (GGA / meta-GGA XC), FP64 / FP32
};

struct XcBatch {
  int64_t g0 = 0, npts = 0;   // grid rows [g0, g0 + npts)
  int64_t lo = 0, nwin = 0;   // AO window [lo, lo + nwin)
  int64_t phi_off = 0;        // element offset of the batch block in phi
};

// Chunking of the grid batches for one output width (xc_grouped.cu), cached per key.
struct XcChunk {
  int64_t b0, b1;         // batches [b0, b1)
  int64_t g0, npts;       // grid points [g0, g0 + npts)
  int64_t group_off;      // offset of the chunk's group records (per spin) in the device table
  int64_t tiles[2];       // work items of the first GEMM, per spin
};
struct XcPlan {
  int64_t key[4] = {-1, -1, -1, -1};  // element size, nb, nocc_a, nocc_b
  std::vector<XcChunk> chunks;
  DevBuf groups;                       // XcGroupDev records
  int64_t max_pts = 0;
};

// Operator over Krylov columns: y[:, 0:nb] = A x[:, 0:nb] with device pointers, ld = n.
using DeviceOp = std::function<void(const double* x, int64_t nb, double* y)>;

// Per-kernel-class timing with CUDA events on the context stream (the reference keeps
// wall-clock (label, seconds) pairs, src/hessian/rscf.rs:33, src/ri_jk/hess_r.rs:192-198).
struct ProfRecord {
  int cls;
  double flops, bytes;
  cudaEvent_t start, stop;
};
struct Profiler {
  bool on = false;
  std::vector<ProfRecord> recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  ~Profiler() {
    for (auto& r : recs) {
      cudaEventDestroy(r.start);
      cudaEventDestroy(r.stop);
    }
    for (auto e : pool) cudaEventDestroy(e);
  }
};
enum ProfClass {
  PROF_GEMM_F64 = 0,
  PROF_GEMM_F32 = 1,
  PROF_TC_KTERM = 2,
  PROF_GEMM_F64E = 3,
  PROF_TC_OZAKI = 4,
  PROF_TC_SPLIT = 5,
  PROF_SLICE = 6,
  PROF_KRYLOV = 7,
  PROF_XC64 = 8,
  PROF_XC32 = 9,
  PROF_TC_WGEN = 10,
  PROF_TC_TERM2 = 11,
  PROF_XC_TC32 = 12,
  PROF_XC_TC64 = 13,
  PROF_OZ_TGEN = 14,
  PROF_OZ_WGEN = 15,
  PROF_OZ_TERM2 = 16,
  PROF_OZC_KTERM = 17,
  PROF_OZC_TGEN = 18,
  PROF_OZC_WGEN = 19,
  PROF_OZC_TERM2 = 20,
  PROF_SLICE_EXACT = 21,
  PROF_OZC3_KTERM = 22,
  PROF_OZC3_TGEN = 23,
  PROF_OZC3_WGEN = 24,
  PROF_OZC3_TERM2 = 25,
  PROF_XC_TC64C = 26,
  PROF_NCLASS = 27
};
extern const char* const kProfNames[PROF_NCLASS];

}  // namespace cphf

struct cphf_ctx {
  cphf_config cfg{};
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t device_bytes = 0;
  int64_t launches = 0;

  // RI-JK plugin
  bool has_rijk = false;
  int64_t nao = 0, naux = 0;
  double scale_j = 0.0, scale_k = 0.0;
  cphf::DevBuf cderi_tp;  // [nao_tp, naux]
  cphf::DevBuf Bd;        // [nao, nao, naux] dense FP64

  // XC plugin
  bool has_xc = false;
  int xc_nspin = 1;
  int64_t ngrids = 0;
  std::vector<cphf::XcBatch> xc_batches;
  cphf::DevBuf phi, weights, fxc;  // phi: batch blocks [npts_b, nwin_b] (grid fastest)
  cphf::DevBuf phi32;
  std::vector<std::unique_ptr<cphf::XcPlan>> xc_plans;  // chunk plans, one per (precision, nb, nocc)
  int xc_den = 0;     // density type: 0 RHO (LDA), 1 SIGMA (GGA), 2 TAU (meta-GGA)
  int xc_nvar = 1;    // XCDenType::num_nvar (src/xceff/flags.rs:33-40)
  cphf::DevBuf phiG;  // GGA / meta-GGA: AO values and gradients [ngrids, nao, 4] FP64
  cphf::DevBuf fxcG;  // GGA / meta-GGA: fxc_eff [ngrids, nvar, nvar] or [ngrids, nvar, 2, nvar, 2]
  cphf::DevBuf s_gket, s_grho;  // GGA / meta-GGA chunk scratch (FP64)

  // prepared orbitals
  bool prepared = false;
  int nspin = 0;
  cphf::SpinState spin[2];

  // scratch (grown on demand)
  cphf::DevBuf ws_gemm, s_c1, s_resp, s_T, s_W, s_d, s_ket, s_rho, s_y, s_x, s_misc, s_host_io;
  cphf::DevBuf k_xs, k_ax, k_h, k_g, k_b, k_xacc, k_x1, k_axt, k_coef, k_ip, k_keep, k_part, k_idx,
      k_hw, k_info, k_r, k_norm, k_finite, k_pre;

  std::unique_ptr<cphf::LowpState> lowp;
  std::unique_ptr<cphf::MlpState> mlp;
  cphf::Profiler prof;
  bool f64_emulate = false;  // route the FP64 GEMMs through the double-float kernel
  bool oz_kterm = false;     // FP64 K term 1 on the tensor cores (exact BF16 slices)
  int oz_correction = 0;       // ... in correction precision: 0 off, else the slices read (3 or 4)
  bool f32_correction = false; // FP64 GEMMs of a correction-precision application run in FP32
  bool oz_xc = false;        // FP64 XC response on the tensor cores (exact BF16 slices)

  int64_t* counter() { return &device_bytes; }
};

namespace cphf {
// Scope that brackets one launch (or a group) with events when profiling is on.
struct ProfScope {
  cphf_ctx* c;
  ProfRecord r{};
  ProfScope(cphf_ctx* ctx, int cls, double flops, double bytes) : c(ctx) {
    if (!c->prof.on) return;
    r.cls = cls;
    r.flops = flops;
    r.bytes = bytes;
    r.start = c->prof.get();
    r.stop = c->prof.get();
    cudaEventRecord(r.start, c->stream);
  }
  ~ProfScope() {
    if (!c->prof.on) return;
    cudaEventRecord(r.stop, c->stream);
    c->prof.recs.push_back(r);
  }
};
}  // namespace cphf

namespace cphf {

// gemm helpers bound to the context (stream, split-K workspace, SM count)
void gemm64(cphf_ctx* c, const GemmDesc& d);
void gemm32(cphf_ctx* c, const GemmDesc& d);  // float compute, float operands/output
template <typename TA, typename TB, typename TC>
void gemm32x(cphf_ctx* c, const GemmDesc& d);

// plugins (device pointers): bra[s], out[s] [nao, nocc_s, nb] contiguous
void rijk_response_fp64(cphf_ctx* c, const double* const* bra, int64_t nb, double* const* out,
                        bool accumulate);
void xc_response_fp64(cphf_ctx* c, const double* const* bra, int64_t nb, double* const* out,
                      bool accumulate);
void rijk_prepare(cphf_ctx* c);
void xc_prepare(cphf_ctx* c);

// response_mo / dimensionless operator over the packed Krylov layout
// x, y: [n, nb] with n = sum_s nmo*nocc_s.
void response_mo_fp64(cphf_ctx* c, const double* x, int64_t nb, double* resp_mo, bool dimless);
// check = false: leave out the device error-flag read (a host synchronisation), for capture
void response_mo_lowp(cphf_ctx* c, const double* x, int64_t nb, double* resp_mo, bool check = true);
void lowp_check(cphf_ctx* c);
// response_mo_lowp as the inner solves apply it, replayed from captured CUDA graphs
void lowp_apply(cphf_ctx* c, const double* x, int64_t nb, double* y);
int64_t krylov_n(const cphf_ctx* c);

// krylov_block on the device (src/util/krylov_block.rs:39-197)
struct KrylovParams {
  double tol, lindep;
  int64_t max_cycle, max_space;
  bool verbose;
};
// returns true if converged; b, x0 (nullable), x: device [n, nset]
bool krylov_device(cphf_ctx* c, const DeviceOp& aop, const double* b, const double* x0, int64_t n,
                   int64_t nset, const KrylovParams& p, double* x, cphf_stats* st);

// max column 2-norm of b - (I + A) x with the FP64 operator; r receives the residual
double fp64_residual(cphf_ctx* c, const double* b, const double* x, int64_t nset, double* r,
                     cphf_stats* st);

// mixed-precision support
void lowp_prepare(cphf_ctx* c);
void lowp_release(cphf_ctx* c);

// Scope in which the FP64 operator (response_mo_fp64) runs in the FP64-accurate arithmetic of
// the mixed context: mode 0 native FP64, 1 double-float GEMMs, 2 double-float plus the RI-K
// term and XC contractions as exact BF16 slice products on the tensor cores.  `used` is the
// mode in effect (2 falls back to 1 where no tensor-core contraction applies).
struct AccurateScope {
  cphf_ctx* c;
  int used = 0;
  AccurateScope(cphf_ctx* ctx, int mode, int correction_slices = 0);
  ~AccurateScope();
  AccurateScope(const AccurateScope&) = delete;
  AccurateScope& operator=(const AccurateScope&) = delete;
};

}  // namespace cphf
