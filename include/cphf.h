/*
 * cphf.h -- C ABI of the GB300 CPHF/CPKS response library (libcphf.so).
 *
 * Drop-in boundary for the CPHF response path of rstsr-showcase-hessian: the
 * RI-J/RI-K response plugin, the numint XC response plugin, the block-Krylov
 * solver and the CPHF driver steps around it.  Every entry point names the
 * reference item it replaces (paths inside the reference project).
 *
 * Conventions
 *  - All arrays are FP64 and col-major (F-order), as in the reference
 *    (src/lib.rs:40-48, src/util/krylov_block.rs:13-16).  Shapes are written
 *    [fastest, ..., slowest].
 *  - A data pointer may point to host memory (pageable or pinned) or to device
 *    memory of the context's GPU; the library detects which and copies
 *    accordingly.  Inputs are borrowed for the duration of the call only.
 *  - Orbitals are ordered occupied first (src/hessian/rscf.rs:253-254).
 *  - Where the reference panics (check_shape!, src/util/panic_handling.rs:36-58;
 *    non-convergence, src/util/krylov_block.rs:188-194) the call returns a
 *    status code; cphf_last_error() gives the message.
 *  - One context per host thread; calls on a context are serialized on the
 *    context's CUDA stream (the reference's &mut self plugin methods,
 *    src/hessian/trait_rhess.rs:162, 189 and src/hessian/trait_uhess.rs:152, 171).
 */
#ifndef CPHF_H
#define CPHF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cphf_status {
  CPHF_OK = 0,
  CPHF_ERR_SHAPE = 1,          /* shape mismatch (check_shape!) */
  CPHF_ERR_NOT_CONVERGED = 2,  /* krylov_block failed to converge */
  CPHF_ERR_NONFINITE = 3,      /* NaN/Inf found in an input or a residual */
  CPHF_ERR_OOM = 4,            /* device allocation failed */
  CPHF_ERR_CUDA = 5,           /* CUDA runtime error */
  CPHF_ERR_TIMEOUT = 6,        /* a bounded device-side wait ran out */
  CPHF_ERR_STATE = 7,          /* call order (e.g. response before prepare) */
  CPHF_ERR_ARG = 8             /* invalid argument */
} cphf_status;

/* Arithmetic of the solve. */
typedef enum cphf_precision {
  CPHF_PRECISION_FP64 = 0,   /* every contraction in FP64 (the reference's arithmetic) */
  CPHF_PRECISION_MIXED = 1   /* split-FP16 tensor-core operator inside FP64 defect correction */
} cphf_precision;

/* HessSCFConfig (src/hessian/rscf.rs:5-18) plus the GPU-side options. */
typedef struct cphf_config {
  double level_shift;        /* default 0.0 */
  double cphf_tol;           /* default 1e-8 */
  int64_t cphf_max_cycle;    /* default 42 */
  int64_t cphf_max_space;    /* default 14 */
  double cphf_lindep;        /* default 1e-14 */
  int32_t precision;         /* cphf_precision, default CPHF_PRECISION_FP64 */
  int32_t device;            /* CUDA device ordinal, default 0 */
  double residual_tol;       /* mixed: stop when max column ||b-(I+A)x||_2 < residual_tol (default 1e-8) */
  double inner_tol;          /* mixed: Krylov tol of the first inner solve, relative to the residual (default
                                1e-6); later inner solves use max(inner_tol, min(1e-2, 0.1 residual_tol / |r|)),
                                the reduction that the remaining residual |r| still needs (until one of them
                                misses the target) */
  int64_t max_refine;        /* mixed: maximum defect-correction steps (default 6) */
  int32_t use_learned_guess; /* learned per-pair MLP (weights set by cphf_mlp_set_weights), default 0 = off.
                                MIXED: 1 = left preconditioner of the first inner solve (the later corrections
                                solve the plain operator), 2 = preconditioner and initial guess of the first
                                inner solve (the guess costs one more operator application for its residual).  FP64: any non-zero value = initial guess
                                x0 only (the Krylov iteration and stopping test stay the reference's). */
  int32_t verbose;           /* print per-cycle diagnostics like krylov_block.rs:148-151 (default 0) */
  int64_t aux_chunk;         /* aux functions per K-term chunk (default 0 = automatic) */
  int32_t tensor_cores;      /* mixed: 1 = tcgen05 split-FP16 K term (default), 0 = FP32 CUDA cores */
  int32_t verify_residual;   /* mixed: how the residual of every correction after the first is obtained and
                                convergence decided.  0 = updated with the split-precision operator,
                                r -= (I + A_lowp) d (no FP64-accurate application);  1 = recomputed with
                                the native FP64 operator;  2 (default) = computed with the FP64-accurate
                                operator of residual_dfloat: with the exact-slice tensor cores (residual_dfloat
                                = 2) as r -= (I + A) d, the correction d applied in correction precision:
                                the fewest BF16 slices per operand whose error bound (3 slices, 6
                                exact-accumulated products: ~2^-14 |r|; 4 slices, 10 products: ~2^-20 |r|)
                                stays below 0.1 residual_tol, else all six; otherwise recomputed in full.
                                With 1 or 2 the solve returns only after such a max_j ||b_j - (I+A)x_j||_2
                                < residual_tol. */
  int32_t fp64_every_step;   /* mixed: FP64 residual after every correction, not only the first (default 0) */
  int64_t xc_chunk_points;   /* grid points per XC chunk (default 0 = 8 GiB of intermediates) */
  int32_t residual_dfloat;   /* mixed: arithmetic of the correction residuals.  0 = native FP64;
                                1 = double-float GEMMs on the FP32 pipes (~1e-14 relative);
                                2 = as 1, with the whole RI-K term and the XC grid contractions on the
                                tensor cores as exact BF16 slice products (6 x 6 bits, ~1e-10 relative
                                to the operand row maxima; default; without tensor cores it behaves
                                as 1).
                                verify_residual = 1 recomputes the later residuals in native FP64. */
  int32_t cuda_graphs;       /* mixed: replay each block width's split-precision operator application
                                from a captured CUDA graph (default 1); bypassed while profiling */
} cphf_config;

/* Solver statistics (the reference reports them by println!, krylov_block.rs:148-151, 175). */
typedef struct cphf_stats {
  int64_t aop_calls;            /* operator applications inside the Krylov solver(s) */
  int64_t aop_columns;          /* sum of the block widths of those applications */
  int64_t cycles;               /* Krylov cycles (summed over restarts and refinement steps) */
  int64_t restarts;             /* hard restarts */
  double max_innerprod;         /* last max ||new trial||^2 (the reference's convergence signal) */
  double residual_max;          /* max column 2-norm of b - (I+A)x, FP64, after the solve */
  int64_t fp64_matvec_columns;  /* columns pushed through the FP64 operator */
  int64_t lowp_matvec_columns;  /* columns pushed through the split-precision operator */
  int64_t refine_steps;         /* defect-correction steps (mixed precision) */
  double seconds;               /* wall time of the call */
  int64_t residual_mode;        /* how residual_max was computed: 0 native FP64, 1 double-float GEMMs,
                                   2 double-float + exact BF16 slice products on the tensor cores,
                                   3 updated with the split-precision operator, 4 as 2 for the first
                                   correction, later corrections subtracted with the exact-slice operator
                                   in correction precision, -1 not computed */
} cphf_stats;

typedef struct cphf_ctx cphf_ctx;

/* Operator callback for cphf_krylov_block: y[:, 0:nblock] = A x[:, 0:nblock],
 * col-major [n, nblock] DEVICE arrays, work issued on `stream` (a cudaStream_t).
 * Return 0 on success.  Mirrors `aop: impl FnMut(TsrView) -> Tsr`
 * (src/util/krylov_block.rs:40). */
typedef int (*cphf_aop_fn)(void* user, const double* x, int64_t n, int64_t nblock, double* y,
                           void* stream);

/* ---- context ---------------------------------------------------------------------------- */
cphf_status cphf_config_default(cphf_config* cfg);
cphf_status cphf_ctx_create(const cphf_config* cfg, cphf_ctx** out);
cphf_status cphf_ctx_destroy(cphf_ctx* ctx);
cphf_status cphf_ctx_set_config(cphf_ctx* ctx, const cphf_config* cfg);
const char* cphf_status_string(cphf_status s);
const char* cphf_last_error(const cphf_ctx* ctx);
void* cphf_ctx_stream(const cphf_ctx* ctx);            /* the context's cudaStream_t */
cphf_status cphf_ctx_synchronize(cphf_ctx* ctx);
int64_t cphf_ctx_device_bytes(const cphf_ctx* ctx);   /* device memory held by the context */
/* Number of kernels this context launched so far (launch counter, for benchmarks). */
int64_t cphf_ctx_kernel_launches(const cphf_ctx* ctx);
/* 1 when the split-precision operator runs its K term on the tensor cores (tcgen05). */
int32_t cphf_ctx_tensor_cores_active(const cphf_ctx* ctx);

/* Per-kernel-class timing with CUDA events (replaces the reference's wall-clock timing
 * vectors, src/hessian/rscf.rs:33).  Enabling clears the records. */
typedef struct cphf_prof_entry {
  char name[32];
  int64_t launches;
  double ms;       /* summed event time */
  double max_ms;   /* longest single launch */
  double flops;    /* algorithmic FLOPs of the recorded launches */
  double bytes;    /* algorithmic bytes of the recorded launches */
} cphf_prof_entry;
cphf_status cphf_ctx_profile(cphf_ctx* ctx, int32_t enable);
/* Fills up to `max` entries (one per kernel class with records); returns the count, or -1. */
int32_t cphf_ctx_profile_report(cphf_ctx* ctx, cphf_prof_entry* out, int32_t max);

/* ---- RI-JK plugin ---------------------------------------------------------------------- */
/* RHessRIJK::new_with_cderi (src/ri_jk/hess_r.rs:1774-1794) / UHessRIJK:
 * cderi [nao*(nao+1)/2, naux], packed upper triangle, element (mu<=nu) at
 * nu*(nu+1)/2+mu (src/util/density_matrices.rs:48-57, hess_r.rs:1725-1735). */
cphf_status cphf_rijk_set_cderi(cphf_ctx* ctx, const double* cderi, int64_t nao, int64_t naux,
                                double scale_j, double scale_k);

/* ---- cderi construction: two-centre metric decomposition and triangular solve (FP64) --- */
/* Outcome of a j2c decomposition. */
typedef struct cphf_j2c_info {
  int32_t eig_fallback;      /* 1 when the eigenvalue-clamping fallback was taken */
  int32_t jacobi_sweeps;     /* sweeps of the fallback's Jacobi eigensolver */
  double min_diag;           /* min diag(U) of the returned factor */
  double seconds_decompose;  /* wall time of the decomposition */
  double seconds_solve;      /* wall time of the triangular solve (cphf_rijk_set_j3c) */
} cphf_j2c_info;

/* decomp_j2c_cd(j2c, threshold, Upper) (src/ri_jk/pure_decompose.rs:29-57): j2c [naux, naux]
 * = U^T U, U upper triangular written to j2c_u [naux, naux] (zeros below the diagonal).  When
 * the factorisation fails or min diag(U) <= threshold, the eigenvalues of j2c are clamped at
 * the threshold and the rebuilt matrix is factored without a further check (pure_decompose.rs:
 * 44-51).  threshold < 0 means no fallback: a failed factorisation returns CPHF_ERR_NONFINITE
 * (the reference panics, pure_decompose.rs:56).  info may be NULL. */
cphf_status cphf_j2c_decompose(cphf_ctx* ctx, const double* j2c, int64_t naux, double threshold, double* j2c_u,
                               cphf_j2c_info* info);
/* generate_cderi_with_decomp (src/ri_jk/hess_r.rs:1725-1735) with the options of
 * RHessRIJK::new_without_cderi (hess_r.rs:1752: Cholesky, threshold 1e-14, Upper) from
 * caller-supplied integrals, then RHessRIJK::new_with_cderi on the result:
 *   j3c [nao*(nao+1)/2, naux] packed (mu nu|P) (same layout as cphf_rijk_set_cderi's cderi),
 *   j2c [naux, naux] (P|Q);  cderi = j3c U^-1 with j2c = U^T U (solve_by_j2c(j3c, Right,
 *   flip_uplo = false), pure_decompose.rs:205-252), FP64 on the GPU.
 * The RI-JK plugin then uses this cderi exactly as if passed to cphf_rijk_set_cderi. */
cphf_status cphf_rijk_set_j3c(cphf_ctx* ctx, const double* j3c, const double* j2c, int64_t nao, int64_t naux,
                              double scale_j, double scale_k, double threshold, cphf_j2c_info* info);
/* Copy the RI-JK plugin's packed cderi [nao*(nao+1)/2, naux] out (host or device pointer). */
cphf_status cphf_rijk_get_cderi(cphf_ctx* ctx, double* cderi);

/* ---- XC plugin (LDA / XCDenType::RHO, src/xceff/flags.rs:33-55) ----------------------- */
/* RHessKSNIMatmul / UHessKSNIMatmul with intmd["cpks_fxc"] (src/numint_matmul/hess_rks.rs:814-824, 895):
 *   ao      [ngrids, nao]  AO values (derivative order 0), the reference's get_cached_ao(0) tensor
 *   weights [ngrids]
 *   fxc     nspin=1: [ngrids] = fxc_eff[g,0,0];  nspin=2: [ngrids, 2, 2] = fxc_eff[g,0,s_in,0,s_out]
 *   batch_offsets [nbatch+1] grid batches (e.g. per atom); NULL = one batch.
 * Must be called after cphf_rijk_set_cderi or cphf_set_nao (nao is taken from there). */
cphf_status cphf_xc_set_grid(cphf_ctx* ctx, const double* ao, const double* weights,
                             const double* fxc, int64_t ngrids, int32_t nspin,
                             const int64_t* batch_offsets, int64_t nbatch);
/* The same plugin for every density type of the reference (XCDenType, src/xceff/flags.rs:33-55):
 *   den_type 0 RHO (LDA, nvar 1), 1 SIGMA (GGA, nvar 4: rho and its gradient), 2 TAU (meta-GGA,
 *   nvar 5: plus tau);
 *   ao [ngrids, nao, ncomp]: AO values (component 0) and first derivatives x, y, z (1-3), the
 *     reference's get_cached_ao(1) tensor; SIGMA / TAU need ncomp >= 4 (only 0-3 are read);
 *   fxc_eff nspin=1: [ngrids, nvar, nvar]; nspin=2: [ngrids, nvar, 2, nvar, 2] (x, s_in, y, s_out),
 *     the reference's intmd["cpks_fxc"];
 *   batch_offsets: as for cphf_xc_set_grid (RHO only; SIGMA / TAU chunk the points themselves).
 * RHO is cphf_xc_set_grid on component 0.  SIGMA / TAU evaluate rho1's gradient / tau terms
 * (pure_eval_rho.rs:289-316) and contract_ao_wv_bra's (pure_xcpot.rs:335-351) with dense AO
 * values on the CUDA cores (FP64; FP32 in the mixed solve's inner operator). */
cphf_status cphf_xc_set_grid_ex(cphf_ctx* ctx, int32_t den_type, const double* ao, int32_t ncomp,
                                const double* weights, const double* fxc_eff, int64_t ngrids, int32_t nspin,
                                const int64_t* batch_offsets, int64_t nbatch);
/* Declare nao when no RI-JK plugin is used. */
cphf_status cphf_set_nao(cphf_ctx* ctx, int64_t nao);

/* ---- response preparation and response (RHessElecInteractAPI) --------------------------- */
/* make_response_preparation (src/hessian/trait_rhess.rs:162, trait_uhess.rs:152; hess_r.rs:1911-1914,
 * hess_rks.rs:886-889) plus the orbital energies the CPHF driver keeps (rscf.rs:21-25):
 *   mo_coeff[s] [nao, nmo], mo_occ[s] [nmo], mo_energy[s] [nmo], s < nspin (1 = RHF/RKS, 2 = UHF/UKS). */
cphf_status cphf_prepare(cphf_ctx* ctx, int32_t nspin, const double* const* mo_coeff,
                         const double* const* mo_occ, const double* const* mo_energy, int64_t nmo);

/* get_response_bra (src/hessian/trait_rhess.rs:189, trait_uhess.rs:171) summed over the set
 * plugins (rscf.rs:210-220 loop body):
 *   bra[s], out[s] [nao, nocc_s, nprop].
 *   RHF: hess_r.rs:1916-1953 (+ hess_rks.rs:891-908); UHF: hess_u.rs:270-313 (+ hess_uks.rs:740-764). */
cphf_status cphf_response_bra(cphf_ctx* ctx, const double* const* bra, int64_t nprop,
                              double* const* out);
/* One plugin only: which = 0 RI-JK, 1 XC. */
cphf_status cphf_plugin_response_bra(cphf_ctx* ctx, int32_t which, const double* const* bra,
                                     int64_t nprop, double* const* out);

/* ---- CPHF driver (src/hessian/rscf.rs, uscf.rs) ----------------------------------------- */
/* response_mo (rscf.rs:210-220, uscf.rs:203-218): mo1[s], resp[s] [nmo, nocc_s, nprop]. */
cphf_status cphf_response_mo(cphf_ctx* ctx, const double* const* mo1, int64_t nprop,
                             double* const* resp);
/* response_dimless_cphf (rscf.rs:237-263, uscf.rs:230-265). */
cphf_status cphf_response_dimless(cphf_ctx* ctx, const double* const* mo1, int64_t nprop,
                                  double* const* resp);
/* The same operator in the split-precision arithmetic of the mixed solve (FP32 / tensor cores);
 * valid after cphf_prepare on a context configured with CPHF_PRECISION_MIXED. */
cphf_status cphf_response_dimless_lowp(cphf_ctx* ctx, const double* const* mo1, int64_t nprop,
                                       double* const* resp);
/* solve_dimless_cphf (rscf.rs:278-300, uscf.rs:278-341): rhs[s], mo1[s] [nmo, nocc_s, nprop];
 * x0 may be NULL.  FP64: krylov_block with the fused dimensionless operator.
 * MIXED: the same solver on the split-precision operator inside FP64 defect correction. */
cphf_status cphf_solve_dimless_cphf(cphf_ctx* ctx, const double* const* rhs, int64_t nprop,
                                    const double* const* x0, double* const* mo1, cphf_stats* stats);
/* compute_dimless_cphf_rhs (rscf.rs:104-182, uscf.rs:78-173) from the summed skeleton
 * derivatives of the providers:  f1ao_core [nao, nao, 3, natm] (core-Hamiltonian derivatives,
 * spin independent; NULL = 0), f1bra_el[s] [nao, nocc_s, 3, natm] (the electron-interaction
 * plugins' get_deriv1_bra, half-transformed; NULL or a NULL entry = 0), s1ao [nao, nao, 3, natm]
 * (overlap derivatives).  Out, per spin, [nmo, nocc_s, 3, natm]: rhs (vir: -(f1mo - s1mo e_i) /
 * (e_a - e_i + level_shift); occ: -0.5 s1mo), f1mo = C^T (f1ao_core Cocc + f1bra_el),
 * s1mo = C^T s1ao Cocc.  FP64. */
cphf_status cphf_compute_dimless_cphf_rhs(cphf_ctx* ctx, const double* f1ao_core, const double* const* f1bra_el,
                                          const double* s1ao, int64_t natm, double* const* rhs, double* const* f1mo,
                                          double* const* s1mo);
/* finalize_cphf (rscf.rs:328-353, uscf.rs:365-406): f1mo[s], s1mo[s] [nmo, nocc_s, 3, natm];
 * mo1[s] in/out; mo_e1[s] [nocc_s, nocc_s, 3, natm] out.  Its one response_mo (rscf.rs:342)
 * runs in native FP64 on an FP64 context and in the FP64-accurate arithmetic selected by
 * residual_dfloat on a MIXED context. */
cphf_status cphf_finalize_cphf(cphf_ctx* ctx, const double* const* f1mo, const double* const* s1mo,
                               int64_t natm, double* const* mo1, double* const* mo_e1);
/* get_cphf_hess (rscf.rs:371-399, uscf.rs:408-446): de [3, 3, natm, natm]. */
cphf_status cphf_get_cphf_hess(cphf_ctx* ctx, const double* const* f1mo, const double* const* s1mo,
                               const double* const* mo1, const double* const* mo_e1, int64_t natm,
                               double* de);

/* ---- block Krylov solver ---------------------------------------------------------------- */
/* krylov_block (src/util/krylov_block.rs:39-197) with a caller-supplied operator:
 * b, x [n, nset]; x0 may be NULL. */
cphf_status cphf_krylov_block(cphf_ctx* ctx, cphf_aop_fn aop, void* user, const double* b,
                              const double* x0, int64_t n, int64_t nset, double tol,
                              int64_t max_cycle, int64_t max_space, double lindep, double* x,
                              cphf_stats* stats);

/* A dense FP64 operator y = A x (A [n, n] col-major, copied to the device), usable as the
 * aop of cphf_krylov_block: pass cphf_dense_op_apply and the op as `user`.  This is the
 * operator of the reference's solver tests (tests/test_krylov_block.rs:18-23). */
typedef struct cphf_dense_op cphf_dense_op;
cphf_status cphf_dense_op_create(cphf_ctx* ctx, const double* A, int64_t n, cphf_dense_op** out);
int cphf_dense_op_apply(void* user, const double* x, int64_t n, int64_t nblock, double* y,
                        void* stream);
cphf_status cphf_dense_op_destroy(cphf_dense_op* op);

/* Copy `bytes` between any host / device pointers on the context's stream and wait. */
cphf_status cphf_copy(cphf_ctx* ctx, void* dst, const void* src, int64_t bytes);

/* ---- allocation-free RI-J response (no counterpart in the reference) -------------------- */
/* For callers that cannot allocate device memory (code running under another framework's
 * allocator or memory budget, or recording work where allocation is not allowed): the
 * Coulomb part of the RI-JK response in bra form, out = scale_j * J[D1] Cocc, computed with
 * no cudaMalloc, no cudaFree and no allocating library call, and without a context.
 *   Z   [nao, nocc, naux]  Z_P = B_P Cocc (device)
 *   bra [nao, nocc, nb], out [nao, nocc, nb] (device), FP64 col-major; stream: a cudaStream_t or NULL.
 * The one intermediate, d[naux, nb], lives in a static 8 MiB device array of the library:
 * naux * nb must not exceed cphf_rij_noalloc_capacity() (1,048,576), else CPHF_ERR_ARG is
 * returned and nothing runs.  The first call on a device resolves that array's device
 * address (cudaGetSymbolAddress) with the device current; make that first call before any
 * stream capture.  All calls share the array: calls that overlap on the GPU (different
 * streams, or different host threads on one device) race and must be serialized by the caller. */
int64_t cphf_rij_noalloc_capacity(void);
cphf_status cphf_rij_response_bra_noalloc(const double* Z, const double* bra, int64_t nao, int64_t nocc,
                                          int64_t naux, int64_t nb, double scale_j, double* out,
                                          void* stream);

/* ---- learned initial guess / preconditioner (no counterpart in the reference) ------------ */
/* Per-(i,a)-pair MLP 3 -> 64 -> 64 -> 2 (GELU), FP32 weights packed as
 * W1[64,3] b1[64] W2[64,64] b2[64] W3[2,64] b3[2] (row-major per matrix), 4546 floats.
 * Sample features [n, 3] (row-major): gap e_a - e_i, dimensionless RHS entry b, (ia|ia).
 * Outputs [n, 2]: o1 (initial guess x0 = b (1 + o1)), o2 (effective diagonal d of the
 * dimensionless operator; preconditioner 1 / (1 + d)).  With use_learned_guess set, a mixed
 * solve left-preconditions its first inner solve (1) and also starts it from the guess (2); an
 * FP64 solve only starts from the guess.  The unmodified operator still defines convergence
 * (mixed: the FP64-accurate residual; FP64: the reference's stopping test), so the answer is
 * unchanged. */
cphf_status cphf_mlp_set_weights(cphf_ctx* ctx, const float* weights, int64_t nweights);
cphf_status cphf_mlp_get_weights(cphf_ctx* ctx, float* weights, int64_t nweights);
/* Features of every (vir a, occ i, column r) sample of rhs[s] [nmo, nocc_s, nprop]
 * (order: spin, then r slowest, then i, a fastest); *n_out receives the count, `feat` may be
 * NULL to query it. */
cphf_status cphf_mlp_features(cphf_ctx* ctx, const double* const* rhs, int64_t nprop, float* feat,
                              int64_t cap, int64_t* n_out);
/* Network outputs; bf16 != 0 selects the BF16 inference kernel, else FP32. */
cphf_status cphf_mlp_forward(cphf_ctx* ctx, const float* feat, int64_t n, float* out, int32_t bf16);
/* Mean loss (b (1 + o1) - x*)^2 + (o2 - d*)^2 and its gradient [4546]; target [n, 2] = (x*, d*). */
cphf_status cphf_mlp_loss_grad(cphf_ctx* ctx, const float* feat, const float* target, int64_t n,
                               float* loss, float* grad);
/* Adam training on the GPU: `epochs` passes over shuffled minibatches; history[epochs] gets
 * the mean minibatch loss per epoch (may be NULL). */
cphf_status cphf_mlp_train(cphf_ctx* ctx, const float* feat, const float* target, int64_t n,
                           int64_t epochs, int64_t batch, float lr, uint64_t seed, float* history);

#ifdef __cplusplus
}
#endif
#endif /* CPHF_H */
