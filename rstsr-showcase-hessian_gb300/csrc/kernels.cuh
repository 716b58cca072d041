// Element-wise, reduction and small dense-algebra kernels of libcphf (host launchers).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace cphf {

// Packed upper triangle [nao_tp, naux] -> dense symmetric [nao, nao, naux] (FP64).
void launch_unpack_cderi(const double* tp, int64_t nao, int64_t naux, double* dense,
                         cudaStream_t s);

// Dimensionless epilogue of response_dimless_cphf (src/hessian/rscf.rs:257-260):
//   out[p, i, a] = 0                                         p <  nocc
//   out[p, i, a] = (y[p-nocc, i, a] - shift x[p, i, a]) / (e[p] - e[i] + shift)   p >= nocc
// y: [nvir, nocc, nb] contiguous; x, out: [nmo, nocc] per column with column stride ldx / ldo.
void launch_dimless(const double* y, const double* x, int64_t ldx, const double* e, int64_t nmo,
                    int64_t nocc, int64_t nb, double shift, double* out, int64_t ldo,
                    cudaStream_t s);
// float input version (split-precision operator output)
void launch_dimless_f32(const float* y, const double* x, int64_t ldx, const double* e, int64_t nmo,
                        int64_t nocc, int64_t nb, double shift, double* out, int64_t ldo,
                        cudaStream_t s);

// XC: rho1[g, a] = sum_i aobra[g, i] ket[g, i, a]   (ket [npts, nocc, nb], g fastest)
template <typename T>
void launch_xc_rho(const T* aobra, int64_t ld_aobra, const T* ket, int64_t npts,
                   int64_t nocc, int64_t nb, T* rho, int64_t ld_rho, cudaStream_t s);
// XC: q[g, i, a] = w[g] * (sum_t f[g, t] rho_t[g, a]) * aobra[g, i], in place of ket.
//   nspin = 1: f[g] (t = 0 only).  nspin = 2: f_t[g] = fxc[g + ng*(t + 2*sout)], rho_t = rho + t*ld_rho_spin.
template <typename T>
void launch_xc_q(const T* aobra, int64_t ld_aobra, const double* w, const double* fxc,
                 int64_t fxc_ld, int nspin, int sout, const T* rho, int64_t ld_rho,
                 int64_t ld_rho_spin, int64_t npts, int64_t nocc, int64_t nb, T* q,
                 cudaStream_t s);
// FP64 -> FP32 copy
void launch_to_f32(const double* src, int64_t n, float* dst, cudaStream_t s);

// r[:, j] = b[:, j] - x[:, j] - ax[:, j] (any pointer may alias r); norms2[j] = ||r[:, j]||^2
// (deterministic two-level reduction).  `partials` needs nblocks_for(n) * nb doubles.
void launch_residual_norms(const double* b, const double* x, const double* ax, double* r,
                           int64_t n, int64_t nb, double* norms2, double* partials,
                           cudaStream_t s);
int64_t residual_partials_size(int64_t n, int64_t nb);

// Right-looking modified Gram-Schmidt over the m columns of V (ld = n), in place,
// following _orth_block / orth_block (src/util/krylov_block.rs:225-253):
// keep[i] = ||v_i||^2 > lindep; ip[i] = ||v_i||^2 after projection.
// `partials`: mgs_partials_size(n, m) doubles.
void launch_mgs(double* V, int64_t n, int64_t m, double lindep, double* ip, int* keep,
                double* partials, cudaStream_t s);
int64_t mgs_partials_size(int64_t n, int64_t m);

// dst[:, j] = src[:, idx[j]] for j < cnt (ld = n both); idx on the device.
void launch_gather_cols(const double* src, int64_t n, const int* idx, int64_t cnt, double* dst,
                        int64_t ld_dst, cudaStream_t s);

// coeff[i, j] /= ip[i]  (coeff [m, nb], ld = ldc)
void launch_scale_rows(double* coeff, int64_t ldc, const double* ip, int64_t m, int64_t nb,
                       cudaStream_t s);

// h[i, i] += ip[i]
void launch_add_diag(double* h, int64_t ldh, const double* ip, int64_t m, cudaStream_t s);

// Solve h c = g in place (LU with partial pivoting); h [m, m] (ld ldh), g [m, nrhs] (ld ldg).
// info (device int) is set to k+1 if a zero pivot is met at step k, else 0.
void launch_lu_solve(double* h, int64_t ldh, double* g, int64_t ldg, int64_t m, int64_t nrhs,
                     int* info, cudaStream_t s);


// y = alpha x + beta y over n elements
void launch_axpby(double alpha, const double* x, double beta, double* y, int64_t n,
                  cudaStream_t s);

// element count of non-finite values in x (device counter, accumulated)
void launch_count_nonfinite(const double* x, int64_t n, int* counter, cudaStream_t s);

// flags[b * nao + m] = 1 if ao[g, m] != 0 for some g of batch b (ao [ngrids, nao], grid fastest)
void launch_nonzero_flags(const double* ao, int64_t ngrids, int64_t nao, const int64_t* offsets,
                          int64_t nbatch, int* flags, cudaStream_t s);

// finalize_cphf element-wise part (src/hessian/rscf.rs:343-350):
//   b1 = f1 - s1 * e[i] + resp;  mo1[vir] = -b1[vir] / (e[a] - e[i]);  mo_e1 = b1[occ] + mo1[occ] * (e[i] - e[j])
// f1, s1, resp, mo1: [nmo, nocc, nprop]; mo_e1: [nocc, nocc, nprop].
void launch_finalize(const double* f1, const double* s1, const double* resp, const double* e,
                     int64_t nmo, int64_t nocc, int64_t nprop, double* mo1, double* mo_e1,
                     cudaStream_t s);

// compute_dimless_cphf_rhs element-wise part (src/hessian/rscf.rs:174-178):
//   rhs[vir] = -(f1mo - s1mo e[i])[vir] / (e[a] - e[i] + shift),  rhs[occ] = -0.5 s1mo[occ]
// f1mo, s1mo, rhs: [nmo, nocc, nprop].
void launch_cphf_rhs(const double* f1, const double* s1, const double* e, int64_t nmo, int64_t nocc, int64_t nprop,
                     double shift, double* rhs, cudaStream_t s);

// get_cphf_hess pair sums (src/hessian/rscf.rs:378-388): G[r, q] += f0 <mo1_r, f1mo_q>
// - f1 <mo1_r, s1mo_q eocc> - f2 <mo_e1_r, s1mo_q[occ]>, r, q over the nprop = 3 natm columns.
void launch_hess_pairs(const double* f1, const double* s1, const double* mo1, const double* mo_e1,
                       const double* e, int64_t nmo, int64_t nocc, int64_t nprop, double f0,
                       double fs, double fe, double* G, cudaStream_t s);
// de[x, y, b, a] = b <= a ? G[(x,b), (y,a)] : G[(y,a), (x,b)]   (rscf.rs:390-396)
void launch_hess_assemble(const double* G, int64_t natm, double* de, cudaStream_t s);

}  // namespace cphf
