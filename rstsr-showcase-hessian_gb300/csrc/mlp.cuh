// Learned initial guess / preconditioner (mlp.cu): host-side entry points used by the solver.
#pragma once
#include <cstdint>

#include "ctx.cuh"

namespace cphf {

int mlp_nweights();
void mlp_require(cphf_ctx* c);
// (ia|ia) = sum_P (C_a^T B_P C_i)^2 for every spin (needs the RI-JK plugin and Z)
void mlp_prepare_iaia(cphf_ctx* c);
// x0 (Krylov layout, ld = n) from the right-hand side b; m (length n, may be null) the
// learned left preconditioner of the dimensionless operator
void mlp_guess(cphf_ctx* c, const double* b, int64_t nb, double* x0, double* m);
// y = (m - 1) x + m y  (left-preconditioned operator (I + A) -> m (I + A) = I + [(m - 1) I + m A])
void launch_apply_precond(const double* m, const double* x, double* y, int64_t n, int64_t nb, cudaStream_t s);
// y = m x row-wise
void launch_scale_rows_by(const double* m, const double* x, double* y, int64_t n, int64_t nb, cudaStream_t s);

}  // namespace cphf
