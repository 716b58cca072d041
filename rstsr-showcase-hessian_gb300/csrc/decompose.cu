// Two-centre metric decomposition and the cderi build, FP64 on the GPU.
//
// Reference: generate_cderi_with_decomp (src/ri_jk/hess_r.rs:1725-1735) with the options of
// RHessRIJK::new_without_cderi (hess_r.rs:1752: Cholesky, threshold 1e-14, Upper):
//   decomp_j2c_cd (src/ri_jk/pure_decompose.rs:29-57)   j2c = U^T U; if the factorisation fails
//       or min diag(U) <= threshold, clamp the eigenvalues of j2c at the threshold,
//       j2c' = V max(e, thr) V^T, and factor j2c' (no second check);
//   solve_by_j2c(j3c, Right, flip_uplo = false) (pure_decompose.rs:205-252)
//       cderi = j3c U^-1, i.e. solve_triangular(U^T, j3c^T, Lower) transposed back.
//
// GPU design (everything FP64, the arithmetic the reference keeps for this step):
//   * blocked right-looking Cholesky of the lower factor L = U^T (j2c = L L^T): a one-CTA kernel
//     factors each 64 x 64 diagonal block in shared memory (records the first non-positive
//     pivot), a row-parallel kernel solves the panel below it, and the trailing update is one
//     FP64 GEMM per block;
//   * the triangular solve X L^T = J (X = cderi, J = j3c, [nao_tp, naux] col-major) runs
//     left-looking over 128-column blocks: S = J_k - X_<k L_k,<k^T (one tall GEMM, K grows with
//     k), X_k = S inv(L_kk)^T (the diagonal blocks inverted once), writing X over J in place;
//   * the eigenvalue fallback is a one-sided (Hestenes) Jacobi eigensolver: round-robin sweeps
//     of n/2 independent column-pair rotations per launch (one CTA per pair) on W = A V and V,
//     until every pair is orthogonal to 1e-15; eigenvalues e_i = v_i . w_i.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "decompose.cuh"
#include "kernels.cuh"

namespace cphf {
namespace {

constexpr int CB = 64;    // Cholesky block
constexpr int TB = 128;   // triangular-solve block
constexpr int kThreads = 256;

unsigned grid1(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(n, kThreads), 1 << 20)); }

// Factor the b x b diagonal block A[k0:k0+b, k0:k0+b] (lower triangle, col-major, ld lda) in
// shared memory: A = L L^T.  info (device) receives k0 + j + 1 at the first pivot that is not
// positive and finite (unchanged when an earlier failure was recorded).
__global__ void chol_diag_kernel(double* __restrict__ A, int64_t lda, int64_t k0, int b, int* info) {
  __shared__ double a[CB][CB + 1];
  __shared__ int bad;
  const int t = threadIdx.x;
  for (int e = t; e < b * b; e += blockDim.x) {
    const int i = e % b, j = e / b;
    a[i][j] = A[(k0 + i) + lda * (k0 + j)];
  }
  if (t == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < b; ++j) {
    if (t == 0) {
      const double d = a[j][j];
      if (!(d > 0.0) || !isfinite(d)) {
        if (!bad) atomicCAS(info, 0, (int)(k0 + j + 1));
        bad = 1;
        a[j][j] = 1.0;  // keep the arithmetic finite; the result is discarded by the host
      } else {
        a[j][j] = sqrt(d);
      }
    }
    __syncthreads();
    const double d = a[j][j];
    for (int i = j + 1 + t; i < b; i += blockDim.x) a[i][j] /= d;
    __syncthreads();
    // trailing update of the lower triangle: a[i][l] -= a[i][j] a[l][j], j < l <= i
    const int m = b - j - 1;
    for (int e = t; e < m * m; e += blockDim.x) {
      const int i = j + 1 + e % m, l = j + 1 + e / m;
      if (l <= i) a[i][l] -= a[i][j] * a[l][j];
    }
    __syncthreads();
  }
  for (int e = t; e < b * b; e += blockDim.x) {
    const int i = e % b, j = e / b;
    if (i >= j) A[(k0 + i) + lda * (k0 + j)] = a[i][j];
  }
}

// Panel below a factored diagonal block: rows r in [k0 + b, n), x L_kk^T = a, in place
// (forward substitution over the b columns; one thread per row, coalesced over rows).
__global__ void chol_panel_kernel(double* __restrict__ A, int64_t lda, int64_t n, int64_t k0, int b) {
  __shared__ double l[CB][CB + 1];
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int i = e % b, j = e / b;
    l[i][j] = i >= j ? A[(k0 + i) + lda * (k0 + j)] : 0.0;
  }
  __syncthreads();
  const int64_t r = k0 + b + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double* row = A + r + lda * k0;
  for (int j = 0; j < b; ++j) {
    double v = row[lda * j];
    for (int q = 0; q < j; ++q) v -= row[lda * q] * l[j][q];
    row[lda * j] = v / l[j][j];
  }
}

// U = L^T (upper, zeros below the diagonal) from the lower factor in A; min |diag| -> dmin bits.
__global__ void chol_upper_kernel(const double* __restrict__ A, int64_t n, double* __restrict__ U,
                                  unsigned long long* dmin) {
  const int64_t total = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, j = e / n;  // U[i, j]
    U[e] = i <= j ? A[j + n * i] : 0.0;
    if (i == j) atomicMin(dmin, (unsigned long long)__double_as_longlong(fabs(A[i + n * i])));
  }
}

// inv(L_kk) for every diagonal block of width <= TB of the lower factor L [n, n]: block k is
// written to inv + k * TB * TB as a w x w col-major lower-triangular matrix; one CTA per block,
// one thread per column of the inverse (forward substitution on L_kk e_j).
__global__ void tri_inv_blocks_kernel(const double* __restrict__ L, int64_t n, double* __restrict__ inv) {
  extern __shared__ double sl[];  // [TB][TB + 1]
  const int64_t k0 = (int64_t)blockIdx.x * TB;
  const int w = (int)(n - k0 < TB ? n - k0 : TB);
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int i = e % w, j = e / w;
    sl[i * (TB + 1) + j] = i >= j ? L[(k0 + i) + n * (k0 + j)] : 0.0;
  }
  __syncthreads();
  const int j = threadIdx.x;
  if (j >= w) return;
  double* x = inv + (int64_t)blockIdx.x * TB * TB + (int64_t)w * j;  // column j of the inverse
  for (int i = 0; i < w; ++i) {
    if (i < j) {
      x[i] = 0.0;
      continue;
    }
    double v = i == j ? 1.0 : 0.0;
    for (int q = j; q < i; ++q) v -= sl[i * (TB + 1) + q] * x[q];
    x[i] = v / sl[i * (TB + 1) + i];
  }
}

// One round of the one-sided Jacobi sweep: CTA c rotates the column pair of round r in the
// circle ordering of m = n rounded up to even (pairs with an index >= n are skipped).
__global__ void jacobi_round_kernel(double* __restrict__ W, double* __restrict__ V, int64_t n, int64_t m, int64_t r,
                                    double tol, unsigned long long* __restrict__ offmax) {
  __shared__ double red[3][32];
  __shared__ double cs[2];
  const int64_t i = blockIdx.x;
  int64_t p, q;
  if (i == 0) {
    p = 0;
    q = 1 + r % (m - 1);
  } else {
    p = 1 + (r + i) % (m - 1);
    q = 1 + (r - i + (m - 1)) % (m - 1);
  }
  if (p >= n || q >= n) return;
  double* wp = W + n * p;
  double* wq = W + n * q;
  double a = 0.0, b = 0.0, g = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
    const double x = wp[k], y = wq[k];
    a += x * x;
    b += y * y;
    g += x * y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    g += __shfl_xor_sync(0xffffffffu, g, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = a;
    red[1][warp] = b;
    red[2][warp] = g;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = g = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += red[0][w];
      b += red[1][w];
      g += red[2][w];
    }
    const double nrm = sqrt(a * b);
    double c = 1.0, s = 0.0;
    if (nrm > 0.0 && fabs(g) > tol * nrm) {
      const double off = fabs(g) / nrm;
      atomicMax(offmax, (unsigned long long)__double_as_longlong(off));
      // rotation [c s; -s c] zeroing the (p, q) inner product (Rutishauser's formulas)
      const double zeta = (b - a) / (2.0 * g);
      const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      c = 1.0 / sqrt(1.0 + t * t);
      s = c * t;
    }
    cs[0] = c;
    cs[1] = s;
  }
  __syncthreads();
  const double c = cs[0], s = cs[1];
  if (s == 0.0) return;
  double* vp = V + n * p;
  double* vq = V + n * q;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
    const double x = wp[k], y = wq[k];
    wp[k] = c * x - s * y;
    wq[k] = s * x + c * y;
    const double u = vp[k], v = vq[k];
    vp[k] = c * u - s * v;
    vq[k] = s * u + c * v;
  }
}

// e_i = v_i . w_i (the eigenvalue of column i once W = A V has orthogonal columns), clamped:
// T[:, i] = V[:, i] max(e_i, thr); one block per column.
__global__ void jacobi_eigs_kernel(const double* __restrict__ W, const double* __restrict__ V, int64_t n, double thr,
                                   double* __restrict__ e, double* __restrict__ T) {
  __shared__ double red[32];
  __shared__ double ev;
  const int64_t i = blockIdx.x;
  double acc = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) acc += V[k + n * i] * W[k + n * i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    e[i] = s;
    ev = fmax(s, thr);
  }
  __syncthreads();
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) T[k + n * i] = V[k + n * i] * ev;
}

__global__ void identity_kernel(double* __restrict__ V, int64_t n) {
  const int64_t total = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    V[e] = (e % n) == (e / n) ? 1.0 : 0.0;
}

// Lower factor L of the symmetric A [n, n] (col-major, overwritten: L in the lower triangle).
// Returns 0, or k + 1 for the first pivot k that is not positive and finite.
int cholesky_lower(cphf_ctx* c, double* A, int64_t n, int* info_dev) {
  cudaStream_t s = c->stream;
  CPHF_CUDA(cudaMemsetAsync(info_dev, 0, sizeof(int), s));
  for (int64_t k0 = 0; k0 < n; k0 += CB) {
    const int b = (int)std::min<int64_t>(CB, n - k0);
    chol_diag_kernel<<<1, kThreads, 0, s>>>(A, n, k0, b, info_dev);
    count_launch();
    const int64_t rest = n - k0 - b;
    if (rest <= 0) break;
    chol_panel_kernel<<<(unsigned)div_up(rest, 128), 128, 0, s>>>(A, n, n, k0, b);
    count_launch();
    GemmDesc g;  // A[r, r'] -= L[r, k] L[r', k], r, r' >= k0 + b (full square of the trailing block)
    g.M = rest; g.N = rest; g.K = b;
    g.A = A + (k0 + b) + n * k0; g.a_m = 1; g.a_k = n;
    g.B = A + (k0 + b) + n * k0; g.b_k = n; g.b_n = 1;
    g.C = A + (k0 + b) + n * (k0 + b); g.c_m = 1; g.c_n = n;
    g.alpha = -1.0; g.beta = 1.0;
    gemm64(c, g);
  }
  CPHF_CUDA(cudaGetLastError());
  int info = 0;
  CPHF_CUDA(cudaMemcpyAsync(&info, info_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
  CPHF_CUDA(cudaStreamSynchronize(s));
  return info;
}

// Eigenvalues clamped at thr and the matrix rebuilt: A <- V max(e, thr) V^T (A symmetric [n, n]).
void eig_clamp(cphf_ctx* c, double* A, int64_t n, double thr, DecompWork& w) {
  cudaStream_t s = c->stream;
  w.W.ensure((size_t)n * n * 8, c->counter());
  w.V.ensure((size_t)n * n * 8, c->counter());
  w.e.ensure((size_t)n * 8, c->counter());
  w.flag.ensure(16, c->counter());
  double* W = w.W.as<double>();
  double* V = w.V.as<double>();
  CPHF_CUDA(cudaMemcpyAsync(W, A, (size_t)n * n * 8, cudaMemcpyDeviceToDevice, s));
  identity_kernel<<<grid1(n * n), kThreads, 0, s>>>(V, n);
  count_launch();
  const int64_t m = n + (n & 1);
  const double tol = 1e-15;
  w.sweeps = 0;
  for (int sweep = 0; sweep < 40; ++sweep) {
    CPHF_CUDA(cudaMemsetAsync(w.flag.p, 0, 8, s));
    for (int64_t r = 0; r < m - 1; ++r) {
      jacobi_round_kernel<<<(unsigned)(m / 2), kThreads, 0, s>>>(W, V, n, m, r, tol, w.flag.as<unsigned long long>());
      count_launch();
    }
    CPHF_CUDA(cudaGetLastError());
    unsigned long long bits = 0;
    CPHF_CUDA(cudaMemcpyAsync(&bits, w.flag.p, 8, cudaMemcpyDeviceToHost, s));
    CPHF_CUDA(cudaStreamSynchronize(s));
    ++w.sweeps;
    double off;
    std::memcpy(&off, &bits, 8);
    if (bits == 0 || off <= tol) break;
  }
  // T = V max(e, thr) (in W), A = T V^T
  jacobi_eigs_kernel<<<(unsigned)n, kThreads, 0, s>>>(W, V, n, thr, w.e.as<double>(), W);
  count_launch();
  GemmDesc g;
  g.M = n; g.N = n; g.K = n;
  g.A = W; g.a_m = 1; g.a_k = n;
  g.B = V; g.b_k = n; g.b_n = 1;
  g.C = A; g.c_m = 1; g.c_n = n;
  gemm64(c, g);
}

}  // namespace

J2cDecomp j2c_cholesky(cphf_ctx* c, const double* j2c_dev, int64_t naux, double threshold, DecompWork& w) {
  J2cDecomp out;
  cudaStream_t s = c->stream;
  w.A.ensure((size_t)naux * naux * 8, c->counter());
  w.flag.ensure(16, c->counter());
  w.info.ensure(sizeof(int), c->counter());
  double* A = w.A.as<double>();
  CPHF_CUDA(cudaMemcpyAsync(A, j2c_dev, (size_t)naux * naux * 8, cudaMemcpyDeviceToDevice, s));
  const int info = cholesky_lower(c, A, naux, w.info.as<int>());
  auto min_diag = [&]() {
    w.U.ensure((size_t)naux * naux * 8, c->counter());
    CPHF_CUDA(cudaMemsetAsync(w.flag.p, 0xFF, 8, s));
    chol_upper_kernel<<<grid1(naux * naux), kThreads, 0, s>>>(A, naux, w.U.as<double>(), w.flag.as<unsigned long long>());
    count_launch();
    unsigned long long bits = 0;
    CPHF_CUDA(cudaMemcpyAsync(&bits, w.flag.p, 8, cudaMemcpyDeviceToHost, s));
    CPHF_CUDA(cudaStreamSynchronize(s));
    double d;
    std::memcpy(&d, &bits, 8);
    return d;
  };
  if (info == 0) {
    out.min_diag = min_diag();
    if (threshold < 0.0 || out.min_diag > threshold) return out;  // pure_decompose.rs:36-41
  } else if (threshold < 0.0) {
    throw Error(CPHF_ERR_NONFINITE, "Cholesky decomposition of j2c failed at pivot " + std::to_string(info) +
                                        " and no threshold is given for the eigenvalue fallback");
  }
  // pure_decompose.rs:44-51: clamp the eigenvalues at the threshold, factor again without a check
  CPHF_CUDA(cudaMemcpyAsync(A, j2c_dev, (size_t)naux * naux * 8, cudaMemcpyDeviceToDevice, s));
  eig_clamp(c, A, naux, threshold, w);
  const int info2 = cholesky_lower(c, A, naux, w.info.as<int>());
  if (info2 != 0)
    throw Error(CPHF_ERR_NONFINITE, "Cholesky decomposition of the eigenvalue-clamped j2c failed at pivot " +
                                        std::to_string(info2));
  out.fallback = true;
  out.sweeps = w.sweeps;
  out.min_diag = min_diag();
  return out;
}

void solve_by_j2c_right(cphf_ctx* c, double* J, int64_t n, int64_t naux, DecompWork& w) {
  cudaStream_t s = c->stream;
  const double* L = w.A.as<double>();  // lower factor from j2c_cholesky
  const int64_t nblk = div_up(naux, TB);
  w.inv.ensure((size_t)nblk * TB * TB * 8, c->counter());
  static bool attr = false;
  const int smem = TB * (TB + 1) * 8;
  if (!attr) {
    CPHF_CUDA(cudaFuncSetAttribute(tri_inv_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr = true;
  }
  tri_inv_blocks_kernel<<<(unsigned)nblk, TB, smem, s>>>(L, naux, w.inv.as<double>());
  count_launch();
  CPHF_CUDA(cudaGetLastError());
  if (n == 0) return;
  w.S.ensure((size_t)n * TB * 8, c->counter());
  double* S = w.S.as<double>();
  for (int64_t k = 0; k < nblk; ++k) {
    const int64_t k0 = k * TB, wd = std::min<int64_t>(TB, naux - k0);
    CPHF_CUDA(cudaMemcpyAsync(S, J + n * k0, (size_t)n * wd * 8, cudaMemcpyDeviceToDevice, s));
    if (k0 > 0) {
      GemmDesc g;  // S -= X[:, :k0] L[k0:k0+wd, :k0]^T
      g.M = n; g.N = wd; g.K = k0;
      g.A = J; g.a_m = 1; g.a_k = n;
      g.B = L + k0; g.b_k = naux; g.b_n = 1;
      g.C = S; g.c_m = 1; g.c_n = n;
      g.alpha = -1.0; g.beta = 1.0;
      gemm64(c, g);
    }
    GemmDesc x;  // X_k = S inv(L_kk)^T
    x.M = n; x.N = wd; x.K = wd;
    x.A = S; x.a_m = 1; x.a_k = n;
    x.B = w.inv.as<double>() + k * TB * TB; x.b_k = wd; x.b_n = 1;
    x.C = J + n * k0; x.c_m = 1; x.c_n = n;
    gemm64(c, x);
  }
}

}  // namespace cphf
