// Element-wise, reduction and small dense-algebra kernels, see kernels.cuh.

#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace cphf {
thread_local int64_t* g_launch_counter = nullptr;
std::atomic<int64_t> g_state_generation{0};

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t total, int64_t cap = 1 << 20) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(total, kThreads), cap));
}

__global__ void unpack_cderi_kernel(const double* __restrict__ tp, int64_t nao, int64_t naux,
                                    double* __restrict__ dense) {
  const int64_t nao_tp = nao * (nao + 1) / 2;
  const int64_t per = nao * nao;
  const int64_t total = per * naux;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t P = e / per;
    const int64_t r = e - P * per;
    const int64_t mu = r % nao, nu = r / nao;
    const int64_t lo = mu < nu ? mu : nu, hi = mu < nu ? nu : mu;
    dense[e] = tp[hi * (hi + 1) / 2 + lo + nao_tp * P];
  }
}

template <typename TY>
__global__ void dimless_kernel(const TY* __restrict__ y, const double* __restrict__ x, int64_t ldx,
                               const double* __restrict__ e, int64_t nmo, int64_t nocc, int64_t nb,
                               double shift, double* __restrict__ out, int64_t ldo) {
  const int64_t per = nmo * nocc;
  const int64_t total = per * nb;
  const int64_t nvir = nmo - nocc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = t / per;
    const int64_t r = t - a * per;
    const int64_t p = r % nmo, i = r / nmo;
    double v = 0.0;
    if (p >= nocc) {
      double yv = (double)y[(p - nocc) + nvir * (i + nocc * a)];
      if (shift != 0.0) yv -= shift * x[r + ldx * a];
      v = yv / (e[p] - e[i] + shift);
    }
    out[r + ldo * a] = v;
  }
}

template <typename T>
__global__ void xc_rho_kernel(const T* __restrict__ aobra, int64_t ld_aobra,
                              const T* __restrict__ ket, int64_t npts, int64_t nocc, int64_t nb,
                              T* __restrict__ rho, int64_t ld_rho) {
  const int64_t total = npts * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t % npts, a = t / npts;
    const T* k = ket + g + npts * nocc * a;
    T s = (T)0;
    for (int64_t i = 0; i < nocc; ++i) s = fma(aobra[g + ld_aobra * i], k[npts * i], s);
    rho[g + ld_rho * a] = s;
  }
}

template <typename T>
__global__ void xc_q_kernel(const T* __restrict__ aobra, int64_t ld_aobra,
                            const double* __restrict__ w, const double* __restrict__ fxc,
                            int64_t fxc_ld, int nspin, int sout, const T* __restrict__ rho,
                            int64_t ld_rho, int64_t ld_rho_spin, int64_t npts, int64_t nocc,
                            int64_t nb, T* __restrict__ q) {
  const int64_t total = npts * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t % npts, a = t / npts;
    double f;
    if (nspin == 1) {
      f = fxc[g] * (double)rho[g + ld_rho * a];
    } else {
      f = fxc[g + fxc_ld * (0 + 2 * sout)] * (double)rho[g + ld_rho * a] +
          fxc[g + fxc_ld * (1 + 2 * sout)] * (double)rho[g + ld_rho * a + ld_rho_spin];
    }
    const T wv = (T)(w[g] * f);
    T* qq = q + g + npts * nocc * a;
    for (int64_t i = 0; i < nocc; ++i) qq[npts * i] = wv * aobra[g + ld_aobra * i];
  }
}

// ---- residual and column norms ---------------------------------------------------------
constexpr int kResRowsPerBlock = 2048;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
  }
  __syncthreads();
  return s;  // valid in thread 0
}

__global__ void residual_kernel(const double* __restrict__ b, const double* __restrict__ x,
                                const double* __restrict__ ax, double* __restrict__ r, int64_t n,
                                double* __restrict__ partials) {
  __shared__ double sh[32];
  const int64_t j = blockIdx.y;
  const int64_t r0 = (int64_t)blockIdx.x * kResRowsPerBlock;
  const int64_t r1 = min(n, r0 + kResRowsPerBlock);
  double acc = 0.0;
  for (int64_t row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
    const int64_t e = row + n * j;
    const double v = b[e] - x[e] - ax[e];
    r[e] = v;
    acc = fma(v, v, acc);
  }
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x + (int64_t)gridDim.x * j] = s;
}

__global__ void sum_partials_kernel(const double* __restrict__ partials, int64_t nblk, int64_t nb,
                                    double* __restrict__ out) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nb) return;
  double s = 0.0;
  for (int64_t k = 0; k < nblk; ++k) s += partials[k + nblk * j];
  out[j] = s;
}

// ---- modified Gram-Schmidt --------------------------------------------------------------
constexpr int kMgsMaxRows = 2048;  // rows per block slice (smem 2 x 16 KB)

struct MgsGeom {
  int64_t nblk, rows;
};

MgsGeom mgs_geom(int64_t n) {
  MgsGeom g;
  int64_t nblk = std::min<int64_t>(304, std::max<int64_t>(1, div_up(n, 64)));
  int64_t rows = div_up(n, nblk);
  if (rows > kMgsMaxRows) {
    rows = kMgsMaxRows;
    nblk = div_up(n, rows);
  }
  g.nblk = nblk;
  g.rows = rows;
  return g;
}

// partials[b + nblk * j] = sum over block-b rows of v_j . v_c, for j in [c, m)
__global__ void mgs_init_kernel(const double* __restrict__ V, int64_t n, int64_t m, int64_t c,
                                int64_t rows, double* __restrict__ partials) {
  const int64_t nblk = gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * rows, r1 = min(n, r0 + rows);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t j = c + wid; j < m; j += nw) {
    double acc = 0.0;
    for (int64_t r = r0 + lane; r < r1; r += 32) acc = fma(V[r + n * j], V[r + n * c], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) partials[blockIdx.x + nblk * j] = acc;
  }
}

// sum of the nblk partials of column j: one warp, lanes over blocks, then a shuffle tree
__device__ __forceinline__ double mgs_sum(const double* __restrict__ partials, int64_t nblk, int64_t j, int lane) {
  double s = 0.0;
  for (int64_t k = lane; k < nblk; k += 32) s += partials[k + nblk * j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// Reduce partials of step i: ip[i], keep[i], coef[j] for j > i.  One warp per column (every
// warp first forms the squared norm of column i itself, so that no block waits on another).
__global__ void mgs_reduce_kernel(const double* __restrict__ partials, int64_t nblk, int64_t m,
                                  int64_t i, double lindep, double* __restrict__ ip,
                                  int* __restrict__ keep, double* __restrict__ coef) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double nsq = mgs_sum(partials, nblk, i, lane);
  const bool kept = nsq > lindep;
  if (w == 0 && lane == 0) {
    ip[i] = nsq;
    keep[i] = kept ? 1 : 0;
  }
  for (int64_t j = i + 1 + w; j < m; j += nw) {
    double s = 0.0;
    if (kept) s = mgs_sum(partials, nblk, j, lane) / nsq;
    if (lane == 0) coef[j] = s;
  }
}

// v_j -= coef[j] v_i (j > i), then partials of step i+1.
__global__ void mgs_update_kernel(double* __restrict__ V, int64_t n, int64_t m, int64_t i,
                                  int64_t rows, const double* __restrict__ coef,
                                  const int* __restrict__ keep, double* __restrict__ partials) {
  __shared__ double vi[kMgsMaxRows];
  __shared__ double vn[kMgsMaxRows];
  const int64_t nblk = gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * rows, r1 = min(n, r0 + rows);
  const int64_t len = r1 - r0;
  const bool kept = keep[i] != 0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t r = threadIdx.x; r < len; r += blockDim.x) vi[r] = V[r0 + r + n * i];
  __syncthreads();
  // column i+1 first: it is the projector of the next step
  const int64_t c = i + 1;
  {
    const double cf = kept ? coef[c] : 0.0;
    for (int64_t r = threadIdx.x; r < len; r += blockDim.x) {
      double v = V[r0 + r + n * c];
      if (kept) v = fma(-cf, vi[r], v);
      V[r0 + r + n * c] = v;
      vn[r] = v;
    }
  }
  __syncthreads();
  for (int64_t j = c + wid; j < m; j += nw) {
    const double cf = kept ? coef[j] : 0.0;
    double acc = 0.0;
    for (int64_t r = lane; r < len; r += 32) {
      double v;
      if (j == c) {
        v = vn[r];
      } else {
        v = V[r0 + r + n * j];
        if (kept) {
          v = fma(-cf, vi[r], v);
          V[r0 + r + n * j] = v;
        }
      }
      acc = fma(v, vn[r], acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) partials[blockIdx.x + nblk * j] = acc;
  }
}

__global__ void gather_cols_kernel(const double* __restrict__ src, int64_t n,
                                   const int* __restrict__ idx, int64_t cnt, double* __restrict__ dst,
                                   int64_t ld_dst) {
  const int64_t total = n * cnt;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % n, j = t / n;
    dst[r + ld_dst * j] = src[r + n * (int64_t)idx[j]];
  }
}

__global__ void scale_rows_kernel(double* coeff, int64_t ldc, const double* ip, int64_t m, int64_t nb) {
  const int64_t total = m * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    coeff[i + ldc * j] /= ip[i];
  }
}

__global__ void add_diag_kernel(double* h, int64_t ldh, const double* ip, int64_t m) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < m) h[i + ldh * i] += ip[i];
}

// ---- LU with partial pivoting -----------------------------------------------------------
__global__ void lu_pivot_kernel(double* h, int64_t ldh, double* g, int64_t ldg, int64_t m,
                                int64_t nrhs, int64_t k, int* info) {
  __shared__ double best_v[kThreads];
  __shared__ int64_t best_i[kThreads];
  __shared__ int64_t piv_sh;
  double bv = -1.0;
  int64_t bi = k;
  for (int64_t r = k + threadIdx.x; r < m; r += blockDim.x) {
    const double v = fabs(h[r + ldh * k]);
    if (v > bv) { bv = v; bi = r; }
  }
  best_v[threadIdx.x] = bv;
  best_i[threadIdx.x] = bi;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = -1.0;
    int64_t p = k;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      if (best_v[t] > v || (best_v[t] == v && best_i[t] < p)) { v = best_v[t]; p = best_i[t]; }
    }
    piv_sh = p;
    if (!(v > 0.0) && *info == 0) *info = (int)(k + 1);
  }
  __syncthreads();
  const int64_t p = piv_sh;
  if (p != k) {
    for (int64_t c = threadIdx.x; c < m; c += blockDim.x) {
      const double t = h[k + ldh * c];
      h[k + ldh * c] = h[p + ldh * c];
      h[p + ldh * c] = t;
    }
    for (int64_t c = threadIdx.x; c < nrhs; c += blockDim.x) {
      const double t = g[k + ldg * c];
      g[k + ldg * c] = g[p + ldg * c];
      g[p + ldg * c] = t;
    }
  }
  __syncthreads();
  const double d = h[k + ldh * k];
  if (d != 0.0) {
    for (int64_t r = k + 1 + threadIdx.x; r < m; r += blockDim.x) h[r + ldh * k] /= d;
  }
}

__global__ void lu_update_kernel(double* __restrict__ h, int64_t ldh, double* __restrict__ g,
                                 int64_t ldg, int64_t m, int64_t nrhs, int64_t k) {
  const int64_t rows = m - k - 1;
  const int64_t cols = (m - k - 1) + nrhs;
  const int64_t total = rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = k + 1 + t % rows;
    const int64_t cc = t / rows;
    const double l = h[r + ldh * k];
    if (cc < m - k - 1) {
      const int64_t c = k + 1 + cc;
      h[r + ldh * c] = fma(-l, h[k + ldh * c], h[r + ldh * c]);
    } else {
      const int64_t c = cc - (m - k - 1);
      g[r + ldg * c] = fma(-l, g[k + ldg * c], g[r + ldg * c]);
    }
  }
}

__global__ void lu_backsub_kernel(const double* __restrict__ h, int64_t ldh, double* __restrict__ g,
                                  int64_t ldg, int64_t k) {
  __shared__ double x_sh;
  const int64_t c = blockIdx.x;
  if (threadIdx.x == 0) x_sh = g[k + ldg * c] / h[k + ldh * k];
  __syncthreads();
  const double x = x_sh;
  for (int64_t r = threadIdx.x; r < k; r += blockDim.x) g[r + ldg * c] = fma(-h[r + ldh * k], x, g[r + ldg * c]);
  if (threadIdx.x == 0) g[k + ldg * c] = x;
}

__global__ void axpby_kernel(double alpha, const double* __restrict__ x, double beta,
                             double* __restrict__ y, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    y[t] = alpha * x[t] + (beta == 0.0 ? 0.0 : beta * y[t]);
}

__global__ void count_nonfinite_kernel(const double* __restrict__ x, int64_t n, int* counter) {
  int local = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    local += isfinite(x[t]) ? 0 : 1;
  if (local) atomicAdd(counter, local);
}

}  // namespace

void launch_unpack_cderi(const double* tp, int64_t nao, int64_t naux, double* dense, cudaStream_t s) {
  unpack_cderi_kernel<<<grid_for(nao * nao * naux), kThreads, 0, s>>>(tp, nao, naux, dense);
  count_launch();
}

void launch_dimless(const double* y, const double* x, int64_t ldx, const double* e, int64_t nmo,
                    int64_t nocc, int64_t nb, double shift, double* out, int64_t ldo, cudaStream_t s) {
  dimless_kernel<double><<<grid_for(nmo * nocc * nb), kThreads, 0, s>>>(y, x, ldx, e, nmo, nocc, nb, shift, out, ldo);
  count_launch();
}

void launch_dimless_f32(const float* y, const double* x, int64_t ldx, const double* e, int64_t nmo,
                        int64_t nocc, int64_t nb, double shift, double* out, int64_t ldo,
                        cudaStream_t s) {
  dimless_kernel<float><<<grid_for(nmo * nocc * nb), kThreads, 0, s>>>(y, x, ldx, e, nmo, nocc, nb, shift, out, ldo);
  count_launch();
}

template <typename T>
void launch_xc_rho(const T* aobra, int64_t ld_aobra, const T* ket, int64_t npts,
                   int64_t nocc, int64_t nb, T* rho, int64_t ld_rho, cudaStream_t s) {
  xc_rho_kernel<T><<<grid_for(npts * nb), kThreads, 0, s>>>(aobra, ld_aobra, ket, npts, nocc, nb, rho, ld_rho);
  count_launch();
}
template void launch_xc_rho<double>(const double*, int64_t, const double*, int64_t, int64_t, int64_t, double*, int64_t, cudaStream_t);
template void launch_xc_rho<float>(const float*, int64_t, const float*, int64_t, int64_t, int64_t, float*, int64_t, cudaStream_t);

template <typename T>
void launch_xc_q(const T* aobra, int64_t ld_aobra, const double* w, const double* fxc,
                 int64_t fxc_ld, int nspin, int sout, const T* rho, int64_t ld_rho,
                 int64_t ld_rho_spin, int64_t npts, int64_t nocc, int64_t nb, T* q,
                 cudaStream_t s) {
  xc_q_kernel<T><<<grid_for(npts * nb), kThreads, 0, s>>>(aobra, ld_aobra, w, fxc, fxc_ld, nspin, sout, rho, ld_rho,
                                                         ld_rho_spin, npts, nocc, nb, q);
  count_launch();
}
template void launch_xc_q<double>(const double*, int64_t, const double*, const double*, int64_t, int, int, const double*, int64_t, int64_t, int64_t, int64_t, int64_t, double*, cudaStream_t);
template void launch_xc_q<float>(const float*, int64_t, const double*, const double*, int64_t, int, int, const float*, int64_t, int64_t, int64_t, int64_t, int64_t, float*, cudaStream_t);

__global__ void to_f32_kernel(const double* __restrict__ src, int64_t n, float* __restrict__ dst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = (float)src[t];
}

void launch_to_f32(const double* src, int64_t n, float* dst, cudaStream_t s) {
  if (n <= 0) return;
  to_f32_kernel<<<grid_for(n), kThreads, 0, s>>>(src, n, dst);
  count_launch();
}

int64_t residual_partials_size(int64_t n, int64_t nb) {
  return std::max<int64_t>(1, div_up(n, kResRowsPerBlock)) * nb;
}

void launch_residual_norms(const double* b, const double* x, const double* ax, double* r, int64_t n,
                           int64_t nb, double* norms2, double* partials, cudaStream_t s) {
  if (nb <= 0) return;
  const int64_t nblk = std::max<int64_t>(1, div_up(n, kResRowsPerBlock));
  dim3 grid((unsigned)nblk, (unsigned)nb);
  residual_kernel<<<grid, kThreads, 0, s>>>(b, x, ax, r, n, partials);
  sum_partials_kernel<<<(unsigned)div_up(nb, 128), 128, 0, s>>>(partials, nblk, nb, norms2);
  count_launch(2);
}

int64_t mgs_partials_size(int64_t n, int64_t m) { return mgs_geom(n).nblk * std::max<int64_t>(m, 1); }

void launch_mgs(double* V, int64_t n, int64_t m, double lindep, double* ip, int* keep,
                double* partials, cudaStream_t s) {
  if (m <= 0) return;
  const MgsGeom g = mgs_geom(n);
  // partials [nblk, m] + coef [m] live in the same scratch
  double* coef = partials + g.nblk * m;
  mgs_init_kernel<<<(unsigned)g.nblk, kThreads, 0, s>>>(V, n, m, 0, g.rows, partials);
  count_launch();
  for (int64_t i = 0; i < m; ++i) {
    // one warp per remaining column (8 per block)
    const unsigned rblocks = (unsigned)std::max<int64_t>(1, div_up(m - i, 8));
    mgs_reduce_kernel<<<rblocks, 256, 0, s>>>(partials, g.nblk, m, i, lindep, ip, keep, coef);
    count_launch();
    if (i + 1 < m) {
      mgs_update_kernel<<<(unsigned)g.nblk, kThreads, 0, s>>>(V, n, m, i, g.rows, coef, keep, partials);
      count_launch();
    }
  }
}

void launch_gather_cols(const double* src, int64_t n, const int* idx, int64_t cnt, double* dst,
                        int64_t ld_dst, cudaStream_t s) {
  if (cnt <= 0) return;
  gather_cols_kernel<<<grid_for(n * cnt), kThreads, 0, s>>>(src, n, idx, cnt, dst, ld_dst);
  count_launch();
}

void launch_scale_rows(double* coeff, int64_t ldc, const double* ip, int64_t m, int64_t nb, cudaStream_t s) {
  if (m <= 0 || nb <= 0) return;
  scale_rows_kernel<<<grid_for(m * nb), kThreads, 0, s>>>(coeff, ldc, ip, m, nb);
  count_launch();
}

void launch_add_diag(double* h, int64_t ldh, const double* ip, int64_t m, cudaStream_t s) {
  if (m <= 0) return;
  add_diag_kernel<<<(unsigned)div_up(m, kThreads), kThreads, 0, s>>>(h, ldh, ip, m);
  count_launch();
}

void launch_lu_solve(double* h, int64_t ldh, double* g, int64_t ldg, int64_t m, int64_t nrhs,
                     int* info, cudaStream_t s) {
  CPHF_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
  for (int64_t k = 0; k < m; ++k) {
    lu_pivot_kernel<<<1, kThreads, 0, s>>>(h, ldh, g, ldg, m, nrhs, k, info);
    const int64_t total = (m - k - 1) * ((m - k - 1) + nrhs);
    if (total > 0) lu_update_kernel<<<grid_for(total, 4096), kThreads, 0, s>>>(h, ldh, g, ldg, m, nrhs, k);
    count_launch(total > 0 ? 2 : 1);
  }
  for (int64_t k = m - 1; k >= 0; --k) {
    lu_backsub_kernel<<<(unsigned)nrhs, kThreads, 0, s>>>(h, ldh, g, ldg, k);
    count_launch();
  }
}

void launch_axpby(double alpha, const double* x, double beta, double* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  axpby_kernel<<<grid_for(n), kThreads, 0, s>>>(alpha, x, beta, y, n);
  count_launch();
}

namespace {
__global__ void nonzero_flags_kernel(const double* __restrict__ ao, int64_t ngrids, int64_t nao,
                                     const int64_t* __restrict__ off, int64_t nbatch, int* flags) {
  // one block per (batch, column)
  const int64_t b = blockIdx.x % nbatch, m = blockIdx.x / nbatch;
  const int64_t g0 = off[b], g1 = off[b + 1];
  int any = 0;
  for (int64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) any |= (ao[g + ngrids * m] != 0.0);
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) flags[b * nao + m] = any;
}

__global__ void finalize_kernel(const double* __restrict__ f1, const double* __restrict__ s1,
                                const double* __restrict__ resp, const double* __restrict__ e,
                                int64_t nmo, int64_t nocc, int64_t nprop, double* __restrict__ mo1,
                                double* __restrict__ mo_e1) {
  const int64_t per = nmo * nocc;
  const int64_t total = per * nprop;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = t / per, r = t - a * per;
    const int64_t p = r % nmo, i = r / nmo;
    const double b1 = f1[t] - s1[t] * e[i] + resp[t];
    if (p >= nocc) {
      mo1[t] = -b1 / (e[p] - e[i]);
    } else {
      mo_e1[p + nocc * (i + nocc * a)] = b1 + mo1[t] * (e[p] - e[i]);
    }
  }
}

// compute_dimless_cphf_rhs element-wise part (src/hessian/rscf.rs:174-178):
//   rhs[vir] = -(f1mo - s1mo e_i)[vir] / (e_a - e_i + shift),  rhs[occ] = -0.5 s1mo[occ]
__global__ void cphf_rhs_kernel(const double* __restrict__ f1, const double* __restrict__ s1,
                                const double* __restrict__ e, int64_t nmo, int64_t nocc, int64_t nprop, double shift,
                                double* __restrict__ rhs) {
  const int64_t per = nmo * nocc;
  const int64_t total = per * nprop;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % per;
    const int64_t p = r % nmo, i = r / nmo;
    rhs[t] = p >= nocc ? -(f1[t] - s1[t] * e[i]) / (e[p] - e[i] + shift) : -0.5 * s1[t];
  }
}

__global__ void hess_pairs_kernel(const double* __restrict__ f1, const double* __restrict__ s1,
                                  const double* __restrict__ mo1, const double* __restrict__ mo_e1,
                                  const double* __restrict__ e, int64_t nmo, int64_t nocc, int64_t nprop,
                                  double f0, double fs, double fe, double* __restrict__ G) {
  __shared__ double sh[32];
  const int64_t r = blockIdx.x % nprop, q = blockIdx.x / nprop;
  const int64_t per = nmo * nocc;
  const double* m1 = mo1 + per * r;
  const double* ff = f1 + per * q;
  const double* ss = s1 + per * q;
  const double* me = mo_e1 + nocc * nocc * r;
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < per; t += blockDim.x) {
    const int64_t p = t % nmo, i = t / nmo;
    acc += f0 * m1[t] * ff[t] - fs * m1[t] * ss[t] * e[i];
    if (p < nocc) acc -= fe * me[p + nocc * i] * ss[t];
  }
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) G[r + nprop * q] += s;
}

__global__ void hess_assemble_kernel(const double* __restrict__ G, int64_t natm, double* __restrict__ de) {
  const int64_t np = 3 * natm;
  const int64_t total = 9 * natm * natm;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = t % 3, y = (t / 3) % 3, b = (t / 9) % natm, a = t / (9 * natm);
    de[t] = b <= a ? G[(x + 3 * b) + np * (y + 3 * a)] : G[(y + 3 * a) + np * (x + 3 * b)];
  }
}
}  // namespace

void launch_nonzero_flags(const double* ao, int64_t ngrids, int64_t nao, const int64_t* offsets,
                          int64_t nbatch, int* flags, cudaStream_t s) {
  if (nbatch <= 0 || nao <= 0) return;
  const int64_t blocks = nbatch * nao;
  for (int64_t b0 = 0; b0 < blocks; b0 += (int64_t)1 << 30) {
    // one launch suffices for every realistic size (grid.x < 2^31)
    nonzero_flags_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(ao, ngrids, nao, offsets, nbatch, flags);
    count_launch();
    break;
  }
}

void launch_finalize(const double* f1, const double* s1, const double* resp, const double* e, int64_t nmo,
                     int64_t nocc, int64_t nprop, double* mo1, double* mo_e1, cudaStream_t s) {
  if (nmo * nocc * nprop <= 0) return;
  finalize_kernel<<<grid_for(nmo * nocc * nprop), kThreads, 0, s>>>(f1, s1, resp, e, nmo, nocc, nprop, mo1, mo_e1);
  count_launch();
}

void launch_cphf_rhs(const double* f1, const double* s1, const double* e, int64_t nmo, int64_t nocc, int64_t nprop,
                     double shift, double* rhs, cudaStream_t s) {
  if (nmo * nocc * nprop <= 0) return;
  cphf_rhs_kernel<<<grid_for(nmo * nocc * nprop), kThreads, 0, s>>>(f1, s1, e, nmo, nocc, nprop, shift, rhs);
  count_launch();
}

void launch_hess_pairs(const double* f1, const double* s1, const double* mo1, const double* mo_e1,
                       const double* e, int64_t nmo, int64_t nocc, int64_t nprop, double f0, double fs,
                       double fe, double* G, cudaStream_t s) {
  if (nprop <= 0) return;
  hess_pairs_kernel<<<(unsigned)(nprop * nprop), kThreads, 0, s>>>(f1, s1, mo1, mo_e1, e, nmo, nocc, nprop, f0,
                                                                   fs, fe, G);
  count_launch();
}

void launch_hess_assemble(const double* G, int64_t natm, double* de, cudaStream_t s) {
  if (natm <= 0) return;
  hess_assemble_kernel<<<grid_for(9 * natm * natm), kThreads, 0, s>>>(G, natm, de);
  count_launch();
}

void launch_count_nonfinite(const double* x, int64_t n, int* counter, cudaStream_t s) {
  if (n <= 0) return;
  count_nonfinite_kernel<<<grid_for(n, 2048), kThreads, 0, s>>>(x, n, counter);
  count_launch();
}

}  // namespace cphf
