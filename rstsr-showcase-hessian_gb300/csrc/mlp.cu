// Learned initial guess and diagonal preconditioner: a per-(i,a)-pair MLP trained and
// evaluated on the GPU by the kernels below.  No counterpart in the reference.
//
// Network 3 -> 64 (GELU) -> 64 (GELU) -> 2, FP32 weights packed row-major as
// W1[64,3] b1[64] W2[64,64] b2[64] W3[2,64] b3[2].  Raw features per sample are the
// orbital-energy gap e_a - e_i, the dimensionless right-hand-side entry b and the RI
// diagonal (ia|ia) = sum_P (C_a^T B_P C_i)^2; the network sees u = (log gap, 10 b,
// 4 (ia|ia) / gap).  Outputs: o1 gives the initial guess x0 = b (1 + o1); o2 (evaluated
// with b = 0) is the effective diagonal d of the dimensionless operator and gives the left
// preconditioner m = 1 / (1 + d) of the Krylov iteration.  Training loss per sample:
// (b (1 + o1) - x*)^2 + (o2 - d*)^2 with x* the converged solution and d* its effective
// diagonal.  Training: FP32 forward/backward per 128-sample block, fixed-order gradient
// reduction, Adam.  Inference: BF16 weights and activations with FP32 accumulation.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "ctx.cuh"
#include "kernels.cuh"
#include "mlp.cuh"

namespace cphf {
namespace {

constexpr int H = 64;
constexpr int NW = H * 3 + H + H * H + H + 2 * H + 2;  // 4546
constexpr int OW1 = 0, OB1 = OW1 + H * 3, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + 2 * H;
constexpr int BS = 128;  // samples (threads) per training block

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.3989422804014327f;
}

__device__ __forceinline__ void net_inputs(const float* f, float* u) {
  const float gap = f[0];
  u[0] = logf(gap);
  u[1] = 10.f * f[1];
  u[2] = 4.f * f[2] / gap;
}

// ---- FP32 forward (evaluation) -----------------------------------------------------------
__global__ void mlp_forward_kernel(const float* __restrict__ w, const float* __restrict__ feat, int64_t n,
                                   float* __restrict__ out) {
  __shared__ float sw[NW];
  for (int k = threadIdx.x; k < NW; k += blockDim.x) sw[k] = w[k];
  __syncthreads();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  float u[3];
  net_inputs(feat + 3 * t, u);
  float h1[H];
#pragma unroll 8
  for (int j = 0; j < H; ++j)
    h1[j] = gelu(sw[OB1 + j] + sw[OW1 + 3 * j] * u[0] + sw[OW1 + 3 * j + 1] * u[1] + sw[OW1 + 3 * j + 2] * u[2]);
  float o0 = sw[OB3], o1 = sw[OB3 + 1];
  for (int j = 0; j < H; ++j) {
    float z = sw[OB2 + j];
#pragma unroll 16
    for (int k = 0; k < H; ++k) z = fmaf(sw[OW2 + H * j + k], h1[k], z);
    const float h = gelu(z);
    o0 = fmaf(sw[OW3 + j], h, o0);
    o1 = fmaf(sw[OW3 + H + j], h, o1);
  }
  out[2 * t] = o0;
  out[2 * t + 1] = o1;
}

// ---- BF16 inference -----------------------------------------------------------------------
__global__ void mlp_infer_bf16_kernel(const float* __restrict__ w, const float* __restrict__ feat, int64_t n,
                                      float* __restrict__ out) {
  __shared__ __nv_bfloat16 sw[NW];
  for (int k = threadIdx.x; k < NW; k += blockDim.x) sw[k] = __float2bfloat16(w[k]);
  __syncthreads();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  float u[3];
  net_inputs(feat + 3 * t, u);
  __nv_bfloat16 h1[H];
#pragma unroll 8
  for (int j = 0; j < H; ++j) {
    float z = __bfloat162float(sw[OB1 + j]);
    for (int c = 0; c < 3; ++c) z = fmaf(__bfloat162float(sw[OW1 + 3 * j + c]), __bfloat162float(__float2bfloat16(u[c])), z);
    h1[j] = __float2bfloat16(gelu(z));
  }
  float o0 = __bfloat162float(sw[OB3]), o1 = __bfloat162float(sw[OB3 + 1]);
  for (int j = 0; j < H; ++j) {
    float z = __bfloat162float(sw[OB2 + j]);
#pragma unroll 16
    for (int k = 0; k < H; ++k) z = fmaf(__bfloat162float(sw[OW2 + H * j + k]), __bfloat162float(h1[k]), z);
    const float h = __bfloat162float(__float2bfloat16(gelu(z)));
    o0 = fmaf(__bfloat162float(sw[OW3 + j]), h, o0);
    o1 = fmaf(__bfloat162float(sw[OW3 + H + j]), h, o1);
  }
  out[2 * t] = o0;
  out[2 * t + 1] = o1;
}

// ---- training: forward + backward per block, per-block gradient partials ------------------
// Shared layout (floats): weights NW | act[4][H][BS] (h1, g1, h2/d2, g2) | u[3][BS] | dz[2][BS] | red[BS]
constexpr int TRAIN_SMEM = (NW + 4 * H * BS + 3 * BS + 2 * BS + BS) * 4;

__global__ void __launch_bounds__(BS) mlp_grad_kernel(const float* __restrict__ w, const float* __restrict__ feat,
                                                      const float* __restrict__ target, const int* __restrict__ idx,
                                                      int64_t n, float inv_n, float* __restrict__ partial,
                                                      float* __restrict__ loss_partial) {
  extern __shared__ float sm[];
  float* sw = sm;
  float* h1 = sw + NW;
  float* g1 = h1 + H * BS;
  float* h2 = g1 + H * BS;
  float* g2 = h2 + H * BS;
  float* su = g2 + H * BS;
  float* dz = su + 3 * BS;
  float* red = dz + 2 * BS;
  const int t = threadIdx.x;
  for (int k = t; k < NW; k += BS) sw[k] = w[k];
  const int64_t s_glob = (int64_t)blockIdx.x * BS + t;
  const bool valid = s_glob < n;
  float u[3] = {0.f, 0.f, 0.f}, bval = 0.f, tx = 0.f, td = 0.f;
  if (valid) {
    const int64_t s = idx ? idx[s_glob] : s_glob;
    net_inputs(feat + 3 * s, u);
    bval = feat[3 * s + 1];
    tx = target[2 * s];
    td = target[2 * s + 1];
  }
  for (int c = 0; c < 3; ++c) su[c * BS + t] = u[c];
  __syncthreads();
  // forward
  for (int j = 0; j < H; ++j) {
    const float z = sw[OB1 + j] + sw[OW1 + 3 * j] * u[0] + sw[OW1 + 3 * j + 1] * u[1] + sw[OW1 + 3 * j + 2] * u[2];
    h1[j * BS + t] = gelu(z);
    g1[j * BS + t] = gelu_grad(z);
  }
  float o0 = sw[OB3], o1 = sw[OB3 + 1];
  for (int j = 0; j < H; ++j) {
    float z = sw[OB2 + j];
    for (int k = 0; k < H; ++k) z = fmaf(sw[OW2 + H * j + k], h1[k * BS + t], z);
    const float h = gelu(z);
    h2[j * BS + t] = h;
    g2[j * BS + t] = gelu_grad(z);
    o0 = fmaf(sw[OW3 + j], h, o0);
    o1 = fmaf(sw[OW3 + H + j], h, o1);
  }
  // loss and output gradients (zero for padding samples)
  const float r1 = bval * (1.f + o0) - tx, r2 = o1 - td;
  red[t] = valid ? (r1 * r1 + r2 * r2) : 0.f;
  const float d0 = valid ? 2.f * r1 * bval * inv_n : 0.f;
  const float d1 = valid ? 2.f * r2 * inv_n : 0.f;
  dz[t] = d0;
  dz[BS + t] = d1;
  __syncthreads();
  float* gp = partial + (int64_t)blockIdx.x * NW;
  // dW3, db3
  for (int q = t; q < 2 * H + 2; q += BS) {
    float acc = 0.f;
    if (q < 2 * H) {
      const int k = q / H, j = q % H;
      for (int s = 0; s < BS; ++s) acc = fmaf(dz[k * BS + s], h2[j * BS + s], acc);
      gp[OW3 + q] = acc;
    } else {
      const int k = q - 2 * H;
      for (int s = 0; s < BS; ++s) acc += dz[k * BS + s];
      gp[OB3 + k] = acc;
    }
  }
  if (t == 0) {
    float acc = 0.f;
    for (int s = 0; s < BS; ++s) acc += red[s];
    loss_partial[blockIdx.x] = acc;
  }
  __syncthreads();
  // delta2 = (dz W3) * g2, stored over h2
  for (int j = 0; j < H; ++j) h2[j * BS + t] = (d0 * sw[OW3 + j] + d1 * sw[OW3 + H + j]) * g2[j * BS + t];
  __syncthreads();
  // dW2[j][k] = sum_s d2[j][s] h1[k][s]; db2
  for (int q = t; q < H * H + H; q += BS) {
    float acc = 0.f;
    if (q < H * H) {
      const int j = q / H, k = q % H;
      for (int s = 0; s < BS; ++s) acc = fmaf(h2[j * BS + s], h1[k * BS + s], acc);
      gp[OW2 + q] = acc;
    } else {
      const int j = q - H * H;
      for (int s = 0; s < BS; ++s) acc += h2[j * BS + s];
      gp[OB2 + j] = acc;
    }
  }
  // delta1 = (d2 W2) * g1, stored over g1 (per thread: own sample column)
  for (int k = 0; k < H; ++k) {
    float acc = 0.f;
    for (int j = 0; j < H; ++j) acc = fmaf(h2[j * BS + t], sw[OW2 + H * j + k], acc);
    g1[k * BS + t] = acc * g1[k * BS + t];
  }
  __syncthreads();
  for (int q = t; q < 3 * H + H; q += BS) {
    float acc = 0.f;
    if (q < 3 * H) {
      const int j = q / 3, c = q % 3;
      for (int s = 0; s < BS; ++s) acc = fmaf(g1[j * BS + s], su[c * BS + s], acc);
      gp[OW1 + q] = acc;
    } else {
      const int j = q - 3 * H;
      for (int s = 0; s < BS; ++s) acc += g1[j * BS + s];
      gp[OB1 + j] = acc;
    }
  }
}

// fixed-order sum of the per-block partials
__global__ void mlp_reduce_kernel(const float* __restrict__ partial, int64_t nblk, float* __restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= NW) return;
  float acc = 0.f;
  for (int64_t b = 0; b < nblk; ++b) acc += partial[b * NW + k];
  grad[k] = acc;
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= NW) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  w[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

// ---- features, guess and preconditioner -----------------------------------------------------
// iaia[a, i] = sum_P bmo[a, (i, P)]^2   (bmo [nvir, nocc * naux] from one GEMM)
__global__ void iaia_kernel(const float* __restrict__ bmo, int64_t nvir, int64_t nocc, int64_t naux,
                            float* __restrict__ iaia) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nvir * nocc) return;
  const int64_t a = t % nvir, i = t / nvir;
  float acc = 0.f;
  for (int64_t P = 0; P < naux; ++P) {
    const float v = bmo[a + nvir * (i + nocc * P)];
    acc = fmaf(v, v, acc);
  }
  iaia[t] = acc;
}

__global__ void add_f32_kernel(const float* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    y[t] += x[t];
}

// samples (a, i, r) of one spin: feat[3 * (off + a + nvir * (i + nocc * r))]
__global__ void features_kernel(const double* __restrict__ b, int64_t ldb, const double* __restrict__ e,
                                const float* __restrict__ iaia, int64_t nmo, int64_t nocc, int64_t nb,
                                float bscale, float* __restrict__ feat) {
  const int64_t nvir = nmo - nocc;
  const int64_t total = nvir * nocc * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = t % nvir, i = (t / nvir) % nocc, r = t / (nvir * nocc);
    feat[3 * t] = (float)(e[nocc + a] - e[i]);
    feat[3 * t + 1] = b ? (float)(bscale * b[(nocc + a) + nmo * i + ldb * r]) : 0.f;
    feat[3 * t + 2] = iaia[a + nvir * i];
  }
}

// x0 = b (1 + o1) on virtual rows, b on occupied rows
__global__ void guess_kernel(const double* __restrict__ b, int64_t ldb, const float* __restrict__ o, int64_t nmo,
                             int64_t nocc, int64_t nb, double* __restrict__ x0, int64_t ldx) {
  const int64_t per = nmo * nocc;
  const int64_t nvir = nmo - nocc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < per * nb; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / per, q = t % per, p = q % nmo, i = q / nmo;
    const double bv = b[q + ldb * r];
    double v = bv;
    if (p >= nocc) v = bv * (1.0 + (double)o[2 * ((p - nocc) + nvir * (i + nocc * r))]);
    x0[q + ldx * r] = v;
  }
}

// m[p, i] = 1 / (1 + max(d, -0.5)) on virtual rows, 1 on occupied rows
__global__ void precond_kernel(const float* __restrict__ o, int64_t nmo, int64_t nocc, double* __restrict__ m) {
  const int64_t per = nmo * nocc, nvir = nmo - nocc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < per; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t % nmo, i = t / nmo;
    double v = 1.0;
    if (p >= nocc) v = 1.0 / (1.0 + fmax((double)o[2 * ((p - nocc) + nvir * i) + 1], -0.5));
    m[t] = v;
  }
}

// y = (m - 1) x + m y over [n, nb], m per row
__global__ void apply_precond_kernel(const double* __restrict__ m, const double* __restrict__ x, double* __restrict__ y,
                                     int64_t n, int64_t nb) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * nb; t += (int64_t)gridDim.x * blockDim.x) {
    const double mv = m[t % n];
    y[t] = (mv - 1.0) * x[t] + mv * y[t];
  }
}

__global__ void scale_rows_by_kernel(const double* __restrict__ m, const double* __restrict__ x, double* __restrict__ y,
                                     int64_t n, int64_t nb) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * nb; t += (int64_t)gridDim.x * blockDim.x)
    y[t] = m[t % n] * x[t];
}

unsigned blocks_for(int64_t total) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(total, 256), 1 << 20));
}

}  // namespace

int mlp_nweights() { return NW; }

void mlp_require(cphf_ctx* c) {
  if (!c->mlp || c->mlp->w.p == nullptr) throw Error(CPHF_ERR_STATE, "MLP weights are not set");
}

void mlp_upload(cphf_ctx* c, const float* w) {
  if (!c->mlp) c->mlp.reset(new MlpState());
  MlpState& M = *c->mlp;
  M.w.ensure(NW * 4, c->counter());
  M.m.ensure(NW * 4, c->counter());
  M.v.ensure(NW * 4, c->counter());
  M.g.ensure(NW * 4, c->counter());
  CPHF_CUDA(cudaMemcpyAsync(M.w.p, w, NW * 4, cudaMemcpyDefault, c->stream));
  CPHF_CUDA(cudaMemsetAsync(M.m.p, 0, NW * 4, c->stream));
  CPHF_CUDA(cudaMemsetAsync(M.v.p, 0, NW * 4, c->stream));
  M.step = 0;
}

void mlp_forward(cphf_ctx* c, const float* feat, int64_t n, float* out, bool bf16) {
  mlp_require(c);
  if (n <= 0) return;
  if (bf16)
    mlp_infer_bf16_kernel<<<(unsigned)div_up(n, 128), 128, 0, c->stream>>>(c->mlp->w.as<float>(), feat, n, out);
  else
    mlp_forward_kernel<<<(unsigned)div_up(n, 128), 128, 0, c->stream>>>(c->mlp->w.as<float>(), feat, n, out);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

float mlp_loss_grad(cphf_ctx* c, const float* feat, const float* target, const int* idx, int64_t n, float* grad) {
  mlp_require(c);
  static bool attr = false;
  if (!attr) {
    CPHF_CUDA(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM));
    attr = true;
  }
  MlpState& M = *c->mlp;
  const int64_t nblk = div_up(n, BS);
  M.part.ensure((size_t)nblk * (NW + 1) * 4, c->counter());
  float* part = M.part.as<float>();
  float* lossp = part + nblk * NW;
  mlp_grad_kernel<<<(unsigned)nblk, BS, TRAIN_SMEM, c->stream>>>(M.w.as<float>(), feat, target, idx, n, 1.f / (float)n,
                                                                part, lossp);
  mlp_reduce_kernel<<<(NW + 255) / 256, 256, 0, c->stream>>>(part, nblk, grad);
  count_launch(2);
  CPHF_CUDA(cudaGetLastError());
  std::vector<float> lp(nblk);
  CPHF_CUDA(cudaMemcpyAsync(lp.data(), lossp, nblk * 4, cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  double s = 0.0;
  for (float v : lp) s += v;
  return (float)(s / (double)n);
}

void mlp_train(cphf_ctx* c, const float* feat, const float* target, int64_t n, int64_t epochs, int64_t batch,
               float lr, uint64_t seed, float* history) {
  mlp_require(c);
  MlpState& M = *c->mlp;
  std::mt19937_64 rng(seed);
  std::vector<int> perm(n);
  M.idx.ensure((size_t)std::max<int64_t>(n, 1) * sizeof(int), c->counter());
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int64_t ep = 0; ep < epochs; ++ep) {
    for (int64_t k = 0; k < n; ++k) perm[k] = (int)k;
    std::shuffle(perm.begin(), perm.end(), rng);
    CPHF_CUDA(cudaMemcpyAsync(M.idx.p, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    double acc = 0.0;
    int64_t nbat = 0;
    for (int64_t s0 = 0; s0 < n; s0 += batch) {
      const int64_t nb = std::min<int64_t>(batch, n - s0);
      const float loss = mlp_loss_grad(c, feat, target, M.idx.as<int>() + s0, nb, M.g.as<float>());
      ++M.step;
      const float c1 = 1.f - std::pow(b1, (float)M.step), c2 = 1.f - std::pow(b2, (float)M.step);
      adam_kernel<<<(NW + 255) / 256, 256, 0, c->stream>>>(M.w.as<float>(), M.g.as<float>(), M.m.as<float>(),
                                                           M.v.as<float>(), lr, b1, b2, c1, c2, eps);
      count_launch();
      acc += loss;
      ++nbat;
    }
    if (history) history[ep] = (float)(acc / std::max<int64_t>(nbat, 1));
  }
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
}

void mlp_prepare_iaia(cphf_ctx* c) {
  if (!c->has_rijk) throw Error(CPHF_ERR_STATE, "the MLP features need the RI-JK plugin (RI diagonal)");
  for (int s = 0; s < c->nspin; ++s) {
    SpinState& sp = c->spin[s];
    const int64_t nvir = sp.nmo - sp.nocc, no = sp.nocc, nao = c->nao, naux = c->naux;
    sp.iaia.ensure((size_t)std::max<int64_t>(nvir * no, 1) * 4, c->counter());
    if (nvir == 0 || no == 0) continue;
    // bmo[a, (i, P)] = sum_mu C[mu, nocc + a] Z[mu, (i, P)] in aux chunks
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(naux, (int64_t(1) << 28) / (nvir * no * 4)));
    DevBuf bmo, acc;
    bmo.ensure((size_t)nvir * no * chunk * 4, c->counter());
    acc.ensure((size_t)nvir * no * 4, c->counter());
    CPHF_CUDA(cudaMemsetAsync(sp.iaia.p, 0, nvir * no * 4, c->stream));
    for (int64_t P0 = 0; P0 < naux; P0 += chunk) {
      const int64_t np = std::min<int64_t>(chunk, naux - P0);
      GemmDesc d;
      d.M = nvir; d.N = no * np; d.K = nao;
      d.A = sp.C.as<double>() + no * nao; d.a_m = nao; d.a_k = 1;
      d.B = sp.Z.as<double>() + P0 * nao * no; d.b_k = 1; d.b_n = nao;
      d.C = bmo.p; d.c_m = 1; d.c_n = nvir;
      gemm32x<double, double, float>(c, d);
      iaia_kernel<<<blocks_for(nvir * no), 256, 0, c->stream>>>(bmo.as<float>(), nvir, no, np, acc.as<float>());
      add_f32_kernel<<<blocks_for(nvir * no), 256, 0, c->stream>>>(acc.as<float>(), sp.iaia.as<float>(), nvir * no);
      count_launch(2);
    }
  }
}

int64_t mlp_features(cphf_ctx* c, const double* b, int64_t nb, float* feat, bool zero_b) {
  const int64_t n = krylov_n(c);
  int64_t off = 0, ooff = 0;
  for (int s = 0; s < c->nspin; ++s) {
    const SpinState& sp = c->spin[s];
    const int64_t nvir = sp.nmo - sp.nocc;
    features_kernel<<<blocks_for(nvir * sp.nocc * nb), 256, 0, c->stream>>>(
        zero_b ? nullptr : b + off, n, sp.e.as<double>(), sp.iaia.as<float>(), sp.nmo, sp.nocc, nb, 1.f,
        feat + 3 * ooff);
    count_launch();
    off += sp.nmo * sp.nocc;
    ooff += nvir * sp.nocc * nb;
  }
  CPHF_CUDA(cudaGetLastError());
  return ooff;
}

void mlp_guess(cphf_ctx* c, const double* b, int64_t nb, double* x0, double* m) {
  mlp_require(c);
  MlpState& M = *c->mlp;
  const int64_t n = krylov_n(c);
  int64_t nsamp = 0, npair = 0;
  for (int s = 0; s < c->nspin; ++s) {
    nsamp += (c->spin[s].nmo - c->spin[s].nocc) * c->spin[s].nocc * nb;
    npair += (c->spin[s].nmo - c->spin[s].nocc) * c->spin[s].nocc;
  }
  M.feat.ensure((size_t)std::max<int64_t>(nsamp, 1) * 3 * 4, c->counter());
  M.out.ensure((size_t)std::max<int64_t>(nsamp, 1) * 2 * 4, c->counter());
  // initial guess from the right-hand side
  mlp_features(c, b, nb, M.feat.as<float>(), false);
  mlp_forward(c, M.feat.as<float>(), nsamp, M.out.as<float>(), true);
  int64_t off = 0, ooff = 0;
  for (int s = 0; s < c->nspin; ++s) {
    const SpinState& sp = c->spin[s];
    guess_kernel<<<blocks_for(sp.nmo * sp.nocc * nb), 256, 0, c->stream>>>(b + off, n, M.out.as<float>() + 2 * ooff,
                                                                          sp.nmo, sp.nocc, nb, x0 + off, n);
    count_launch();
    off += sp.nmo * sp.nocc;
    ooff += (sp.nmo - sp.nocc) * sp.nocc * nb;
  }
  if (m) {  // preconditioner from the pair features alone (b = 0)
    mlp_features(c, nullptr, 1, M.feat.as<float>(), true);
    mlp_forward(c, M.feat.as<float>(), npair, M.out.as<float>(), true);
    off = 0;
    ooff = 0;
    for (int s = 0; s < c->nspin; ++s) {
      const SpinState& sp = c->spin[s];
      precond_kernel<<<blocks_for(sp.nmo * sp.nocc), 256, 0, c->stream>>>(M.out.as<float>() + 2 * ooff, sp.nmo,
                                                                         sp.nocc, m + off);
      count_launch();
      off += sp.nmo * sp.nocc;
      ooff += (sp.nmo - sp.nocc) * sp.nocc;
    }
  }
  CPHF_CUDA(cudaGetLastError());
}

void launch_apply_precond(const double* m, const double* x, double* y, int64_t n, int64_t nb, cudaStream_t s) {
  apply_precond_kernel<<<blocks_for(n * nb), 256, 0, s>>>(m, x, y, n, nb);
  count_launch();
}

void launch_scale_rows_by(const double* m, const double* x, double* y, int64_t n, int64_t nb, cudaStream_t s) {
  scale_rows_by_kernel<<<blocks_for(n * nb), 256, 0, s>>>(m, x, y, n, nb);
  count_launch();
}

}  // namespace cphf

using namespace cphf;

namespace {
template <typename F>
cphf_status mlp_guarded(cphf_ctx* c, F&& f) {
  if (!c) return CPHF_ERR_ARG;
  int64_t* prev = g_launch_counter;
  g_launch_counter = &c->launches;
  try {
    CPHF_CUDA(cudaSetDevice(c->device));
    f();
    g_launch_counter = prev;
    return CPHF_OK;
  } catch (const Error& e) {
    g_launch_counter = prev;
    c->last_error = e.what();
    return e.status;
  }
}
}  // namespace

extern "C" {

cphf_status cphf_mlp_set_weights(cphf_ctx* c, const float* weights, int64_t nweights) {
  return mlp_guarded(c, [&] {
    CPHF_CHECK_SHAPE(weights != nullptr && nweights == NW, "MLP weights must hold " + std::to_string(NW) + " floats");
    mlp_upload(c, weights);
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_mlp_get_weights(cphf_ctx* c, float* weights, int64_t nweights) {
  return mlp_guarded(c, [&] {
    mlp_require(c);
    CPHF_CHECK_SHAPE(weights != nullptr && nweights == NW, "MLP weights must hold " + std::to_string(NW) + " floats");
    CPHF_CUDA(cudaMemcpyAsync(weights, c->mlp->w.p, NW * 4, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_mlp_features(cphf_ctx* c, const double* const* rhs, int64_t nprop, float* feat, int64_t cap,
                              int64_t* n_out) {
  return mlp_guarded(c, [&] {
    if (!c->prepared) throw Error(CPHF_ERR_STATE, "cphf_prepare has not been called");
    CPHF_CHECK_ARG(rhs && n_out, "null arrays");
    if (c->spin[0].iaia.p == nullptr) mlp_prepare_iaia(c);
    const int64_t n = krylov_n(c);
    int64_t nsamp = 0;
    for (int s = 0; s < c->nspin; ++s) nsamp += (c->spin[s].nmo - c->spin[s].nocc) * c->spin[s].nocc * nprop;
    *n_out = nsamp;
    if (!feat) return;
    CPHF_CHECK_SHAPE(cap >= nsamp, "feature buffer too small");
    DevBuf b, f;
    b.ensure((size_t)std::max<int64_t>(n * nprop, 1) * 8, c->counter());
    f.ensure((size_t)std::max<int64_t>(nsamp, 1) * 12, c->counter());
    int64_t off = 0;
    for (int s = 0; s < c->nspin; ++s) {
      const int64_t len = c->spin[s].nmo * c->spin[s].nocc;
      if (len > 0)
        CPHF_CUDA(cudaMemcpy2DAsync(b.as<double>() + off, n * 8, rhs[s], len * 8, len * 8, nprop, cudaMemcpyDefault,
                                    c->stream));
      off += len;
    }
    mlp_features(c, b.as<double>(), nprop, f.as<float>(), false);
    CPHF_CUDA(cudaMemcpyAsync(feat, f.p, nsamp * 12, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_mlp_forward(cphf_ctx* c, const float* feat, int64_t n, float* out, int32_t bf16) {
  return mlp_guarded(c, [&] {
    CPHF_CHECK_ARG(feat && out && n >= 0, "invalid arguments");
    DevBuf f, o;
    f.ensure((size_t)std::max<int64_t>(n, 1) * 12, c->counter());
    o.ensure((size_t)std::max<int64_t>(n, 1) * 8, c->counter());
    CPHF_CUDA(cudaMemcpyAsync(f.p, feat, n * 12, cudaMemcpyDefault, c->stream));
    mlp_forward(c, f.as<float>(), n, o.as<float>(), bf16 != 0);
    CPHF_CUDA(cudaMemcpyAsync(out, o.p, n * 8, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_mlp_loss_grad(cphf_ctx* c, const float* feat, const float* target, int64_t n, float* loss,
                               float* grad) {
  return mlp_guarded(c, [&] {
    CPHF_CHECK_ARG(feat && target && n > 0, "invalid arguments");
    DevBuf f, t;
    f.ensure((size_t)n * 12, c->counter());
    t.ensure((size_t)n * 8, c->counter());
    CPHF_CUDA(cudaMemcpyAsync(f.p, feat, n * 12, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaMemcpyAsync(t.p, target, n * 8, cudaMemcpyDefault, c->stream));
    mlp_require(c);
    const float l = mlp_loss_grad(c, f.as<float>(), t.as<float>(), nullptr, n, c->mlp->g.as<float>());
    if (loss) *loss = l;
    if (grad) CPHF_CUDA(cudaMemcpyAsync(grad, c->mlp->g.p, NW * 4, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

cphf_status cphf_mlp_train(cphf_ctx* c, const float* feat, const float* target, int64_t n, int64_t epochs,
                           int64_t batch, float lr, uint64_t seed, float* history) {
  return mlp_guarded(c, [&] {
    CPHF_CHECK_ARG(feat && target && n > 0 && epochs >= 0 && batch > 0, "invalid arguments");
    DevBuf f, t;
    f.ensure((size_t)n * 12, c->counter());
    t.ensure((size_t)n * 8, c->counter());
    CPHF_CUDA(cudaMemcpyAsync(f.p, feat, n * 12, cudaMemcpyDefault, c->stream));
    CPHF_CUDA(cudaMemcpyAsync(t.p, target, n * 8, cudaMemcpyDefault, c->stream));
    mlp_train(c, f.as<float>(), t.as<float>(), n, epochs, batch, lr, seed, history);
  });
}

}  // extern "C"
