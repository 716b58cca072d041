// Generic strided/batched SIMT GEMM, see gemm_simt.cuh.
#include "gemm_simt.cuh"
#include "common.cuh"
#include "dfloat.cuh"

#include <algorithm>

namespace cphf {

namespace {

// FP64: 64x64 tile, 4x4 per thread, 256 threads.  FP64-pipe bound on GB300.
struct CfgF64 {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};
// FP32: 128x128 tile, 8x8 per thread, 256 threads.
struct CfgF32 {
  static constexpr int BM = 128, BN = 128, BK = 16, TM = 8, TN = 8;
};
// FP32 for narrow outputs (N <= 64, e.g. the occupied index of the K-term intermediates):
// 256x64 tile, 8x8 per thread, 256 threads.
struct CfgF32Tall {
  static constexpr int BM = 256, BN = 64, BK = 16, TM = 8, TN = 8;
};

// offset of row m (or column n) with optional two-level index m = m0 + div * m1
__device__ __forceinline__ int64_t off2(int64_t m, int64_t div, int64_t s1, int64_t s2) {
  if (div <= 0) return m * s1;
  const int64_t q = m / div;
  return (m - q * div) * s1 + q * s2;
}

template <typename T, typename Cfg, typename TA, typename TB, typename TC>
__global__ void __launch_bounds__(256) gemm_kernel(GemmDesc d, int ksplit, int64_t kchunk, T* ws) {
  constexpr int BM = Cfg::BM, BN = Cfg::BN, BK = Cfg::BK, TM = Cfg::TM, TN = Cfg::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  constexpr int LA = BM * BK / NT, LB = BK * BN / NT;
  __shared__ T As[2][BK][BM];
  __shared__ T Bs[2][BK][BN];

  const int tid = threadIdx.x;
  const int tx = tid % NTX, ty = tid / NTX;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  const int64_t z = blockIdx.z;
  const int split = (int)(z % ksplit);
  const int64_t bidx = z / ksplit;
  const int64_t b1 = bidx % d.batch1, b2 = bidx / d.batch1;

  const TA* __restrict__ A = static_cast<const TA*>(d.A) + b1 * d.a_b1 + b2 * d.a_b2;
  const TB* __restrict__ B = static_cast<const TB*>(d.B) + b1 * d.b_b1 + b2 * d.b_b2;
  TC* __restrict__ C = static_cast<TC*>(d.C) + b1 * d.c_b1 + b2 * d.c_b2;

  const int64_t kbeg = (int64_t)split * kchunk;
  const int64_t kend = min(d.K, kbeg + kchunk);
  // load mapping: consecutive threads along the unit-stride index (offsets are precomputed, so
  // a two-level index still coalesces inside each contiguous block)
  const bool a_mfast = (d.a_m == 1);
  const bool b_nfast = (d.b_n == 1);

  // per-thread fixed row / column of each load, and its offset
  int a_mm[LA], a_kk[LA], b_nn[LB], b_kk[LB];
  int64_t a_off[LA], b_off[LB];
  bool a_ok[LA], b_ok[LB];
#pragma unroll
  for (int i = 0; i < LA; ++i) {
    const int e = tid + i * NT;
    if (a_mfast) { a_mm[i] = e % BM; a_kk[i] = e / BM; } else { a_kk[i] = e % BK; a_mm[i] = e / BK; }
    const int64_t gm = m0 + a_mm[i];
    a_ok[i] = gm < d.M;
    a_off[i] = a_ok[i] ? off2(gm, d.m_div, d.a_m, d.a_m2) : 0;
  }
#pragma unroll
  for (int i = 0; i < LB; ++i) {
    const int e = tid + i * NT;
    if (b_nfast) { b_nn[i] = e % BN; b_kk[i] = e / BN; } else { b_kk[i] = e % BK; b_nn[i] = e / BK; }
    const int64_t gn = n0 + b_nn[i];
    b_ok[i] = gn < d.N;
    b_off[i] = b_ok[i] ? off2(gn, d.n_div, d.b_n, d.b_n2) : 0;
  }

  T ra[LA], rb[LB];
  auto load_tiles = [&](int64_t k0) {
#pragma unroll
    for (int i = 0; i < LA; ++i) {
      const int64_t gk = k0 + a_kk[i];
      ra[i] = (a_ok[i] && gk < kend) ? (T)A[a_off[i] + gk * d.a_k] : (T)0;
    }
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      const int64_t gk = k0 + b_kk[i];
      rb[i] = (b_ok[i] && gk < kend) ? (T)B[b_off[i] + gk * d.b_k] : (T)0;
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int i = 0; i < LA; ++i) As[buf][a_kk[i]][a_mm[i]] = ra[i];
#pragma unroll
    for (int i = 0; i < LB; ++i) Bs[buf][b_kk[i]][b_nn[i]] = rb[i];
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = (T)0;

  int buf = 0;
  if (kbeg < kend) {
    load_tiles(kbeg);
    store_tiles(0);
    __syncthreads();
    for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
      const bool has_next = (k0 + BK < kend);
      if (has_next) load_tiles(k0 + BK);
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][ty + i * NTY];
#pragma unroll
        for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][tx + j * NTX];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = madd(a[i], b[j], acc[i][j]);
      }
      if (has_next) {
        store_tiles(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }
  }

  if (ksplit == 1) {
    const T alpha = (T)d.alpha, beta = (T)d.beta;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t gm = m0 + ty + i * NTY;
      if (gm >= d.M) continue;
      const int64_t cm = off2(gm, d.m_div, d.c_m, d.c_m2);
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int64_t gn = n0 + tx + j * NTX;
        if (gn >= d.N) continue;
        TC* p = C + cm + off2(gn, d.n_div, d.c_n, d.c_n2);
        T v = alpha * acc[i][j];
        if (beta != (T)0) v = madd(beta, (T)(*p), v);
        *p = (TC)v;
      }
    }
  } else {
    // split-K partial sums, [split][batch][M][N] row-major in the workspace
    T* W = ws + ((int64_t)split * (d.batch1 * d.batch2) + bidx) * d.M * d.N;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t gm = m0 + ty + i * NTY;
      if (gm >= d.M) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int64_t gn = n0 + tx + j * NTX;
        if (gn < d.N) W[gm * d.N + gn] = acc[i][j];
      }
    }
  }
}

// Fixed-order reduction of the split-K partials: C = alpha * sum_s W[s] + beta * C.
template <typename T, typename TC>
__global__ void splitk_reduce_kernel(GemmDesc d, int ksplit, const T* __restrict__ ws) {
  const int64_t nb = d.batch1 * d.batch2;
  const int64_t total = nb * d.M * d.N;
  const T alpha = (T)d.alpha, beta = (T)d.beta;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = e % d.N;
    const int64_t m = (e / d.N) % d.M;
    const int64_t bidx = e / (d.N * d.M);
    const int64_t b1 = bidx % d.batch1, b2 = bidx / d.batch1;
    T s = (T)0;
    for (int k = 0; k < ksplit; ++k) s += ws[(int64_t)k * total + e];
    TC* p = static_cast<TC*>(d.C) + b1 * d.c_b1 + b2 * d.c_b2 + off2(m, d.m_div, d.c_m, d.c_m2) +
            off2(n, d.n_div, d.c_n, d.c_n2);
    T v = alpha * s;
    if (beta != (T)0) v = madd(beta, (T)(*p), v);
    *p = (TC)v;
  }
}

template <typename Cfg>
int choose_split(const GemmDesc& d, int num_sms) {
  const int64_t tiles = ((d.M + Cfg::BM - 1) / Cfg::BM) * ((d.N + Cfg::BN - 1) / Cfg::BN) *
                        d.batch1 * d.batch2;
  if (tiles >= 2 * (int64_t)num_sms) return 1;
  int64_t want = (2 * (int64_t)num_sms + tiles - 1) / tiles;
  const int64_t kmax = d.K / (4 * Cfg::BK);
  want = std::min<int64_t>(want, std::max<int64_t>(kmax, 1));
  want = std::min<int64_t>(want, 32);
  return (int)std::max<int64_t>(want, 1);
}

template <typename T, typename Cfg, typename TA, typename TB, typename TC>
cudaError_t run(const GemmDesc& d, cudaStream_t stream, void* workspace, size_t ws_bytes, int num_sms) {
  const int64_t nb = d.batch1 * d.batch2;
  int ksplit = choose_split<Cfg>(d, num_sms);
  if (ksplit > 1) {
    const size_t need = (size_t)ksplit * nb * d.M * d.N * sizeof(T);
    if (workspace == nullptr || need > ws_bytes) ksplit = 1;
  }
  int64_t kchunk = (d.K + ksplit - 1) / ksplit;
  kchunk = ((kchunk + Cfg::BK - 1) / Cfg::BK) * Cfg::BK;
  ksplit = (int)((d.K + kchunk - 1) / kchunk);
  const int64_t gx = (d.M + Cfg::BM - 1) / Cfg::BM;
  const int64_t gy = (d.N + Cfg::BN - 1) / Cfg::BN;
  if (gy > 65535) return cudaErrorInvalidConfiguration;
  // batches beyond the grid z limit are issued in several launches
  const int64_t zmax = 65535 / ksplit;
  for (int64_t b0 = 0; b0 < nb; b0 += zmax) {
    const int64_t bn = std::min<int64_t>(zmax, nb - b0);
    GemmDesc s = d;
    if (b0 != 0 || bn != nb) {
      if (d.batch2 != 1) return cudaErrorInvalidConfiguration;
      s.A = static_cast<const char*>(d.A) + b0 * d.a_b1 * (int64_t)sizeof(TA);
      s.B = static_cast<const char*>(d.B) + b0 * d.b_b1 * (int64_t)sizeof(TB);
      s.C = static_cast<char*>(d.C) + b0 * d.c_b1 * (int64_t)sizeof(TC);
      s.batch1 = bn;
    }
    dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)(bn * ksplit));
    gemm_kernel<T, Cfg, TA, TB, TC><<<grid, 256, 0, stream>>>(s, ksplit, kchunk, static_cast<T*>(workspace));
    count_launch();
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    if (ksplit > 1) {
      const int64_t total = bn * d.M * d.N;
      const int64_t blocks = std::min<int64_t>((total + 255) / 256, 8 * (int64_t)num_sms);
      splitk_reduce_kernel<T, TC><<<(unsigned)blocks, 256, 0, stream>>>(s, ksplit, static_cast<const T*>(workspace));
      count_launch();
      err = cudaGetLastError();
      if (err != cudaSuccess) return err;
    }
  }
  return cudaSuccess;
}

// narrow-output FP32 shapes take the 256 x 64 tile
bool use_tall(const GemmDesc& d) { return d.N <= 64 && d.M >= 512; }

}  // namespace

size_t gemm_workspace_bytes(const GemmDesc& d, size_t elem_bytes, int num_sms) {
  int s;
  if (elem_bytes == 8) s = choose_split<CfgF64>(d, num_sms);
  else s = use_tall(d) ? choose_split<CfgF32Tall>(d, num_sms) : choose_split<CfgF32>(d, num_sms);
  if (s <= 1) return 0;
  return (size_t)s * d.batch1 * d.batch2 * d.M * d.N * elem_bytes;
}

template <typename T, typename TA, typename TB, typename TC>
cudaError_t gemm(const GemmDesc& d, cudaStream_t stream, void* workspace, size_t ws_bytes, int num_sms) {
  if (d.M <= 0 || d.N <= 0) return cudaSuccess;
  const int64_t nb = d.batch1 * d.batch2;
  if (d.K <= 0) {
    // C = beta * C (alpha term is empty)
    GemmDesc z = d;
    z.K = 0;
    splitk_reduce_kernel<T, TC><<<std::max<int64_t>(1, std::min<int64_t>(4096, (nb * d.M * d.N + 255) / 256)), 256, 0, stream>>>(z, 0, (const T*)nullptr);
    count_launch();
    return cudaGetLastError();
  }
  if constexpr (sizeof(T) == 8) {
    return run<T, CfgF64, TA, TB, TC>(d, stream, workspace, ws_bytes, num_sms);
  } else {
    if (use_tall(d)) return run<T, CfgF32Tall, TA, TB, TC>(d, stream, workspace, ws_bytes, num_sms);
    return run<T, CfgF32, TA, TB, TC>(d, stream, workspace, ws_bytes, num_sms);
  }
}

#define CPHF_INST(T, TA, TB, TC) \
  template cudaError_t gemm<T, TA, TB, TC>(const GemmDesc&, cudaStream_t, void*, size_t, int);
CPHF_INST(double, double, double, double)
CPHF_INST(float, float, float, float)
CPHF_INST(float, float, float, double)
CPHF_INST(float, float, double, float)
CPHF_INST(float, double, float, float)
CPHF_INST(float, float, double, double)
CPHF_INST(float, double, double, float)
CPHF_INST(float, double, float, double)
CPHF_INST(float, double, double, double)
#undef CPHF_INST

cudaError_t gemm_f64_emulated(const GemmDesc& d, cudaStream_t stream, void* workspace, size_t ws_bytes,
                              int num_sms) {
  return gemm<dfloat, double, double, double>(d, stream, workspace, ws_bytes, num_sms);
}

}  // namespace cphf
