// FP64-accurate RI-K term 1 on the tensor cores (sm_103a): exact-slice BF16 products
// accumulated in TMEM (an Ozaki-type splitting), for the FP64 residual of the mixed solve.
//
//   out[mu, n] += alpha * sum_P sum_nu B_P[mu, nu] T_P[nu, n],   T_P[nu, (i,a)] = sum_j bra[nu,j,a] O_P[j,i]
//
// (term 1 of the exchange response, src/ri_jk/hess_r.rs:168-170).
//
// Slicing.  Each row mu of B (over all nu, P) and each column n of T (over nu and the P of a
// chunk) is scaled by a power of two so that |v| < 1, then cut into S = 6 slices of 6 bits,
//   v = sum_t q_t 2^(-6(t+1)) + r,   q_0 in [-64, 64], q_t in [-32, 32] (t > 0), |r| <= 2^-37,
// with q_t = rint(2^6 (remainder)); every slice is an integer of at most 7 bits times a
// power of two and is exact in BF16.  The product v_A v_B is approximated by the 21 slice
// products with t + u <= 5 (dropped terms and remainders ~2^-34 relative).
//
// Exact accumulation.  A slice product q_t q_u 2^(-6(t+u+2)) is a multiple of 2^(-6(g+2)),
// g = t + u.  Groups g = 0, 1, 2 each get their own TMEM accumulator; over the K range of
// one CTA (at most KMAX = 3072 terms) their integer sums stay below 2^24 (g0: 64*64*K,
// g1: 2*64*32*K, g2: (2*64*32 + 32*32)*K), so the FP32 accumulation is exact.  Groups 3-5
// share a fourth accumulator whose FP32 rounding is ~2^-24 of a term of size 2^-18.
// The epilogue adds the four accumulators in FP64, applies alpha * 2^(eA_mu + eT_n) and
// atomically adds into the FP64 output (split over K ranges across CTAs).
//
// Kernel structure (one CTA per SM, 4 warps, 194 KB shared memory):
//   warp 0 lane 0  -- TMA producer: 3-D tiled loads of the 6 + 6 slice tiles (K = nu, 32
//                     wide, 64B swizzle) into a 2-stage ring;
//   warp 1 lane 0  -- MMA issuer: 21 x tcgen05.mma.kind::f16 (BF16, M=128, N=128, K=16)
//                     per K step into 4 accumulators (4 x 128 TMEM columns);
//   warp 2         -- TMEM allocation (512 columns) and release;
//   warps 0-3      -- epilogue.
// Every mbarrier wait is bounded; on expiry the kernel raises the error flag and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "kernels.cuh"
#include "tc_ozaki.cuh"
#include "tc_ptx.cuh"

namespace cphf {
namespace {
using namespace tcx;

constexpr int S = 6;          // slices per operand
constexpr int BM = 128, BN = 128, BK = 32;
constexpr int STAGES = 2;
constexpr int TILE = BM * BK * 2;                  // one BF16 slice tile, 8 KB (BN == BM)
constexpr int STAGE_BYTES = 2 * S * TILE;          // 96 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*barriers*/ + 1024 /*alignment*/;
constexpr int TMEM_COLS = 512;                     // 4 accumulators x BN columns
constexpr int KMAX = 3072;                         // exactness bound of the CTA's K range
constexpr int KB_PER_CTA = KMAX / BK;              // 96

static_assert(BN == BM, "one tile size for both operands");
static_assert(4 * BN <= TMEM_COLS, "four accumulators");

struct OzArgs {
  double* out;
  int64_t ld_out;          // out[mu + ld_out * n]
  int M, N;
  int nkb;                 // K blocks of 32 per aux function
  int total_kb;            // np * nkb
  int pA0;                 // global aux index of the chunk's first function
  int depthA, depthB;      // aux functions per slice plane of A (naux) and B (np)
  int m_tiles;
  const double* rowscale;  // [M] 2^eA
  const double* colscale;  // [N] alpha * 2^eT
  int* err;
};

__global__ void __launch_bounds__(128, 1)
    tc_ozaki_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, OzArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 8);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), accum = smem_u32(bars + 2 * STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_tile = blockIdx.x % args.m_tiles, n_tile = blockIdx.x / args.m_tiles;
  const int m0 = m_tile * BM, n0 = n_tile * BN;
  const int kb0 = blockIdx.y * KB_PER_CTA;
  const int total = min(args.total_kb - kb0, KB_PER_CTA);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) tmem_alloc(smem_u32(tmem_slot), TMEM_COLS);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (total > 0) {
    if (warp == 0 && lane == 0) {
      // producer
      int issued = 0;
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(empty0 + 8 * s, ph ^ 1, args.err)) break;
        issued = it + 1;
        const uint32_t full = full0 + 8 * s;
        mbar_expect_tx(full, STAGE_BYTES);
        const int kb = kb0 + it;
        const int P = kb / args.nkb;
        const int k0 = (kb % args.nkb) * BK;
        const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int t = 0; t < S; ++t) {
          tma_load_3d(st + t * TILE, &mA, full, k0, m0, t * args.depthA + args.pA0 + P);
          tma_load_3d(st + (S + t) * TILE, &mB, full, k0, n0, t * args.depthB + P);
        }
      }
      for (int it = max(0, issued - STAGES); it < issued; ++it) {
        mbar_wait(full0 + 8 * (it % STAGES), (it / STAGES) & 1, nullptr);
      }
    } else if (warp == 1 && lane == 0) {
      // MMA issuer
      constexpr uint32_t idesc = instr_desc_f16(BM, BN, true);
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(full0 + 8 * s, ph, args.err)) break;
        fence_after_sync();
        const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          const uint64_t dk = (uint64_t)((k * 32) >> 4);  // 16 BF16 = 32 B along K inside the swizzle row
#pragma unroll
          for (int g = 0; g < S; ++g) {
#pragma unroll
            for (int t = 0; t <= g; ++t) {
              const int u = g - t;
              const int acc = g < 3 ? g : 3;
              const bool first = it == 0 && k == 0 && t == 0 && g <= 3;
              mma_f16(tmem + (uint32_t)(acc * BN), smem_desc<64>(st + t * TILE) + dk,
                      smem_desc<64>(st + (S + u) * TILE) + dk, idesc, first ? 0u : 1u);
            }
          }
        }
        mma_commit(empty0 + 8 * s);
      }
      mma_commit(accum);  // arrives when every issued MMA has retired (also after an early exit)
    }
    __syncwarp();
    const bool have = mbar_wait(accum, 0, args.err);
    fence_after_sync();
    if (have && *(volatile int*)args.err == 0) {
      const int row = m0 + warp * 32 + lane;
      const double rs = row < args.M ? args.rowscale[row] : 0.0;
      const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
      for (int c = 0; c < BN / 32; ++c) {
        float v0[32], v1[32], v2[32], v3[32];
        tmem_ld32(lane_base + (uint32_t)(0 * BN + c * 32), v0);
        tmem_ld32(lane_base + (uint32_t)(1 * BN + c * 32), v1);
        tmem_ld32(lane_base + (uint32_t)(2 * BN + c * 32), v2);
        tmem_ld32(lane_base + (uint32_t)(3 * BN + c * 32), v3);
        if (row < args.M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c * 32 + j;
            if (n < args.N) {
              const double v = ((double)v0[j] + (double)v1[j]) + ((double)v2[j] + (double)v3[j]);
              atomicAdd(args.out + row + args.ld_out * (int64_t)n, v * rs * args.colscale[n]);
            }
          }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 2) tmem_dealloc(tmem, TMEM_COLS);
}

// ---- slicing (integer arithmetic on the FP64 bit pattern; the FP64 pipe is not used) ------
// |x| as an ordered integer key (non-negative doubles order like their bit patterns)
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// F = round(x 2^(36 - e)) for |x| < 2^e, so |F| <= 2^36; then the six digits
// q_0 = round(F / 2^30), q_t = round(R_t / 2^(30 - 6t)) of the running remainder, written
// as BF16 slices q_t 2^(-6(t+1)) (plane stride `plane`).
__device__ __forceinline__ void slice6(double x, int e, __nv_bfloat16* dst, int64_t plane) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((bits >> 52) & 0x7FF);
  const long long mant = (long long)(bits & 0xFFFFFFFFFFFFFull);
  long long F = 0;
  if (E != 0x7FF) {
    const long long M = E ? (mant | (1ll << 52)) : mant;
    const int sh = 1039 + e - (E ? E : 1);  // x = M 2^(E - 1075), F = M 2^-sh (sh >= 17 for |x| < 2^e)
    if (sh <= 0) {
      F = 1ll << 40;                        // |x| >= 2^e cannot happen for a finite max; flag by overflow
    } else if (sh < 63) {
      F = (M + (1ll << (sh - 1))) >> sh;
    }
    if (bits >> 63) F = -F;
  }
  long long R = F;
#pragma unroll
  for (int t = 0; t < S; ++t) {
    const int s = 30 - 6 * t;
    const long long q = s > 0 ? ((R + (1ll << (s - 1))) >> s) : R;
    R -= q << s;
    float v = (float)(int)q * __int_as_float((127 - 6 * (t + 1)) << 23);  // q 2^(-6(t+1)), exact
    if (E == 0x7FF) v = __int_as_float(0x7FC00000);                        // NaN / Inf propagate as NaN
    dst[t * plane] = __float2bfloat16_rn(v);
  }
}

// power of two strictly above max |x| (exponent e with max = f 2^e, f in [0.5, 1)); 0 for zero
__device__ __forceinline__ int pow2_exp(double m) {
  if (!(m > 0.0) || !isfinite(m)) return 0;
  int e;
  frexp(m, &e);
  return e;
}

// max |B_P[mu, nu]| over (nu, P) per row mu; Bd [P][nu][mu] (mu fastest)
__global__ void rowmax_cderi_kernel(const double* __restrict__ Bd, int64_t nao, int64_t nrows_total,
                                    unsigned long long* __restrict__ mx) {
  const int64_t mu = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (mu >= nao) return;
  unsigned long long m = 0;
  for (int64_t r = blockIdx.y; r < nrows_total; r += gridDim.y) m = max(m, abs_key(Bd[mu + nao * r]));
  atomicMax(mx + mu, m);
}

__global__ void exp_scale_kernel(const unsigned long long* __restrict__ mx, int64_t n, double mult,
                                 int* __restrict__ e_out, double* __restrict__ scale) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int e = pow2_exp(__longlong_as_double((long long)mx[i]));
  e_out[i] = e;
  scale[i] = mult * ldexp(1.0, e);
}

// A slices [t][P][mu][ldk] of v = B_P[mu, nu] 2^-e_mu (B_P symmetric: read Bd[nu + nao mu + nao^2 P])
__global__ void slice_cderi_kernel(const double* __restrict__ Bd, int64_t nao, int64_t naux, int64_t ldk,
                                   const int* __restrict__ e_row, __nv_bfloat16* __restrict__ out) {
  const int64_t total = naux * nao * nao;
  const int64_t plane = naux * nao * ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t nu = t % nao;
    const int64_t r = t / nao;  // P * nao + mu
    const int64_t mu = r % nao;
    slice6(Bd[t], e_row[mu], out + nu + ldk * r, plane);
  }
}

// max |T[Pl][n][nu]| over (Pl, nu < nao) per column n: one warp per row (Pl, n)
__global__ void colmax_t_kernel(const double* __restrict__ T, int64_t rows, int64_t N, int64_t ldk, int64_t nao,
                                unsigned long long* __restrict__ mx) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < rows; r += nw) {
    unsigned long long m = 0;
    for (int64_t k = lane; k < nao; k += 32) m = max(m, abs_key(T[r * ldk + k]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) atomicMax(mx + (r % N), m);
  }
}

// B slices [u][Pl][n][ldk] of v = T[Pl][n][nu] 2^-e_n
__global__ void slice_t_kernel(const double* __restrict__ T, int64_t rows, int64_t N, int64_t ldk, int64_t nao,
                               const int* __restrict__ e_col, __nv_bfloat16* __restrict__ out) {
  const int64_t total = rows * nao;
  const int64_t plane = rows * ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t % nao;
    const int64_t r = t / nao;
    slice6(T[r * ldk + k], e_col[r % N], out + r * ldk + k, plane);
  }
}

unsigned grid_for(int64_t total) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(total, 256), 1 << 20)); }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// 3-D BF16 tensor map: dims {K, rows, depth}, row stride ldk elements, box {32, 128, 1}, 64B swizzle.
CUtensorMap make_map(const void* base, int64_t K, int64_t rows, int64_t depth, int64_t ldk) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  auto fn = encode_fn();
  if (!fn) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)(ldk * 2), (cuuint64_t)(ldk * 2 * rows)};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)BM, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

}  // namespace

bool oz_available(cphf_ctx* c) {
  int major = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c->device);
  if (major != 10 || encode_fn() == nullptr) return false;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(tc_ozaki_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
        cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    attr_set = true;
  }
  return true;
}

void oz_prepare_cderi(cphf_ctx* c, OzState& z) {
  const int64_t nao = c->nao, naux = c->naux;
  z.ldk = (nao + 7) / 8 * 8;
  z.A.ensure((size_t)S * naux * nao * z.ldk * 2, c->counter());
  z.rowscale.ensure((size_t)nao * 8, c->counter());
  z.e_row.ensure((size_t)nao * 4, c->counter());
  z.mx.ensure((size_t)std::max<int64_t>(nao, 1) * 8, c->counter());
  CPHF_CUDA(cudaMemsetAsync(z.mx.p, 0, (size_t)nao * 8, c->stream));
  const unsigned gx = (unsigned)div_up(nao, 256);
  const unsigned gy = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nao * naux, 8 * (int64_t)c->num_sms / gx + 1));
  rowmax_cderi_kernel<<<dim3(gx, gy), 256, 0, c->stream>>>(c->Bd.as<double>(), nao, nao * naux,
                                                            z.mx.as<unsigned long long>());
  exp_scale_kernel<<<grid_for(nao), 256, 0, c->stream>>>(z.mx.as<unsigned long long>(), nao, 1.0, z.e_row.as<int>(),
                                                         z.rowscale.as<double>());
  slice_cderi_kernel<<<grid_for(naux * nao * nao), 256, 0, c->stream>>>(c->Bd.as<double>(), nao, naux, z.ldk,
                                                                        z.e_row.as<int>(), z.A.as<__nv_bfloat16>());
  count_launch(3);
  CPHF_CUDA(cudaGetLastError());
  z.ready = true;
}

void oz_k_term1(cphf_ctx* c, OzState& z, const double* bra, const double* O64, int64_t no, int64_t nb,
                double alpha, double* out) {
  if (!z.ready) oz_prepare_cderi(c, z);
  const int64_t nao = c->nao, naux = c->naux, ldk = z.ldk;
  const int64_t N = no * nb;
  if (N <= 0 || nao <= 0) return;
  // chunk of aux functions: FP64 T staging (8 B) + 6 BF16 slices (12 B) per element within ~3 GiB
  int64_t np = std::max<int64_t>(1, (int64_t(3) << 30) / std::max<int64_t>(20 * N * ldk, 1));
  if (c->cfg.aux_chunk > 0) np = c->cfg.aux_chunk;
  np = std::min<int64_t>(np, naux);
  z.T.ensure((size_t)np * N * ldk * 8, c->counter());
  z.B.ensure((size_t)S * np * N * ldk * 2, c->counter());
  z.colscale.ensure((size_t)N * 8, c->counter());
  z.e_col.ensure((size_t)N * 4, c->counter());
  z.mxc.ensure((size_t)N * 8, c->counter());
  z.err.ensure(sizeof(int), c->counter());
  CPHF_CUDA(cudaMemsetAsync(z.err.p, 0, sizeof(int), c->stream));
  const int m_tiles = (int)div_up(nao, BM), n_tiles = (int)div_up(N, BN);
  const int nkb = (int)div_up(nao, BK);
  const CUtensorMap mA = make_map(z.A.p, nao, nao, S * naux, ldk);
  for (int64_t P0 = 0; P0 < naux; P0 += np) {
    const int64_t npc = std::min<int64_t>(np, naux - P0);
    // T[Pl][(i,a)][nu] = sum_j bra[nu, j, a] O_P[j, i] in FP64 (rows (nu, a) two-level, columns i)
    GemmDesc t;
    t.M = nao * nb; t.N = no; t.K = no; t.batch1 = npc;
    t.A = bra; t.a_m = 1; t.m_div = nao; t.a_m2 = nao * no; t.a_k = nao; t.a_b1 = 0;
    t.B = O64 + P0 * no * no; t.b_k = 1; t.b_n = no; t.b_b1 = no * no;
    t.C = z.T.p; t.c_m = 1; t.c_m2 = ldk * no; t.c_n = ldk; t.c_b1 = N * ldk;
    gemm64(c, t);
    CPHF_CUDA(cudaMemsetAsync(z.mxc.p, 0, (size_t)N * 8, c->stream));
    const int64_t rows = npc * N;
    colmax_t_kernel<<<(unsigned)std::min<int64_t>(div_up(rows * 32, 256), 16 * (int64_t)c->num_sms), 256, 0,
                      c->stream>>>(z.T.as<double>(), rows, N, ldk, nao, z.mxc.as<unsigned long long>());
    exp_scale_kernel<<<grid_for(N), 256, 0, c->stream>>>(z.mxc.as<unsigned long long>(), N, alpha,
                                                         z.e_col.as<int>(), z.colscale.as<double>());
    slice_t_kernel<<<grid_for(rows * nao), 256, 0, c->stream>>>(z.T.as<double>(), rows, N, ldk, nao,
                                                                z.e_col.as<int>(), z.B.as<__nv_bfloat16>());
    count_launch(3);
    const CUtensorMap mB = make_map(z.B.p, nao, N, S * npc, ldk);
    OzArgs a;
    a.out = out;
    a.ld_out = nao;
    a.M = (int)nao;
    a.N = (int)N;
    a.nkb = nkb;
    a.total_kb = (int)(npc * nkb);
    a.pA0 = (int)P0;
    a.depthA = (int)naux;
    a.depthB = (int)npc;
    a.m_tiles = m_tiles;
    a.rowscale = z.rowscale.as<double>();
    a.colscale = z.colscale.as<double>();
    a.err = z.err.as<int>();
    dim3 grid((unsigned)(m_tiles * n_tiles), (unsigned)div_up(npc * nkb, KB_PER_CTA));
    // algorithmic FLOPs of the FP64 contraction (the tensor pipe executes 21 slice products)
    ProfScope ps(c, PROF_TC_OZAKI, 2.0 * nao * N * nao * npc, 2.0 * S * nao * npc * (nao + N));
    tc_ozaki_kernel<<<grid, 128, SMEM_BYTES, c->stream>>>(mA, mB, a);
    count_launch();
    CPHF_CUDA(cudaGetLastError());
  }
  int flag = 0;
  CPHF_CUDA(cudaMemcpyAsync(&flag, z.err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  if (flag) throw Error(CPHF_ERR_TIMEOUT, "tensor-core FP64 K-term kernel: a bounded pipeline wait expired");
}

}  // namespace cphf
