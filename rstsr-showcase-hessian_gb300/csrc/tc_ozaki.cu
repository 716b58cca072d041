// FP64-accurate RI-K term on the tensor cores (sm_103a): exact-slice BF16 products
// accumulated in TMEM (an Ozaki-type splitting), for the FP64 residual of the mixed solve.
//
// The exchange response K_s = -sum_P [B_P bra O_P + Z_P (Z_P^T bra)^T] (src/ri_jk/hess_r.rs:
// 159-176) is evaluated per chunk of aux functions as four contractions, all on tcgen05:
//   T-gen   T_P[nu, (i,a)] = sum_j bra[nu, j, a] O_P[j, i]        batched over P, K = j
//   term 1  out[mu, n]   += alpha sum_{P,nu} B_P[mu, nu] T_P[nu, n]  K = (P, nu), split over CTAs
//   W-gen   W_P[j, (i,a)] = sum_nu bra[nu, j, a] Z_P[nu, i]       batched over P, K = nu
//   term 2  out[mu, n]   += alpha sum_{P,j} Z_P[mu, j] W_P[j, n]   K = (P, j), split over CTAs
// with A[m, k] B[n, k] operands stored K-major.
//
// Slicing.  Each operand row (over its K range) is scaled by a power of two 2^-e so that
// |v| < 1, rounded to the 36-bit fixed-point integer F = round(v 2^36) and cut into six
// balanced base-64 digits, F = sum_t q_t 2^(30 - 6t), q_0 in [-64, 64], q_t in [-32, 32];
// slice t = q_t 2^(-6(t+1)) is exact in BF16.  The product is approximated by the 21 slice
// products with t + u <= 5 (dropped terms and rounding ~2^-34 relative to |row max| x
// |column max|).  All slicing is integer arithmetic on the FP64 / FP32 bit patterns.
//
// Exact accumulation.  A slice product q_t q_u 2^(-6(t+u+2)) is a multiple of 2^(-6(g+2)),
// g = t + u.  Groups g = 0, 1, 2 each get their own TMEM accumulator; over the K range of
// one CTA (at most KMAX = 3072 terms) their integer sums stay below 2^24 (g0: 64*64*K,
// g1: 2*64*32*K, g2: (2*64*32 + 32*32)*K), so the FP32 accumulation is exact.  Groups 3-5
// share a fourth accumulator whose FP32 rounding is ~2^-24 of a term of size 2^-18.  The
// epilogue adds the four accumulators as an FP32 pair (two-sum), then either atomically
// adds alpha 2^(eA + eB) (hi + lo) into the FP64 output (terms 1 and 2, split over K ranges
// across CTAs) or stores the pair 2^(eA + eB) (hi, lo) into a staging array (T, W).
//
// Kernel structure (one CTA per SM, 4 warps):
//   warp 0 lane 0  -- TMA producer: 3-D tiled loads of the 6 + 6 slice tiles (K = 32 wide,
//                     64B swizzle) into a 2-stage ring;
//   warp 1 lane 0  -- MMA issuer: 21 x tcgen05.mma.kind::f16 (BF16, M=128, N=BN, K=16)
//                     per K step into 4 accumulators (4 x BN TMEM columns);
//   warp 2         -- TMEM allocation and release;
//   warps 0-3      -- epilogue.
// Every mbarrier wait is bounded; on expiry the kernel raises the error flag and returns.
//
// The same kernel template also runs the split-precision operator of the inner solves
// (Split2): two FP16 planes per operand (x 2^(14-e) = hi + lo), three products hi*hi +
// hi*lo + lo*hi into one FP32 accumulator, FP32 outputs; ~1e-7 relative to the row maxima.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "kernels.cuh"
#include "tc_gemm.cuh"
#include "tc_ozaki.cuh"
#include "slices.cuh"
#include "tc_ptx.cuh"

namespace cphf {
namespace {
using namespace tcx;

constexpr int BM = 128, BK = 32;
constexpr int KMAX = 3072;         // exactness bound of the K range of one CTA
constexpr int KB_PER_CTA = KMAX / BK;
constexpr int SHORT_STAGES = 3;    // split-FP16 stages for K ranges of a few blocks (two CTAs per SM)

constexpr int S = Exact6::S;

template <class PR, int BN, int ST = PR::STAGES>
struct Cfg {
  static constexpr int A_TILE = BM * BK * 2;                 // 8 KB
  static constexpr int B_TILE = BN * BK * 2;                 // 8 / 4 KB
  static constexpr int STAGES = ST;
  static constexpr int STAGE_BYTES = PR::S * (A_TILE + B_TILE);
  static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*barriers*/ + 1024 /*alignment*/;
  static_assert(BN == 64 || BN == 128, "tile width");
  static_assert(SMEM_BYTES <= 232448, "shared memory");
};

struct OzArgs {
  void* out;
  int M, N;
  int m_tiles;
  int nkb;                  // K blocks of 32 per aux function
  int total_kb;             // split mode: K blocks of the chunk (np * nkb)
  int a_depth, b_depth;     // plane stride of A / B in depth units (slice t at depth t * stride)
  int a_off, b_off;         // depth offset of the chunk's aux function 0
  int a_per_p;              // A depth advances with the aux function
  int a_row0;               // split mode: first A row of the contraction (A rows need no alignment)
  int b_k0;                 // split mode: K offset of B (elements, a multiple of 16 bytes)
  int store;                // split mode with one K range per tile: store instead of accumulating
  // split-FP16 split mode, rho1 epilogue (when rho is set): instead of out, accumulate
  // rho[m + ld_rho a] += sum_i value[m, n = i + rho_nocc a] ao[m + ld_ao i]
  float* rho;
  const float* rho_ao;
  int64_t ld_rho, ld_ao;
  int rho_nocc;
  int np, p_per_cta;        // batched: aux functions of the launch, per CTA
  int kb_per_cta;           // split: K blocks per CTA (<= KMAX / BK, the exactness bound)
  // batched split-FP16 T generation writing the FP16 hi / lo planes of T * (*tscale) for
  // tc_gemm.cu's term 1
  const float* tscale;
  void* out_lo;             // the lo plane (same layout as out, the hi plane)
  // split mode epilogue: out [m + ld_out n] += value rowscale[m] colscale[n] (double: Exact6, float: Split2)
  const double* rowscale;
  const double* colscale;
  int64_t ld_out;
  // batched mode epilogue: out [(m % m_div) s_m1 + (m / m_div) s_m2 + n s_n + Pl s_p]
  //   = 2^(e_row[m] + e_col[(b_off + Pl) N + n] - 2 EOFF) value (float2 pair: Exact6, float: Split2;
  //   EPI_SPLIT16 takes e_col uniform over an aux function's columns and reads its first)
  const int* e_row;
  const int* e_col;
  int64_t m_div, s_m1, s_m2, s_n, s_p;
  unsigned long long* colmax;  // EPI_STOREMAX: column maxima (float bits of |value|)
  int* err;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) ~ a0 + a1 + a2 + a3 (a0, a1, a2 exact integer sums, a3 rounded)
__device__ __forceinline__ void combine4(float a0, float a1, float a2, float a3, float& hi, float& lo) {
  float s, e, e2;
  two_sum(a0, a1, s, e);
  two_sum(s, a2, s, e2);
  e += e2;
  two_sum(s, a3, s, e2);
  e += e2;
  hi = s + e;
  lo = e - (hi - s);
}

// Split-K contractions (terms 1 and 2): one CTA per (tile, K range of at most KMAX).  ST
// pipeline stages (fewer for short K ranges, so that two CTAs share an SM and one's epilogue
// overlaps the other's MMAs).
template <class PR, int BN, int ST = PR::STAGES>
__global__ void __launch_bounds__(128, 1)
    tc_slice_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, OzArgs args) {
  using C = Cfg<PR, BN, ST>;
  constexpr int STAGES = C::STAGES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * C::STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), accum = smem_u32(bars + 2 * STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // x = tile (M fastest: CTAs that share a B tile run together), y = K range
  const int m_tile = blockIdx.x % args.m_tiles, n_tile = blockIdx.x / args.m_tiles;
  const int m0 = m_tile * BM, n0 = n_tile * BN;
  const int kb0 = blockIdx.y * args.kb_per_cta;
  const int total = min(args.total_kb - kb0, args.kb_per_cta);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  constexpr uint32_t TMEM_COLS = PR::NACC * BN;  // one accumulator per group
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
        mbar_expect_tx(full, C::STAGE_BYTES);
        const int kb = kb0 + it;
        const int P = kb / args.nkb;
        const int k0 = (kb % args.nkb) * BK;
        const int da = args.a_off + (args.a_per_p ? P : 0);
        const int db = args.b_off + P;
        const uint32_t st = smem_u32(smem + s * C::STAGE_BYTES);
#pragma unroll
        for (int t = 0; t < PR::S; ++t) {
          tma_load_3d(st + t * C::A_TILE, &mA, full, k0, m0 + args.a_row0, t * args.a_depth + da);
          tma_load_3d(st + PR::S * C::A_TILE + t * C::B_TILE, &mB, full, k0 + args.b_k0, n0, t * args.b_depth + db);
        }
      }
      for (int it = max(0, issued - STAGES); it < issued; ++it)
        mbar_wait(full0 + 8 * (it % STAGES), (it / STAGES) & 1, nullptr);
    } else if (warp == 1 && lane == 0) {
      // MMA issuer
      constexpr uint32_t idesc = instr_desc_f16(BM, BN, PR::BF16);
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(full0 + 8 * s, ph, args.err)) break;
        fence_after_sync();
        const uint32_t st = smem_u32(smem + s * C::STAGE_BYTES);
        const uint32_t sb = st + PR::S * C::A_TILE;
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          const uint64_t dk = (uint64_t)((k * 32) >> 4);  // 16 elements = 32 B along K inside the swizzle row
          if constexpr (PR::NACC == 4) {
#pragma unroll
            for (int g = 0; g < PR::S; ++g) {
#pragma unroll
              for (int t = 0; t <= g; ++t) {
                const int u = g - t;
                const int acc = g < 3 ? g : 3;
                const bool first = it == 0 && k == 0 && t == 0 && g <= 3;
                mma_f16(tmem + (uint32_t)(acc * BN), smem_desc<64>(st + t * C::A_TILE) + dk,
                        smem_desc<64>(sb + u * C::B_TILE) + dk, idesc, first ? 0u : 1u);
              }
            }
          } else {
            // hi*hi + hi*lo + lo*hi
            mma_f16(tmem, smem_desc<64>(st) + dk, smem_desc<64>(sb) + dk, idesc, (it > 0 || k > 0) ? 1u : 0u);
            mma_f16(tmem, smem_desc<64>(st) + dk, smem_desc<64>(sb + C::B_TILE) + dk, idesc, 1u);
            mma_f16(tmem, smem_desc<64>(st + C::A_TILE) + dk, smem_desc<64>(sb) + dk, idesc, 1u);
          }
        }
        mma_commit(empty0 + 8 * s);
      }
      mma_commit(accum);  // arrives when every issued MMA has retired (also after an early exit)
    }
    __syncwarp();
    // warp-uniform decision: tcgen05.ld is a whole-warp instruction
    const bool have = __all_sync(0xffffffffu, mbar_wait(accum, 0, args.err) && *(volatile int*)args.err == 0);
    fence_after_sync();
    if (have) {
      const int row = m0 + warp * 32 + lane;
      const bool row_ok = row < args.M;
      const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
      const double rs = row_ok ? args.rowscale[row] : 0.0;
      const float rsf = (float)rs;
      // rho1 epilogue state: orbital i and right-hand side a of column n0, partial sum
      int rho_i = 0, rho_a = 0;
      float rho_acc = 0.f;
      const float* rho_ao_row = nullptr;
      if constexpr (PR::NACC == 1) {
        if (args.rho != nullptr) {
          rho_i = n0 % args.rho_nocc;
          rho_a = n0 / args.rho_nocc;
          rho_ao_row = args.rho_ao + (row_ok ? row : 0);
        }
      }
      for (int c = 0; c < BN / 32; ++c) {
        if constexpr (PR::NACC == 4) {
          float v0[32], v1[32], v2[32], v3[32];
          tmem_ld32(lane_base + (uint32_t)(0 * BN + c * 32), v0);
          tmem_ld32(lane_base + (uint32_t)(1 * BN + c * 32), v1);
          tmem_ld32(lane_base + (uint32_t)(2 * BN + c * 32), v2);
          if constexpr (PR::S > 3) {
            tmem_ld32(lane_base + (uint32_t)(3 * BN + c * 32), v3);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v3[j] = 0.f;  // groups 0-2 only: the fourth accumulator is unused
          }
          if (row_ok) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = n0 + c * 32 + j;
              if (n < args.N) {
                float hi, lo;
                combine4(v0[j], v1[j], v2[j], v3[j], hi, lo);
                const double v = ((double)hi + (double)lo) * (rs * args.colscale[n]);
                double* o = reinterpret_cast<double*>(args.out) + row + args.ld_out * (int64_t)n;
                if (args.store) *o = v;
                else atomicAdd(o, v);
              }
            }
          }
        } else {
          float v[32];
          tmem_ld32(lane_base + (uint32_t)(c * 32), v);
          // the chunk's 32 column scales: one load per lane, broadcast by shuffles (no FP64 per
          // element); rowscale and colscale are powers of two (times a small factor), so the
          // FP32 product equals the FP64 one
          float cs[32];
          {
            const int nl = n0 + c * 32 + lane;
            const float csl = nl < args.N ? (float)args.colscale[nl] : 0.f;
#pragma unroll
            for (int j = 0; j < 32; ++j) cs[j] = __shfl_sync(0xffffffffu, csl, j) * rsf;
          }
          if (row_ok && args.rho != nullptr) {
            // rho1 of this row: columns n = i + nocc a, the running i / a carried across chunks.
            // The chunk's 32 ao values are loaded first, back to back (independent L2 loads),
            // then reduced.
            float aov[32];
            {
              int ii = rho_i;
#pragma unroll
              for (int j = 0; j < 32; ++j) {
                aov[j] = n0 + c * 32 + j < args.N ? rho_ao_row[args.ld_ao * (int64_t)ii] : 0.f;
                if (++ii == args.rho_nocc) ii = 0;
              }
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = n0 + c * 32 + j;
              if (n < args.N) {
                rho_acc += v[j] * cs[j] * aov[j];
                if (++rho_i == args.rho_nocc) {
                  atomicAdd(args.rho + row + args.ld_rho * (int64_t)rho_a, rho_acc);
                  rho_acc = 0.f;
                  rho_i = 0;
                  ++rho_a;
                }
              }
            }
          } else if (row_ok) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = n0 + c * 32 + j;
              if (n < args.N) {
                float* o = reinterpret_cast<float*>(args.out) + row + args.ld_out * (int64_t)n;
                const float x = v[j] * cs[j];
                if (args.store) *o = x;
                else atomicAdd(o, x);
              }
            }
          }
        }
      }
      if constexpr (PR::NACC == 1) {
        if (row_ok && args.rho != nullptr && rho_i > 0) atomicAdd(args.rho + row + args.ld_rho * (int64_t)rho_a, rho_acc);
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 2) tmem_dealloc(tmem, TMEM_COLS);
}

// Batched contractions (T-gen, W-gen): one CTA per (tile, range of aux functions), the A tile
// shared by the range.  The accumulators are double-buffered in TMEM, so the epilogue of aux
// function p overlaps the MMAs of p + 1.  Ten warps: 0 TMA producer, 1 MMA issuer and TMEM
// owner, 2-9 epilogue (warp w drains TMEM lanes [32 (w % 4), 32 (w % 4) + 32) and column half
// (w - 2) / 4 of the 64-column tile).
template <class PR>
struct Batched {
  static constexpr int BN = 64;
  // stages of S x 12 KB: as many as the shared memory of the one CTA per SM holds for the exact
  // slices (3 x 72 KB, 4 x 48 KB, 5 x 36 KB); split FP16 (two CTAs per SM): 3 x 24 KB
  static constexpr int STAGES = PR::NACC == 4 ? (PR::S == 6 ? 3 : PR::S == 4 ? 4 : 5) : 3;
  static constexpr int THREADS = 320;
  static constexpr int EPI_WARPS = 8;
  static constexpr int SMEM_BYTES = STAGES * Cfg<PR, BN>::STAGE_BYTES + 1024 + 1024;
};

// 2^e as a float for any int e, exact: normal, subnormal below 2^-126, 0 below 2^-149, inf
// above 2^127 (branch-free integer arithmetic on the bit pattern)
__device__ __forceinline__ float pow2f(int e) {
  const int c = min(max(e, -150), 128);
  const unsigned normal = (unsigned)(c + 127) << 23;                 // c in [-126, 128]
  const unsigned sub = c >= -149 ? 1u << ((c + 149) & 31) : 0u;      // c in [-149, -127]
  return __uint_as_float(c >= -126 ? normal : sub);
}

// FP16 hi / lo planes of v[j] f to ph[j sn], pl[j sn] for j < jn, as streaming (evict-first)
// stores: T is read once, by term 1, after its chunk is complete.  A full chunk (jn = 32, the
// warp-uniform common case) runs without per-element predicates.
__device__ __forceinline__ void store_split32(const float* v, float f, __half* ph, __half* pl, int sn, int jn) {
  if (jn >= 32) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const float x = v[j] * f;
      const __half h = __float2half_rn(x);
      __stcs(ph + j * sn, h);
      __stcs(pl + j * sn, __float2half_rn(x - __half2float(h)));
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      if (j < jn) {
        const float x = v[j] * f;
        const __half h = __float2half_rn(x);
        __stcs(ph + j * sn, h);
        __stcs(pl + j * sn, __float2half_rn(x - __half2float(h)));
      }
    }
  }
}

// exponent of a power-of-two float (normal or inf)
__device__ __forceinline__ int pow2_exponent(float s) { return (int)((__float_as_uint(s) >> 23) & 0xFF) - 127; }

// EPI: store the scaled values (T / W staging) or FP16 hi / lo planes of them times *tscale.
// EPI_STOREMAX (exact slices): store as EPI_STORE and reduce max |value| per staging column
// n_T = n + N (row / m_div) over the CTA's rows and aux functions into colmax (the column
// scales of the next slicing pass, without a pass over the staging array).
enum { EPI_STORE = 0, EPI_STOREMAX = 1, EPI_SPLIT16 = 2 };

template <class PR, int BN, int EPI = EPI_STORE>
__global__ void __launch_bounds__(320, PR::NACC == 4 ? 1 : 2)
    tc_slice_batched_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB,
                            OzArgs args) {
  using C = Cfg<PR, BN>;
  static_assert(BN == Batched<PR>::BN, "batched tile width");
  constexpr int STAGES = Batched<PR>::STAGES;
  constexpr uint32_t ACC = PR::NACC * BN;  // TMEM columns of one accumulator set
  static_assert(2 * ACC <= 512, "two accumulator sets");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * C::STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);
  const uint32_t accf0 = smem_u32(bars + 2 * STAGES), acce0 = smem_u32(bars + 2 * STAGES + 2);
  const uint32_t done = smem_u32(bars + 2 * STAGES + 4);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.y;
  const int m_tile = tile % args.m_tiles, n_tile = tile / args.m_tiles;
  const int m0 = m_tile * BM, n0 = n_tile * BN;
  const int p_begin = blockIdx.x * args.p_per_cta;
  const int nP = min(args.np - p_begin, args.p_per_cta);
  const int nkb = args.nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);  // tcgen05.commit of the MMA issuer
      mbar_init(acce0 + 8 * b, Batched<PR>::EPI_WARPS);  // one arrive per epilogue warp
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tmem_slot), 2 * ACC);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (nP > 0) {
    if (warp == 0 && lane == 0) {
      // producer: K blocks of every aux function of the range, back to back through the ring
      const int total = nP * nkb;
      int issued = 0;
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(empty0 + 8 * s, ph ^ 1, args.err)) break;
        issued = it + 1;
        const uint32_t full = full0 + 8 * s;
        mbar_expect_tx(full, C::STAGE_BYTES);
        const int P = p_begin + it / nkb;
        const int k0 = (it % nkb) * BK;
        const int db = args.b_off + P;
        const uint32_t st = smem_u32(smem + s * C::STAGE_BYTES);
#pragma unroll
        for (int t = 0; t < PR::S; ++t) {
          tma_load_3d(st + t * C::A_TILE, &mA, full, k0, m0, t * args.a_depth + args.a_off);
          tma_load_3d(st + PR::S * C::A_TILE + t * C::B_TILE, &mB, full, k0, n0, t * args.b_depth + db);
        }
      }
      for (int it = max(0, issued - STAGES); it < issued; ++it)
        mbar_wait(full0 + 8 * (it % STAGES), (it / STAGES) & 1, nullptr);
    } else if (warp == 1 && lane == 0) {
      // MMA issuer
      constexpr uint32_t idesc = instr_desc_f16(BM, BN, PR::BF16);
      bool ok = true;
      for (int p = 0; p < nP && ok; ++p) {
        const int b = p & 1;
        if (!mbar_wait(acce0 + 8 * b, ((p >> 1) & 1) ^ 1, args.err)) break;
        fence_after_sync();
        const uint32_t acc_base = tmem + (uint32_t)b * ACC;
        for (int kb = 0; kb < nkb; ++kb) {
          const int it = p * nkb + kb;
          const int s = it % STAGES;
          if (!mbar_wait(full0 + 8 * s, (it / STAGES) & 1, args.err)) { ok = false; break; }
          fence_after_sync();
          const uint32_t st = smem_u32(smem + s * C::STAGE_BYTES);
          const uint32_t sb = st + PR::S * C::A_TILE;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint64_t dk = (uint64_t)((k * 32) >> 4);
            if constexpr (PR::NACC == 4) {
#pragma unroll
              for (int g = 0; g < PR::S; ++g) {
#pragma unroll
                for (int t = 0; t <= g; ++t) {
                  const int acc = g < 3 ? g : 3;
                  const bool first = kb == 0 && k == 0 && t == 0 && g <= 3;
                  mma_f16(acc_base + (uint32_t)(acc * BN), smem_desc<64>(st + t * C::A_TILE) + dk,
                          smem_desc<64>(sb + (g - t) * C::B_TILE) + dk, idesc, first ? 0u : 1u);
                }
              }
            } else {
              mma_f16(acc_base, smem_desc<64>(st) + dk, smem_desc<64>(sb) + dk, idesc, (kb > 0 || k > 0) ? 1u : 0u);
              mma_f16(acc_base, smem_desc<64>(st) + dk, smem_desc<64>(sb + C::B_TILE) + dk, idesc, 1u);
              mma_f16(acc_base, smem_desc<64>(st + C::A_TILE) + dk, smem_desc<64>(sb) + dk, idesc, 1u);
            }
          }
          mma_commit(empty0 + 8 * s);
        }
        if (ok) mma_commit(accf0 + 8 * b);  // accumulator set b complete when these MMAs retire
      }
      // every issued MMA has retired before TMEM is released (also after an early exit)
      mma_commit(done);
      mbar_wait(done, 0, nullptr);
    } else if (warp >= 2) {
      // epilogue: TMEM lane quarter q, 32-column chunk c
      const int q = warp & 3;
      const int c = (warp - 2) >> 2;
      const int row = m0 + q * 32 + lane;
      const bool row_ok = row < args.M;
      int erow = 0;
      int64_t base = 0;
      if (row_ok) {
        erow = args.e_row[row] - 2 * PR::EOFF;
        base = args.m_div > 0 ? (row % args.m_div) * args.s_m1 + (row / args.m_div) * args.s_m2 : row * args.s_m1;
      }
      const int ncol = n0 + c * 32 + lane;  // the column whose exponent this lane fetches
      // EPI_STOREMAX: the row's block index a = row / m_div selects the staging column n + N a
      const int64_t arow = (row_ok && args.m_div > 0) ? row / args.m_div : 0;
      float cmax[EPI == EPI_STOREMAX ? 32 : 1];
      if constexpr (EPI == EPI_STOREMAX) {
#pragma unroll
        for (int j = 0; j < 32; ++j) cmax[j] = 0.f;
      }
      // the column exponent of aux function p + 1 is fetched while p is processed (its load
      // latency would otherwise stall every aux function's epilogue)
      const int* const ecp = args.e_col + (int64_t)(args.b_off + p_begin) * args.N + ncol;
      int ec_next = (nP > 0 && ncol < args.N) ? ecp[0] : 0;
      for (int p = 0; p < nP; ++p) {
        const int b = p & 1;
        const int ec = ec_next;
        if (p + 1 < nP && ncol < args.N) ec_next = ecp[(int64_t)(p + 1) * args.N];
        // warp-uniform decision: tcgen05.ld is a whole-warp instruction
        if (!__all_sync(0xffffffffu, mbar_wait(accf0 + 8 * b, (p >> 1) & 1, args.err))) break;
        fence_after_sync();
        const int Pl = p_begin + p;
        const uint32_t lane_base = tmem + (uint32_t)b * ACC + ((uint32_t)(q * 32) << 16);
        const int64_t pbase = base + (int64_t)Pl * args.s_p;
        if constexpr (PR::NACC == 4) {
          float2* const o = reinterpret_cast<float2*>(args.out) + pbase + (int64_t)(n0 + c * 32) * args.s_n;
          const int sn = (int)args.s_n;
          // the common case without per-element predicates or range checks: every row and
          // column of the chunk in range, every factor 2^(erow + ec) a normal float (its bit
          // pattern (erow + ec + 127) << 23)
          int emn = ec, emx = ec;
          for (int o2 = 16; o2 > 0; o2 >>= 1) {
            emn = min(emn, __shfl_xor_sync(0xffffffffu, emn, o2));
            emx = max(emx, __shfl_xor_sync(0xffffffffu, emx, o2));
          }
          const bool fast = __all_sync(0xffffffffu, row_ok && erow + emn >= -126 && erow + emx <= 127) &&
                            args.N - (n0 + c * 32) >= 32;
          const int eb = erow + 127;
          // two halves of 16 columns: four accumulators of 16 columns in registers at a time
#pragma unroll
          for (int hf = 0; hf < 2; ++hf) {
            float v0[16], v1[16], v2[16], v3[16];
            tmem_ld16x4(lane_base + (uint32_t)(0 * BN + c * 32 + 16 * hf), lane_base + (uint32_t)(1 * BN + c * 32 + 16 * hf),
                        lane_base + (uint32_t)(2 * BN + c * 32 + 16 * hf), lane_base + (uint32_t)(3 * BN + c * 32 + 16 * hf),
                        v0, v1, v2, v3);
            if constexpr (PR::S <= 3) {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) v3[jj] = 0.f;  // groups 0-2 only: the fourth accumulator is unused
            }
            if (fast) {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) {
                const int j = 16 * hf + jj;
                const float f = __uint_as_float((unsigned)(eb + __shfl_sync(0xffffffffu, ec, j)) << 23);
                float hi, lo;
                combine4(v0[jj], v1[jj], v2[jj], v3[jj], hi, lo);
                __stcs(o + j * sn, make_float2(hi * f, lo * f));
                if constexpr (EPI == EPI_STOREMAX) cmax[j] = fmaxf(cmax[j], fabsf(hi * f));
              }
            } else {
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) {
                const int j = 16 * hf + jj;
                const float f = pow2f(erow + __shfl_sync(0xffffffffu, ec, j));
                if (row_ok && n0 + c * 32 + j < args.N) {
                  float hi, lo;
                  combine4(v0[jj], v1[jj], v2[jj], v3[jj], hi, lo);
                  __stcs(o + j * sn, make_float2(hi * f, lo * f));
                  if constexpr (EPI == EPI_STOREMAX) cmax[j] = fmaxf(cmax[j], fabsf(hi * f));
                }
              }
            }
          }
        } else if constexpr (EPI == EPI_SPLIT16) {
          // B (O_P) carries one exponent per aux function: one factor per row and P, with
          // T's power-of-two scale folded into the exponent
          float v[32];
          tmem_ld32(lane_base + (uint32_t)(c * 32), v);
          // (every column of O_P carries the aux function's exponent: lane 0's, fetched ahead)
          const float f = pow2f(erow + __shfl_sync(0xffffffffu, ec, 0) + pow2_exponent(*args.tscale));
          const int64_t off = pbase + (int64_t)(n0 + c * 32) * args.s_n;
          if (row_ok)
            store_split32(v, f, reinterpret_cast<__half*>(args.out) + off, reinterpret_cast<__half*>(args.out_lo) + off,
                          (int)args.s_n, min(32, args.N - (n0 + c * 32)));
        } else {
          float v[32];
          tmem_ld32(lane_base + (uint32_t)(c * 32), v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c * 32 + j;
            const float f = pow2f(erow + __shfl_sync(0xffffffffu, ec, j));
            if (row_ok && n < args.N) __stcs(reinterpret_cast<float*>(args.out) + pbase + n * args.s_n, v[j] * f);
          }
        }
        fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce0 + 8 * b);
      }
      if constexpr (EPI == EPI_STOREMAX) {
        // column maxima over the warp's 32 rows: one atomic per column when the rows share a
        // block index, else one per row
        const int64_t a0 = __shfl_sync(0xffffffffu, arow, 0);
        const bool uniform = __all_sync(0xffffffffu, !row_ok || arow == a0) && __any_sync(0xffffffffu, row_ok);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c * 32 + j;
          if (n >= args.N) continue;
          float m = row_ok ? cmax[j] : 0.f;
          if (uniform) {
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) atomicMax(args.colmax + n + (int64_t)args.N * a0, (unsigned long long)__float_as_uint(m));
          } else if (row_ok) {
            atomicMax(args.colmax + n + (int64_t)args.N * arow, (unsigned long long)__float_as_uint(m));
          }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 1) tmem_dealloc(tmem, 2 * ACC);
}

// Inner T generation with the bra tile resident (split FP16, K = nocc <= 128): one CTA per SM
// and (row tile, range of aux functions).  A row tile is 128 consecutive nu of one perturbation
// a (the last tile of each a is partial), so that T_P's tile is one box of the planes' layout.
// The A tile -- every K block of the bra rows, both planes -- is loaded once and stays in
// shared memory; O_P's 128-row tile (all i of a column, N = 128 >= nocc) streams through a
// 4-stage ring.  Double-buffered TMEM accumulators (2 x 128 columns) let the epilogue of aux
// function p overlap the MMAs of p + 1.  Each epilogue warp (32 nu x 64 i) writes the FP16
// hi / lo planes of T * tscale of its part into its own shared-memory tile [64 i][32 nu] and
// stores them with TMA (cp.async.bulk.tensor, clipped at nu = nao): the global writes are bulk
// transfers off the warps' issue path, and a warp waits only for its own previous stores to
// have left shared memory, so the stores of aux function p drain while p + 1 is computed.
// Warp 0: TMA loads, warp 1: MMA issuer and TMEM owner, warps 2-9: epilogue.
struct ResT {
  static constexpr int BN = 128, STAGES = 4, MAX_KB = 4, THREADS = 320, EPI_WARPS = 8;
  static constexpr int A_TILE = BM * BK * 2;            // 8 KB: one K block of one plane
  static constexpr int B_TILE = BN * BK * 2;            // 8 KB
  static constexpr int A_BYTES = MAX_KB * 2 * A_TILE;   // 64 KB resident
  static constexpr int STAGE_BYTES = 2 * B_TILE;        // hi + lo of one K block of O_P
  static constexpr int WARP_OUT = 2 * 64 * 32 * 2;     // one warp's staged hi + lo tiles: 64 i x 32 nu
  static constexpr int OUT_BYTES = EPI_WARPS * WARP_OUT;
  static constexpr int SMEM_BYTES = A_BYTES + STAGES * STAGE_BYTES + OUT_BYTES + 1024 + 1024;
};

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// L2 policy that evicts the lines written first (T is streamed: read once, by term 1, after
// the chunk is complete), so that the O tiles the next aux functions read stay in L2
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, uint32_t src, int c0, int c1, int c2,
                                             uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group.L2::cache_hint [%0, {%2, %3, %4}], [%1], %5;" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(src), "r"(c0), "r"(c1), "r"(c2), "l"(policy)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__global__ void __launch_bounds__(320, 1)
    tc_tgen_resident_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB,
                            const __grid_constant__ CUtensorMap mTh0, const __grid_constant__ CUtensorMap mTh1,
                            const __grid_constant__ CUtensorMap mTl0, const __grid_constant__ CUtensorMap mTl1,
                            OzArgs args) {
  constexpr int STAGES = ResT::STAGES, BN = ResT::BN;
  constexpr uint32_t ACC = BN;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* ares = smem;
  uint8_t* ring = smem + ResT::A_BYTES;
  uint8_t* outs = ring + STAGES * ResT::STAGE_BYTES;  // per epilogue warp: [plane][64 i][32 nu] FP16
  uint64_t* bars = reinterpret_cast<uint64_t*>(outs + ResT::OUT_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 6);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);
  const uint32_t accf0 = smem_u32(bars + 2 * STAGES), acce0 = smem_u32(bars + 2 * STAGES + 2);
  const uint32_t done = smem_u32(bars + 2 * STAGES + 4), abar = smem_u32(bars + 2 * STAGES + 5);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // row tile: 128 nu of perturbation a (rows a nao + nu of the bra planes)
  const int nao = (int)args.m_div;
  const int tpa = (nao + BM - 1) / BM;
  const int a_pert = blockIdx.y / tpa, nu0 = (blockIdx.y % tpa) * BM;
  const int m0 = a_pert * nao + nu0;
  const int p_begin = blockIdx.x * args.p_per_cta;
  const int nP = min(args.np - p_begin, args.p_per_cta);
  const int nkb = args.nkb;  // <= MAX_KB (host checks)
  const int no = args.N;     // <= BN (host checks)

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, ResT::EPI_WARPS);
    }
    mbar_init(done, 1);
    mbar_init(abar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tmem_slot), 2 * ACC);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (nP > 0) {
    if (warp == 0 && lane == 0) {
      // resident A: every K block of both planes, once
      mbar_expect_tx(abar, (uint32_t)(nkb * 2 * ResT::A_TILE));
      for (int kb = 0; kb < nkb; ++kb)
        for (int t = 0; t < 2; ++t)
          tma_load_3d(smem_u32(ares + (kb * 2 + t) * ResT::A_TILE), &mA, abar, kb * BK, m0, t * args.a_depth + args.a_off);
      // O_P tiles of the aux range through the ring
      const int total = nP * nkb;
      int issued = 0;
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        if (!mbar_wait(empty0 + 8 * s, ((it / STAGES) & 1) ^ 1, args.err)) break;
        issued = it + 1;
        const uint32_t full = full0 + 8 * s;
        mbar_expect_tx(full, ResT::STAGE_BYTES);
        const int P = p_begin + it / nkb;
        const int k0 = (it % nkb) * BK;
        const uint32_t st = smem_u32(ring + s * ResT::STAGE_BYTES);
        for (int t = 0; t < 2; ++t) tma_load_3d(st + t * ResT::B_TILE, &mB, full, k0, 0, t * args.b_depth + args.b_off + P);
      }
      for (int it = max(0, issued - STAGES); it < issued; ++it)
        mbar_wait(full0 + 8 * (it % STAGES), (it / STAGES) & 1, nullptr);
      mbar_wait(abar, 0, nullptr);  // the resident copies have landed before the CTA may exit
    } else if (warp == 1 && lane == 0) {
      constexpr uint32_t idesc = instr_desc_f16(BM, BN, false);
      bool ok = mbar_wait(abar, 0, args.err);
      fence_after_sync();
      for (int p = 0; p < nP && ok; ++p) {
        const int b = p & 1;
        if (!mbar_wait(acce0 + 8 * b, ((p >> 1) & 1) ^ 1, args.err)) break;
        fence_after_sync();
        const uint32_t acc_base = tmem + (uint32_t)b * ACC;
        for (int kb = 0; kb < nkb; ++kb) {
          const int it = p * nkb + kb;
          const int s = it % STAGES;
          if (!mbar_wait(full0 + 8 * s, (it / STAGES) & 1, args.err)) { ok = false; break; }
          fence_after_sync();
          const uint32_t ah = smem_u32(ares + (kb * 2 + 0) * ResT::A_TILE), al = ah + ResT::A_TILE;
          const uint32_t bh = smem_u32(ring + s * ResT::STAGE_BYTES), bl = bh + ResT::B_TILE;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint64_t dk = (uint64_t)((k * 32) >> 4);
            mma_f16(acc_base, smem_desc<64>(ah) + dk, smem_desc<64>(bh) + dk, idesc, (kb > 0 || k > 0) ? 1u : 0u);
            mma_f16(acc_base, smem_desc<64>(ah) + dk, smem_desc<64>(bl) + dk, idesc, 1u);
            mma_f16(acc_base, smem_desc<64>(al) + dk, smem_desc<64>(bh) + dk, idesc, 1u);
          }
          mma_commit(empty0 + 8 * s);
        }
        if (ok) mma_commit(accf0 + 8 * b);
      }
      mma_commit(done);
      mbar_wait(done, 0, nullptr);
    } else if (warp >= 2) {
      // epilogue: TMEM lane quarter q (rows nu0 + 32 q + lane), columns i in [64 h, 64 h + ni)
      const int q = warp & 3;
      const int h = (warp - 2) >> 2;
      const int ni = min(64, no - 64 * h);  // this warp's columns (none when nocc <= 64 and h = 1)
      const int nul = q * 32 + lane;
      const bool row_ok = nu0 + nul < nao;
      const int erow = row_ok ? args.e_row[m0 + nul] - 2 * Split2::EOFF : 0;
      // T's scale is a power of two: its exponent joins the row's and the aux function's
      const int ets = pow2_exponent(*args.tscale);
      // O_P's planes carry one exponent per aux function, so the row has one factor per P; the
      // exponent of p + 1 is fetched while p is processed
      const int* const eP = args.e_col + (int64_t)(args.b_off + p_begin) * args.N;
      int e_next = eP[0];
      uint8_t* const wst = outs + (warp - 2) * ResT::WARP_OUT;
      __half* const sh = reinterpret_cast<__half*>(wst) + lane;  // [64 i][32 nu]
      __half* const sl = sh + 64 * 32;
      const CUtensorMap* const mh = h == 0 ? &mTh0 : &mTh1;
      const CUtensorMap* const ml = h == 0 ? &mTl0 : &mTl1;
      const uint64_t policy = l2_evict_first();
      for (int p = 0; p < nP; ++p) {
        const int b = p & 1;
        const int e_p = e_next;
        if (p + 1 < nP) e_next = eP[(int64_t)(p + 1) * args.N];
        // this warp's staged tiles of p - 1 have left shared memory before they are overwritten
        if (lane == 0) bulk_wait_read0();
        __syncwarp();
        if (!__all_sync(0xffffffffu, mbar_wait(accf0 + 8 * b, (p >> 1) & 1, args.err))) break;
        fence_after_sync();
        float v[2][32];
        const uint32_t tb = tmem + (uint32_t)b * ACC + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 64);
        tmem_ld32x2(tb, tb + 32, v[0], v[1]);
        fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce0 + 8 * b);  // accumulator b may take aux p + 2
        if (ni <= 0) continue;
        const float f = pow2f(erow + e_p + ets);
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
          const int jn = min(32, ni - 32 * cc);
          if (jn >= 32) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float x = v[cc][j] * f;
              const __half hh = __float2half_rn(x);
              sh[(32 * cc + j) * 32] = hh;
              sl[(32 * cc + j) * 32] = __float2half_rn(x - __half2float(hh));
            }
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (j < jn) {
                const float x = v[cc][j] * f;
                const __half hh = __float2half_rn(x);
                sh[(32 * cc + j) * 32] = hh;
                sl[(32 * cc + j) * 32] = __float2half_rn(x - __half2float(hh));
              }
            }
          }
        }
        fence_proxy_async();  // the generic-proxy writes are visible to the TMA stores
        __syncwarp();
        if (lane == 0 && nu0 + 32 * q < nao) {  // (a box wholly past nu = nao has nothing to store)
          const int Pl = p_begin + p;
          tma_store_3d(mh, smem_u32(wst), nu0 + 32 * q, a_pert * no + 64 * h, Pl, policy);
          tma_store_3d(ml, smem_u32(wst + ResT::WARP_OUT / 2), nu0 + 32 * q, a_pert * no + 64 * h, Pl, policy);
          bulk_commit();
        }
      }
      if (lane == 0) bulk_wait0();  // the stores are complete before the CTA exits
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 1) tmem_dealloc(tmem, 2 * ACC);
}

// Generic row slicer: row r, element k at src[(r % rdiv) rs1 + (r / rdiv) rs2 + k ks]
// (rdiv = 0: r rs1 + k ks); one warp per row: exponent of the row max, then the six slices
// to dst[t plane + r ld + k]; e_out[r] = exponent, scale_out[r] = 2^exponent (if non-null).
template <class PR, class TIn>
__global__ void slice_rows_kernel(const TIn* __restrict__ src, int64_t rows, int64_t K, int64_t rdiv, int64_t rs1,
                                  int64_t rs2, int64_t ks, typename PR::Elem* __restrict__ dst, int64_t ld,
                                  int64_t plane, int* __restrict__ e_out) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < rows; r += nw) {
    const TIn* p = src + (rdiv > 0 ? (r % rdiv) * rs1 + (r / rdiv) * rs2 : r * rs1);
    unsigned long long m = 0;
    for (int64_t k = lane; k < K; k += 32) m = max(m, abs_key(p[k * ks]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = key_exp(m, float_key<TIn>());
    for (int64_t k = lane; k < K; k += 32) Put<PR>::put(p[k * ks], e, dst + r * ld + k, plane);
    if (lane == 0) e_out[r] = e;
  }
}

// Group slicer: rows [g rpg, (g + 1) rpg) of src (row r, element k at src[r K + k]) share one
// exponent, that of the group's max; one block per group.  Planes to dst[t plane + r ld + k],
// the exponent to e_out[r] for every row of the group.
template <class PR, class TIn>
__global__ void slice_groups_kernel(const TIn* __restrict__ src, int64_t groups, int64_t rpg, int64_t K,
                                    typename PR::Elem* __restrict__ dst, int64_t ld, int64_t plane,
                                    int* __restrict__ e_out) {
  __shared__ unsigned long long red[32];
  const int64_t n = rpg * K;
  for (int64_t g = blockIdx.x; g < groups; g += gridDim.x) {
    const TIn* p = src + g * n;
    unsigned long long m = 0;
    for (int64_t t = threadIdx.x; t < n; t += blockDim.x) m = max(m, abs_key(p[t]));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
      m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0ull;
      for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (threadIdx.x == 0) red[0] = m;
    }
    __syncthreads();
    const int e = key_exp(red[0], float_key<TIn>());
    for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
      const int64_t r = g * rpg + t / K, k = t % K;
      Put<PR>::put(p[t], e, dst + r * ld + k, plane);
    }
    for (int64_t r = threadIdx.x; r < rpg; r += blockDim.x) e_out[g * rpg + r] = e;
    __syncthreads();
  }
}

// max |X[mu + n r]| over r in [0, nr) per mu (X col-major [n, nr]); atomics per thread
template <class TIn>
__global__ void rowmax_strided_kernel(const TIn* __restrict__ X, int64_t n, int64_t nr,
                                      unsigned long long* __restrict__ mx) {
  const int64_t mu = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (mu >= n) return;
  unsigned long long m = 0;
  for (int64_t r = blockIdx.y; r < nr; r += gridDim.y) m = max(m, abs_key(X[mu + n * r]));
  atomicMax(mx + mu, m);
}

// e = exponent of the max; scale = mult 2^(e - eoff)
__global__ void exp_scale_kernel(const unsigned long long* __restrict__ mx, int64_t n, double mult, bool is_float,
                                 int eoff, int* __restrict__ e_out, double* __restrict__ scale) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int e = key_exp(mx[i], is_float);
  e_out[i] = e;
  scale[i] = mult * ldexp(1.0, e - eoff);
}

// cderi slices [t][P][mu][ldk] of B_P[mu, nu] 2^-e_mu (B_P symmetric: read Bd[nu + nao mu + nao^2 P])
__global__ void slice_cderi_kernel(const double* __restrict__ Bd, int64_t nao, int64_t naux, int64_t ldk,
                                   const int* __restrict__ e_row, __nv_bfloat16* __restrict__ out) {
  const int64_t total = naux * nao * nao;
  const int64_t plane = naux * nao * ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t nu = t % nao;
    const int64_t r = t / nao;  // P * nao + mu
    slice6(Bd[t], e_row[r % nao], out + nu + ldk * r, plane);
  }
}

// Z^T slices [t][P][mu][ldj] of Z_P[mu, j] (row exponent e_mu), Z col-major [nao, nocc, naux]
template <class PR, class TIn>
__global__ void slice_zt_kernel(const TIn* __restrict__ Z, int64_t nao, int64_t no, int64_t naux, int64_t ldj,
                                const int* __restrict__ e_row, typename PR::Elem* __restrict__ out) {
  const int64_t total = nao * no * naux;
  const int64_t plane = naux * nao * ldj;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t mu = t % nao;
    const int64_t r = t / nao;  // j + no * P
    const int64_t j = r % no, P = r / no;
    Put<PR>::put(Z[t], e_row[mu], out + j + ldj * (mu + nao * P), plane);
  }
}

// Exact BF16 slices (the first NS planes) of FP32-pair staging rows: row r holds K pairs at
// T[r ld + k] with the exponent of staging column r % N; planes [t][r][ld].  One warp per row,
// two elements per lane and step (16-byte loads, BF16-pair stores), the scale 2^(36 - e) as two
// exact power-of-two factors (e in [-149, 128] keeps both normal).
template <int NS>
__global__ void slice_pairs_kernel(const float2* __restrict__ T, int64_t rows, int64_t N, int64_t ld, int K,
                                   const int* __restrict__ e_col, __nv_bfloat16* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t plane = rows * ld;
  for (int64_t r = w0; r < rows; r += nw) {
    const int sc = 36 - e_col[r % N], s1 = sc >> 1, s2 = sc - s1;
    const float f1 = __int_as_float((127 + s1) << 23), f2 = __int_as_float((127 + s2) << 23);
    const float2* src = T + r * ld;
    __nv_bfloat16* dst = out + r * ld;
    for (int k = 2 * lane; k < K; k += 64) {
      if (k + 1 < K) {
        const float4 p = *reinterpret_cast<const float4*>(src + k);
        float d0[NS], d1[NS];
        digits_pair<NS>(p.x, p.y, f1, f2, d0);
        digits_pair<NS>(p.z, p.w, f1, f2, d1);
#pragma unroll
        for (int t = 0; t < NS; ++t)
          *reinterpret_cast<__nv_bfloat162*>(dst + t * plane + k) = __floats2bfloat162_rn(d0[t], d1[t]);
      } else {
        const float2 p = src[k];
        float d0[NS];
        digits_pair<NS>(p.x, p.y, f1, f2, d0);
#pragma unroll
        for (int t = 0; t < NS; ++t) dst[t * plane + k] = __float2bfloat16_rn(d0[t]);
      }
    }
  }
}

// max_{j,i} |O_P[j, i]| per aux function P (float bits); one block per P
__global__ void omax_kernel(const float* __restrict__ O, int64_t no2, int64_t naux, unsigned* __restrict__ omax) {
  __shared__ float red[32];
  for (int64_t P = blockIdx.x; P < naux; P += gridDim.x) {
    float m = 0.f;
    for (int64_t t = threadIdx.x; t < no2; t += blockDim.x) m = fmaxf(m, fabsf(O[P * no2 + t]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
      omax[P] = __float_as_uint(m);
    }
    __syncthreads();
  }
}

// max over (nu, a) of sum_j |bra[nu + nao j + nao no a]| (float bits, atomicMax into *out)
__global__ void bra_rowsum_max_kernel(const float* __restrict__ bra, int64_t nao, int64_t no, int64_t nb,
                                      unsigned* __restrict__ out) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // nu + nao a
  float sum = 0.f;
  if (r < nao * nb) {
    const int64_t nu = r % nao, a = r / nao;
    for (int64_t j = 0; j < no; ++j) sum += fabsf(bra[nu + nao * j + nao * no * a]);
  }
  for (int o = 16; o > 0; o >>= 1) sum = fmaxf(sum, __shfl_xor_sync(0xffffffffu, sum, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(sum));
}

// max over rows m of sum_k |x[k + K m]| (float bits, atomicMax into *out); one warp per row
__global__ void rowsum_abs_max_kernel(const float* __restrict__ x, int64_t K, int64_t rows, unsigned* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float best = 0.f;
  for (int64_t r = w0; r < rows; r += nw) {
    float sum = 0.f;
    for (int64_t k = lane; k < K; k += 32) sum += fabsf(x[r * K + k]);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    best = fmaxf(best, sum);
  }
  // rounding of the FP32 sums is covered by the FP16 planes' headroom (the bound maps to 2^14,
  // FP16 holds 2^15)
  if (lane == 0 && best > 0.f) atomicMax(out, __float_as_uint(best * 1.0001f));
}

// *mx = an upper bound of |T_P[nu, (i,a)]| = |sum_j bra[nu,j,a] O_P[j,i]| over P in [0, npc):
// (max_{nu,a} sum_j |bra|) (max_{P,j,i} |O_P|), rounded up (float bits); one block
__global__ void tbound_kernel(const unsigned* __restrict__ bra_s, const unsigned* __restrict__ omax, int64_t npc,
                              unsigned* __restrict__ mx) {
  __shared__ float red[32];
  float m = 0.f;
  for (int64_t p = threadIdx.x; p < npc; p += blockDim.x) m = fmaxf(m, __uint_as_float(omax[p]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
    *mx = __float_as_uint(__uint_as_float(*bra_s) * m * 1.0001f);
  }
}

unsigned grid_for(int64_t total) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(total, 256), 1 << 20)); }
unsigned grid_warps(int64_t rows, int num_sms) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(rows * 32, 256), 16 * (int64_t)num_sms));
}

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

// 3-D BF16 / FP16 tensor map: dims {K, rows, depth}, row stride ld elements, box {32, box_rows, 1},
// 64B swizzle.
CUtensorMap make_map(const void* base, int64_t K, int64_t rows, int64_t depth, int64_t ld, int box_rows,
                     bool bf16 = true) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  auto fn = encode_fn();
  if (!fn) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)(ld * 2), (cuuint64_t)(ld * 2 * rows)};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(&m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

template <class PR, int BN>
bool set_short_smem_attr() {
  if constexpr (PR::NACC == 4) {
    return true;
  } else {
    return cudaFuncSetAttribute(tc_slice_kernel<PR, BN, SHORT_STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                Cfg<PR, BN, SHORT_STAGES>::SMEM_BYTES) == cudaSuccess;
  }
}

template <class PR, int BN>
bool set_smem_attr() {
  bool ok = cudaFuncSetAttribute(tc_slice_kernel<PR, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Cfg<PR, BN>::SMEM_BYTES) == cudaSuccess &&
            set_short_smem_attr<PR, BN>() &&
            cudaFuncSetAttribute(tc_slice_batched_kernel<PR, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Batched<PR>::SMEM_BYTES) == cudaSuccess;
  if constexpr (PR::NACC == 4)
    ok = ok && cudaFuncSetAttribute(tc_slice_batched_kernel<PR, 64, EPI_STOREMAX>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, Batched<PR>::SMEM_BYTES) == cudaSuccess;
  else
    ok = ok && cudaFuncSetAttribute(tc_slice_batched_kernel<PR, 64, EPI_SPLIT16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, Batched<PR>::SMEM_BYTES) == cudaSuccess;
  return ok;
}

// ---- launch-shape autotuner ---------------------------------------------------------------
// The first eager launch of each contraction shape times the candidate launch shapes with CUDA
// events and keeps the fastest for the process: K blocks per CTA for the split-K kernels
// (atomics into the output against parallelism; all within the exactness bound) and aux
// functions per CTA for the batched kernels (CTA count in waves of the SM count).  Not during
// stream capture, where the cached (or default) shape is used.
struct TuneKey {
  int kind;
  int64_t M, N, nkb, np;
  bool operator<(const TuneKey& o) const {
    return std::tie(kind, M, N, nkb, np) < std::tie(o.kind, o.M, o.N, o.nkb, o.np);
  }
};
struct TuneTable {
  std::mutex mu;
  std::map<TuneKey, int> best;
  bool find(const TuneKey& k, int& v) {
    std::lock_guard<std::mutex> g(mu);
    auto it = best.find(k);
    if (it == best.end()) return false;
    v = it->second;
    return true;
  }
  void put(const TuneKey& k, int v) {
    std::lock_guard<std::mutex> g(mu);
    best[k] = v;
  }
};
TuneTable& tune_table() {
  static TuneTable t;
  return t;
}
bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone;
}
template <class F>
float time_launch(cudaStream_t s, F&& launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  launch();
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

// split-K contraction: grid (tiles, K ranges)
template <class PR, int BN, int ST = PR::STAGES>
void launch_split_raw(cphf_ctx* c, const CUtensorMap& mA, const CUtensorMap& mB, const OzArgs& a) {
  const unsigned tiles = (unsigned)(a.m_tiles * div_up(a.N, BN));
  const int64_t ranges = div_up(a.total_kb, a.kb_per_cta);
  if (ranges > 65535) throw Error(CPHF_ERR_ARG, "tensor-core K term: grid too large");
  tc_slice_kernel<PR, BN, ST><<<dim3(tiles, (unsigned)ranges), 128, Cfg<PR, BN, ST>::SMEM_BYTES, c->stream>>>(mA, mB, a);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

template <class PR, int BN>
void launch_split(cphf_ctx* c, OzState& z, const CUtensorMap& mA, const CUtensorMap& mB, OzArgs a) {
  const TuneKey key{PR::S * 1000 + BN, a.M, a.N, a.nkb, a.total_kb};
  auto& tab = tune_table();
  int best = PR::NACC == 1 ? (int)std::max<int64_t>(1, div_up(a.total_kb, 4)) : KB_PER_CTA;
  if (!tab.find(key, best) && !capturing(c->stream)) {
    // candidates run into a scratch output (the real one accumulates)
    const size_t esize = PR::NACC == 4 ? 8 : 4;
    const size_t bytes = (size_t)a.ld_out * a.N * esize;
    z.tune_out.ensure(bytes, c->counter());
    OzArgs t = a;
    t.out = z.tune_out.p;
    float best_ms = 0.f;
    // exact slices: K ranges within the exactness bound; split FP16 (no bound): 1, 2 or 4
    // waves of CTAs over the tiles, each K range as long as that leaves it
    int cand[3] = {KB_PER_CTA, KB_PER_CTA / 2, KB_PER_CTA / 3};
    if (PR::NACC == 1) {
      const int64_t tiles = (int64_t)a.m_tiles * div_up(a.N, BN);
      const int64_t r0 = std::max<int64_t>(1, div_up(2 * (int64_t)c->num_sms, tiles));
      for (int q = 0; q < 3; ++q)
        cand[q] = (int)std::max<int64_t>(1, div_up(a.total_kb, std::min<int64_t>(r0 << q, a.total_kb)));
    }
    for (int kb : cand) {
      t.kb_per_cta = kb;
      if (div_up(t.total_kb, kb) > 65535) continue;
      const float ms = time_launch(c->stream, [&] { launch_split_raw<PR, BN>(c, mA, mB, t); });
      if (best_ms == 0.f || ms < best_ms) best_ms = ms, best = kb;
    }
    tab.put(key, best);
  }
  a.kb_per_cta = best;
  launch_split_raw<PR, BN>(c, mA, mB, a);
}

// batched contraction over a.np aux functions: grid (aux ranges, tiles)
template <class PR, int EPI>
void launch_batched_raw(cphf_ctx* c, const CUtensorMap& mA, const CUtensorMap& mB, OzArgs a, int waves) {
  const int64_t tiles = (int64_t)a.m_tiles * div_up(a.N, 64);
  if (tiles > 65535) throw Error(CPHF_ERR_ARG, "tensor-core K term: grid too large");
  a.p_per_cta = (int)std::max<int64_t>(1, std::min<int64_t>(a.np, a.np * tiles / (waves * (int64_t)c->num_sms)));
  const dim3 grid((unsigned)div_up(a.np, a.p_per_cta), (unsigned)tiles);
  tc_slice_batched_kernel<PR, 64, EPI><<<grid, Batched<PR>::THREADS, Batched<PR>::SMEM_BYTES, c->stream>>>(mA, mB, a);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

template <class PR, int EPI = EPI_STORE>
void launch_batched(cphf_ctx* c, const CUtensorMap& mA, const CUtensorMap& mB, const OzArgs& a) {
  const TuneKey key{PR::S * 1000 + 64 + 100 * EPI, a.M, a.N, a.nkb, a.np};
  auto& tab = tune_table();
  int best = 2;
  if (!tab.find(key, best) && !capturing(c->stream)) {
    // every candidate writes the same staging values: time them on the real output
    float best_ms = 0.f;
    for (int w : {2, 4, 8}) {
      const float ms = time_launch(c->stream, [&] { launch_batched_raw<PR, EPI>(c, mA, mB, a, w); });
      if (best_ms == 0.f || ms < best_ms) best_ms = ms, best = w;
    }
    tab.put(key, best);
    return;  // the last candidate already wrote the output
  }
  launch_batched_raw<PR, EPI>(c, mA, mB, a, best);
}

bool res_attr_ok() {
  static int state = -1;
  if (state < 0) {
    state = cudaFuncSetAttribute(tc_tgen_resident_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 ResT::SMEM_BYTES) == cudaSuccess ? 1 : 0;
    if (!state) cudaGetLastError();
  }
  return state == 1;
}

// row tiles: 128 nu of one perturbation (m_div = nao, M = nao nb)
void launch_tgen_resident_raw(cphf_ctx* c, const CUtensorMap& mA, const CUtensorMap& mB, const CUtensorMap* mT,
                              OzArgs a, int waves) {
  const int64_t tiles = div_up(a.m_div, (int64_t)BM) * (a.M / a.m_div);
  if (tiles > 65535) throw Error(CPHF_ERR_ARG, "tensor-core T generation: grid too large");
  a.p_per_cta = (int)std::max<int64_t>(1, std::min<int64_t>(a.np, a.np * tiles / (waves * (int64_t)c->num_sms)));
  const dim3 grid((unsigned)div_up(a.np, a.p_per_cta), (unsigned)tiles);
  tc_tgen_resident_kernel<<<grid, ResT::THREADS, ResT::SMEM_BYTES, c->stream>>>(mA, mB, mT[0], mT[1], mT[2], mT[3],
                                                                                 a);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

// aux functions per CTA from the waves of CTAs over the SMs, tuned once per shape (every
// candidate writes the same planes, so the last one's output stands)
void launch_tgen_resident(cphf_ctx* c, const CUtensorMap& mA, const CUtensorMap& mB, const CUtensorMap* mT,
                          const OzArgs& a) {
  const TuneKey key{9001, a.M, a.N, a.nkb, a.np};
  auto& tab = tune_table();
  int best = 2;
  if (!tab.find(key, best) && !capturing(c->stream)) {
    float best_ms = 0.f;
    for (int w : {1, 2, 4, 8}) {
      const float ms = time_launch(c->stream, [&] { launch_tgen_resident_raw(c, mA, mB, mT, a, w); });
      if (best_ms == 0.f || ms < best_ms) best_ms = ms, best = w;
    }
    tab.put(key, best);
    return;
  }
  launch_tgen_resident_raw(c, mA, mB, mT, a, best);
}

// 3-D FP16 map of T's planes for the TMA stores of the resident T generation: dims {nu (nao),
// n = i + nocc a (N), Pl (npc)}, row stride ldt, box {32 nu, ni, 1} (one epilogue warp's part,
// ni of its 64 columns), no swizzle (the staged tile is [ni][32] dense)
CUtensorMap make_t_store_map(const __half* base, int64_t nao, int64_t N, int64_t npc, int64_t ldt, int64_t ni) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  auto fn = encode_fn();
  if (!fn) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)nao, (cuuint64_t)N, (cuuint64_t)npc};
  cuuint64_t strides[2] = {(cuuint64_t)(ldt * 2), (cuuint64_t)(ldt * 2 * N)};
  cuuint32_t box[3] = {32, (cuuint32_t)ni, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<__half*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}


OzArgs base_args(OzState& z, int M, int N) {
  OzArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = M;
  a.N = N;
  a.m_tiles = (int)div_up(M, BM);
  a.kb_per_cta = KB_PER_CTA;
  a.err = z.err.as<int>();
  return a;
}

}  // namespace

bool oz_available(cphf_ctx* c) {
  int major = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c->device);
  if (major != 10 || encode_fn() == nullptr) return false;
  static bool attr_ok = false, tried = false;
  if (!tried) {
    tried = true;
    attr_ok = set_smem_attr<Exact6, 128>() && set_smem_attr<Exact6c, 128>() && set_smem_attr<Exact6c3, 128>() &&
              set_smem_attr<Split2, 128>();
    if (!attr_ok) cudaGetLastError();
  }
  return attr_ok;
}

bool oz_supported(const cphf_ctx* c) {
  for (int s = 0; s < c->nspin; ++s)
    if (c->spin[s].nocc > KMAX) return false;
  return c->nao <= KMAX;
}

void oz_prepare_cderi(cphf_ctx* c, OzState& z) {
  const int64_t nao = c->nao, naux = c->naux;
  z.ldk = (nao + 7) / 8 * 8;
  z.A.ensure((size_t)S * naux * nao * z.ldk * 2, c->counter());
  z.rowscale.ensure((size_t)nao * 8, c->counter());
  z.e_row.ensure((size_t)nao * 4, c->counter());
  z.mx.ensure((size_t)std::max<int64_t>(nao, 1) * 8, c->counter());
  z.err.ensure(sizeof(int), c->counter());
  CPHF_CUDA(cudaMemsetAsync(z.mx.p, 0, (size_t)nao * 8, c->stream));
  const unsigned gx = (unsigned)div_up(nao, 256);
  const unsigned gy = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nao * naux, 8 * (int64_t)c->num_sms / gx + 1));
  rowmax_strided_kernel<double><<<dim3(gx, gy), 256, 0, c->stream>>>(c->Bd.as<double>(), nao, nao * naux,
                                                              z.mx.as<unsigned long long>());
  exp_scale_kernel<<<grid_for(nao), 256, 0, c->stream>>>(z.mx.as<unsigned long long>(), nao, 1.0, false, 0,
                                                         z.e_row.as<int>(), z.rowscale.as<double>());
  slice_cderi_kernel<<<grid_for(naux * nao * nao), 256, 0, c->stream>>>(c->Bd.as<double>(), nao, naux, z.ldk,
                                                                        z.e_row.as<int>(), z.A.as<__nv_bfloat16>());
  count_launch(3);
  CPHF_CUDA(cudaGetLastError());
  for (auto& sp : z.spin) sp.ready = false;
  z.ready = true;
}

// O, Z (K = nu) and Z^T (K = j) slices of one spin
static void oz_prepare_spin(cphf_ctx* c, OzState& z, int s) {
  const SpinState& sp = c->spin[s];
  OzSpin& o = z.spin[s];
  const int64_t nao = c->nao, naux = c->naux, no = sp.nocc, ldk = z.ldk;
  const int64_t ldj = o.ldj = (no + 7) / 8 * 8;
  // O_P[j, i]: rows (i, P) at O + no (i + no P), K = j
  o.O.ensure((size_t)S * naux * no * ldj * 2, c->counter());
  o.eO.ensure((size_t)naux * no * 4, c->counter());
  slice_rows_kernel<Exact6, double><<<grid_warps(naux * no, c->num_sms), 256, 0, c->stream>>>(
      sp.O.as<double>(), naux * no, no, 0, no, 0, 1, o.O.as<__nv_bfloat16>(), ldj, naux * no * ldj, o.eO.as<int>());
  // Z_P[nu, i]: rows (i, P) at Z + nao (i + no P), K = nu
  o.Z.ensure((size_t)S * naux * no * ldk * 2, c->counter());
  o.eZ.ensure((size_t)naux * no * 4, c->counter());
  slice_rows_kernel<Exact6, double><<<grid_warps(naux * no, c->num_sms), 256, 0, c->stream>>>(
      sp.Z.as<double>(), naux * no, nao, 0, nao, 0, 1, o.Z.as<__nv_bfloat16>(), ldk, naux * no * ldk, o.eZ.as<int>());
  // Z_P[mu, j]: rows mu (scale over all j, P), per-P blocks of K = j
  o.Zt.ensure((size_t)S * naux * nao * ldj * 2, c->counter());
  o.sZt.ensure((size_t)nao * 8, c->counter());
  o.eZt.ensure((size_t)nao * 4, c->counter());
  CPHF_CUDA(cudaMemsetAsync(z.mx.p, 0, (size_t)nao * 8, c->stream));
  const unsigned gx = (unsigned)div_up(nao, 256);
  const unsigned gy = (unsigned)std::max<int64_t>(1, std::min<int64_t>(no * naux, 8 * (int64_t)c->num_sms / gx + 1));
  rowmax_strided_kernel<double><<<dim3(gx, gy), 256, 0, c->stream>>>(sp.Z.as<double>(), nao, no * naux,
                                                              z.mx.as<unsigned long long>());
  exp_scale_kernel<<<grid_for(nao), 256, 0, c->stream>>>(z.mx.as<unsigned long long>(), nao, 1.0, false, 0,
                                                         o.eZt.as<int>(), o.sZt.as<double>());
  slice_zt_kernel<Exact6, double><<<grid_for(nao * no * naux), 256, 0, c->stream>>>(sp.Z.as<double>(), nao, no, naux, ldj,
                                                                    o.eZt.as<int>(), o.Zt.as<__nv_bfloat16>());
  count_launch(5);
  CPHF_CUDA(cudaGetLastError());
  o.ready = true;
}

template <class PC>
static void oz_k_terms_t(cphf_ctx* c, OzState& z, int s, const double* bra, int64_t nb, double alpha,
                         double* out) {
  // correction precisions are profiled as their own classes
  constexpr int kP = PC::S == 6 ? PROF_TC_OZAKI : PC::S == 4 ? PROF_OZC_KTERM : PROF_OZC3_KTERM;
  constexpr int tP = PC::S == 6 ? PROF_OZ_TGEN : PC::S == 4 ? PROF_OZC_TGEN : PROF_OZC3_TGEN;
  constexpr int wP = PC::S == 6 ? PROF_OZ_WGEN : PC::S == 4 ? PROF_OZC_WGEN : PROF_OZC3_WGEN;
  constexpr int qP = PC::S == 6 ? PROF_OZ_TERM2 : PC::S == 4 ? PROF_OZC_TERM2 : PROF_OZC3_TERM2;
  const int64_t nao = c->nao, naux = c->naux, no = c->spin[s].nocc;
  const int64_t N = no * nb;
  if (N <= 0 || nao <= 0) return;
  if (!z.ready) oz_prepare_cderi(c, z);
  OzSpin& os = z.spin[s];
  if (!os.ready) oz_prepare_spin(c, z, s);
  const int64_t ldk = z.ldk, ldj = os.ldj;
  CPHF_CUDA(cudaMemsetAsync(z.err.p, 0, sizeof(int), c->stream));

  // bra slices, both K orders: rows (j, a) over nu (W-gen A) and rows (nu, a) over j (T-gen A)
  z.braw.ensure((size_t)S * N * ldk * 2, c->counter());
  z.ebraw.ensure((size_t)N * 4, c->counter());
  {
    ProfScope ps_slice(c, PROF_SLICE_EXACT, 0.0, 16.0 * N * nao + 12.0 * N * ldk + 12.0 * nao * nb * ldj);
    slice_rows_kernel<Exact6, double><<<grid_warps(N, c->num_sms), 256, 0, c->stream>>>(
        bra, N, nao, 0, nao, 0, 1, z.braw.as<__nv_bfloat16>(), ldk, N * ldk, z.ebraw.as<int>());
    z.brat.ensure((size_t)S * nao * nb * ldj * 2, c->counter());
    z.ebrat.ensure((size_t)nao * nb * 4, c->counter());
    slice_rows_kernel<Exact6, double><<<grid_warps(nao * nb, c->num_sms), 256, 0, c->stream>>>(
        bra, nao * nb, no, nao, 1, nao * no, nao, z.brat.as<__nv_bfloat16>(), ldj, nao * nb * ldj, z.ebrat.as<int>());
    count_launch(2);
  }

  // chunk of aux functions: T staging (FP32 pair, 8 B) + slices (12 B) per element within the
  // context's chunk budget (8 GiB when there is room)
  const int64_t budget = c->lowp ? c->lowp->budget : (int64_t(8) << 30);
  int64_t np = std::max<int64_t>(1, budget / std::max<int64_t>(20 * N * ldk, 1));
  if (c->cfg.aux_chunk > 0) np = c->cfg.aux_chunk;
  np = std::min<int64_t>(std::min<int64_t>(np, naux), 65535);
  z.T.ensure((size_t)np * N * ldk * 8, c->counter());
  z.B.ensure((size_t)S * np * N * ldk * 2, c->counter());
  z.W.ensure((size_t)np * N * ldj * 8, c->counter());
  z.Ws.ensure((size_t)S * np * N * ldj * 2, c->counter());
  z.colscale.ensure((size_t)N * 8, c->counter());
  z.e_col.ensure((size_t)N * 4, c->counter());
  z.mxc.ensure((size_t)N * 8, c->counter());

  const CUtensorMap mCd = make_map(z.A.p, nao, nao, S * naux, ldk, BM);            // term 1 A
  const CUtensorMap mBt = make_map(z.brat.p, no, nao * nb, S, ldj, BM);            // T-gen A
  const CUtensorMap mO = make_map(os.O.p, no, no, S * naux, ldj, 64);               // T-gen B
  const CUtensorMap mBw = make_map(z.braw.p, nao, N, S, ldk, BM);                  // W-gen A
  const CUtensorMap mZ = make_map(os.Z.p, nao, no, S * naux, ldk, 64);             // W-gen B
  const CUtensorMap mZt = make_map(os.Zt.p, no, nao, S * naux, ldj, BM);           // term 2 A
  const int nkb_nao = (int)div_up(nao, BK), nkb_no = (int)div_up(no, BK);

  for (int64_t P0 = 0; P0 < naux; P0 += np) {
    const int64_t npc = std::min<int64_t>(np, naux - P0);
    const int64_t rows = npc * N;
    {
      // T-gen: T[Pl][(i,a)][nu] (FP32 pair), rows m = nu + nao a, columns i, K = j
      OzArgs a = base_args(z, (int)(nao * nb), (int)no);
      a.out = z.T.p;
      a.nkb = nkb_no;
      a.a_depth = 1;
      a.b_depth = (int)naux;
      a.b_off = (int)P0;
      a.e_row = z.ebrat.as<int>();
      a.e_col = os.eO.as<int>();
      a.m_div = nao; a.s_m1 = 1; a.s_m2 = ldk * no; a.s_n = ldk; a.s_p = N * ldk;
      a.colmax = z.mxc.as<unsigned long long>();  // T's column maxima, reduced in the epilogue
      ProfScope ps(c, tP, 2.0 * nao * nb * no * no * npc, 0.0);
      a.np = (int)npc;
      CPHF_CUDA(cudaMemsetAsync(z.mxc.p, 0, (size_t)N * 8, c->stream));
      launch_batched<PC, EPI_STOREMAX>(c, mBt, mO, a);
    }
    {
      ProfScope ps_slice(c, PROF_SLICE_EXACT, 0.0, (double)rows * (8.0 * nao + 2.0 * PC::S * ldk));
      exp_scale_kernel<<<grid_for(N), 256, 0, c->stream>>>(z.mxc.as<unsigned long long>(), N, alpha, true, 0,
                                                           z.e_col.as<int>(), z.colscale.as<double>());
      slice_pairs_kernel<PC::S><<<grid_warps(rows, c->num_sms), 256, 0, c->stream>>>(
          z.T.as<float2>(), rows, N, ldk, (int)nao, z.e_col.as<int>(), z.B.as<__nv_bfloat16>());
      count_launch(2);
    }
    {
      // term 1: out[mu, n] += alpha sum_{P, nu} B_P[mu, nu] T_P[nu, n]
      const CUtensorMap mT = make_map(z.B.p, nao, N, S * npc, ldk, BM);
      OzArgs a = base_args(z, (int)nao, (int)N);
      a.out = out;
      a.nkb = nkb_nao;
      a.total_kb = (int)(npc * nkb_nao);
      a.a_depth = (int)naux;
      a.a_off = (int)P0;
      a.a_per_p = 1;
      a.b_depth = (int)npc;
      a.rowscale = z.rowscale.as<double>();
      a.colscale = z.colscale.as<double>();
      a.ld_out = nao;
      ProfScope ps(c, kP, 2.0 * nao * N * nao * npc, 2.0 * S * nao * npc * (nao + N));
      launch_split<PC, 128>(c, z, mCd, mT, a);
    }
    {
      // W-gen: W[Pl][(i,a)][j] (FP32 pair), rows m = j + no a, columns i, K = nu
      OzArgs a = base_args(z, (int)N, (int)no);
      a.out = z.W.p;
      a.nkb = nkb_nao;
      a.a_depth = 1;
      a.b_depth = (int)naux;
      a.b_off = (int)P0;
      a.e_row = z.ebraw.as<int>();
      a.e_col = os.eZ.as<int>();
      a.m_div = no; a.s_m1 = 1; a.s_m2 = ldj * no; a.s_n = ldj; a.s_p = N * ldj;
      // W's staging column (i, a) = i + nocc (row / nocc): its maxima reduced in the epilogue
      a.colmax = z.mxc.as<unsigned long long>();
      ProfScope ps(c, wP, 2.0 * N * no * nao * npc, 0.0);
      a.np = (int)npc;
      CPHF_CUDA(cudaMemsetAsync(z.mxc.p, 0, (size_t)N * 8, c->stream));
      launch_batched<PC, EPI_STOREMAX>(c, mBw, mZ, a);
    }
    {
      ProfScope ps_slice(c, PROF_SLICE_EXACT, 0.0, (double)rows * (8.0 * no + 2.0 * PC::S * ldj));
      exp_scale_kernel<<<grid_for(N), 256, 0, c->stream>>>(z.mxc.as<unsigned long long>(), N, alpha, true, 0,
                                                           z.e_col.as<int>(), z.colscale.as<double>());
      slice_pairs_kernel<PC::S><<<grid_warps(rows, c->num_sms), 256, 0, c->stream>>>(
          z.W.as<float2>(), rows, N, ldj, (int)no, z.e_col.as<int>(), z.Ws.as<__nv_bfloat16>());
      count_launch(2);
    }
    {
      // term 2: out[mu, n] += alpha sum_{P, j} Z_P[mu, j] W_P[j, n]
      const CUtensorMap mW = make_map(z.Ws.p, no, N, S * npc, ldj, BM);
      OzArgs a = base_args(z, (int)nao, (int)N);
      a.out = out;
      a.nkb = nkb_no;
      a.total_kb = (int)(npc * nkb_no);
      a.a_depth = (int)naux;
      a.a_off = (int)P0;
      a.a_per_p = 1;
      a.b_depth = (int)npc;
      a.rowscale = os.sZt.as<double>();
      a.colscale = z.colscale.as<double>();
      a.ld_out = nao;
      ProfScope ps(c, qP, 2.0 * nao * N * no * npc, 2.0 * S * no * npc * (nao + N));
      launch_split<PC, 128>(c, z, mZt, mW, a);
    }
  }
  int flag = 0;
  CPHF_CUDA(cudaMemcpyAsync(&flag, z.err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  if (flag) throw Error(CPHF_ERR_TIMEOUT, "tensor-core FP64 K-term kernel: a bounded pipeline wait expired");
}

void oz_k_terms(cphf_ctx* c, OzState& z, int s, const double* bra, int64_t nb, double alpha, double* out,
                int correction_slices) {
  if (correction_slices == 3) oz_k_terms_t<Exact6c3>(c, z, s, bra, nb, alpha, out);
  else if (correction_slices == 4) oz_k_terms_t<Exact6c>(c, z, s, bra, nb, alpha, out);
  else oz_k_terms_t<Exact6>(c, z, s, bra, nb, alpha, out);
}

// ---- split-FP16 operator of the inner solves ----------------------------------------------
// O, Z (K = nu) and Z^T (K = j) split-FP16 planes of one spin, from the FP32 copies
static void lp_prepare_spin(cphf_ctx* c, OzState& z, int s) {
  const SpinState& sp = c->spin[s];
  OzSpin& o = z.spin[s];
  const int64_t nao = c->nao, naux = c->naux, no = sp.nocc;
  constexpr int S2 = Split2::S;
  z.ldk = (nao + 7) / 8 * 8;
  const int64_t ldk = z.ldk, ldj = o.ldj = (no + 7) / 8 * 8;
  z.mx.ensure((size_t)std::max<int64_t>(nao, 1) * 8, c->counter());
  o.O.ensure((size_t)S2 * naux * no * ldj * 2, c->counter());
  o.eO.ensure((size_t)naux * no * 4, c->counter());
  // one exponent per aux function (all its rows): the T-generation epilogue then scales a row
  // of an aux function's T by one factor.  The planes resolve O_P to 2^-38 max |O_P|, which
  // moves T_P[nu, (i,a)] by at most 2^-38 sum_j |bra| max |O_P| <= 2^-38 of the bound that
  // scales T's own FP16 planes (their finest step), so T loses nothing it keeps.
  slice_groups_kernel<Split2, float><<<(unsigned)std::min<int64_t>(naux, 65535), 256, 0, c->stream>>>(
      sp.O32.as<float>(), naux, no, no, o.O.as<__half>(), ldj, naux * no * ldj, o.eO.as<int>());
  o.Z.ensure((size_t)S2 * naux * no * ldk * 2, c->counter());
  o.eZ.ensure((size_t)naux * no * 4, c->counter());
  slice_rows_kernel<Split2, float><<<grid_warps(naux * no, c->num_sms), 256, 0, c->stream>>>(
      sp.Z32.as<float>(), naux * no, nao, 0, nao, 0, 1, o.Z.as<__half>(), ldk, naux * no * ldk, o.eZ.as<int>());
  o.Zt.ensure((size_t)S2 * naux * nao * ldj * 2, c->counter());
  o.sZt.ensure((size_t)nao * 8, c->counter());
  o.eZt.ensure((size_t)nao * 4, c->counter());
  CPHF_CUDA(cudaMemsetAsync(z.mx.p, 0, (size_t)nao * 8, c->stream));
  const unsigned gx = (unsigned)div_up(nao, 256);
  const unsigned gy = (unsigned)std::max<int64_t>(1, std::min<int64_t>(no * naux, 8 * (int64_t)c->num_sms / gx + 1));
  rowmax_strided_kernel<float><<<dim3(gx, gy), 256, 0, c->stream>>>(sp.Z32.as<float>(), nao, no * naux,
                                                                     z.mx.as<unsigned long long>());
  exp_scale_kernel<<<grid_for(nao), 256, 0, c->stream>>>(z.mx.as<unsigned long long>(), nao, 1.0, true,
                                                         Split2::EOFF, o.eZt.as<int>(), o.sZt.as<double>());
  slice_zt_kernel<Split2, float><<<grid_for(nao * no * naux), 256, 0, c->stream>>>(
      sp.Z32.as<float>(), nao, no, naux, ldj, o.eZt.as<int>(), o.Zt.as<__half>());
  o.Omax.ensure((size_t)naux * 4, c->counter());
  omax_kernel<<<(unsigned)std::min<int64_t>(naux, 65535), 256, 0, c->stream>>>(sp.O32.as<float>(), no * no, naux,
                                                                              o.Omax.as<unsigned>());
  o.Zmax.ensure((size_t)naux * 4, c->counter());
  omax_kernel<<<(unsigned)std::min<int64_t>(naux, 65535), 256, 0, c->stream>>>(sp.Z32.as<float>(), nao * no, naux,
                                                                              o.Zmax.as<unsigned>());
  count_launch(7);
  CPHF_CUDA(cudaGetLastError());
  o.ready = true;
}

void lp_begin(cphf_ctx* c, OzState& z, int s, const float* bra, int64_t nb) {
  if (!z.spin[s].ready) lp_prepare_spin(c, z, s);
  const int64_t nao = c->nao, no = c->spin[s].nocc, N = no * nb;
  const int64_t ldk = z.ldk, ldj = z.spin[s].ldj;
  constexpr int S2 = Split2::S;
  // rows (j, a) over nu (W-gen A) and rows (nu, a) over j (T-gen A)
  z.braw.ensure((size_t)S2 * N * ldk * 2, c->counter());
  z.ebraw.ensure((size_t)N * 4, c->counter());
  {
    ProfScope ps_slice(c, PROF_SLICE, 0.0, 8.0 * N * nao + 4.0 * N * ldk + 4.0 * nao * nb * ldj);
    slice_rows_kernel<Split2, float><<<grid_warps(N, c->num_sms), 256, 0, c->stream>>>(
        bra, N, nao, 0, nao, 0, 1, z.braw.as<__half>(), ldk, N * ldk, z.ebraw.as<int>());
    z.brat.ensure((size_t)S2 * nao * nb * ldj * 2, c->counter());
    z.ebrat.ensure((size_t)nao * nb * 4, c->counter());
    slice_rows_kernel<Split2, float><<<grid_warps(nao * nb, c->num_sms), 256, 0, c->stream>>>(
        bra, nao * nb, no, nao, 1, nao * no, nao, z.brat.as<__half>(), ldj, nao * nb * ldj, z.ebrat.as<int>());
    z.braS.ensure(sizeof(unsigned), c->counter());
    CPHF_CUDA(cudaMemsetAsync(z.braS.p, 0, sizeof(unsigned), c->stream));
    bra_rowsum_max_kernel<<<grid_for(nao * nb), 256, 0, c->stream>>>(bra, nao, no, nb, z.braS.as<unsigned>());
    // max over (j, a) of sum_nu |bra|, for the W bound
    z.braWS.ensure(sizeof(unsigned), c->counter());
    CPHF_CUDA(cudaMemsetAsync(z.braWS.p, 0, sizeof(unsigned), c->stream));
    rowsum_abs_max_kernel<<<grid_warps(N, c->num_sms), 256, 0, c->stream>>>(bra, nao, N, z.braWS.as<unsigned>());
    count_launch(4);
  }
  CPHF_CUDA(cudaGetLastError());
}

void lp_tgen_planes(cphf_ctx* c, OzState& z, int s, int64_t P0, int64_t npc, int64_t nb, int64_t ldt, __half* hi,
                    __half* lo, unsigned* mx, float* scale, float sA, float alpha, int* err) {
  const int64_t nao = c->nao, naux = c->naux, no = c->spin[s].nocc, N = no * nb;
  const int64_t ldj = z.spin[s].ldj;
  constexpr int S2 = Split2::S;
  const CUtensorMap mBt = make_map(z.brat.p, no, nao * nb, S2, ldj, BM, false);
  const CUtensorMap mO = make_map(z.spin[s].O.p, no, no, S2 * naux, ldj, 64, false);
  OzArgs a = base_args(z, (int)(nao * nb), (int)no);
  a.err = err;
  a.nkb = (int)div_up(no, BK);
  a.a_depth = 1;
  a.b_depth = (int)naux;
  a.b_off = (int)P0;
  a.e_row = z.ebrat.as<int>();
  a.e_col = z.spin[s].eO.as<int>();
  a.m_div = nao; a.s_m1 = 1; a.s_m2 = ldt * no; a.s_n = ldt; a.s_p = N * ldt;
  a.np = (int)npc;
  a.tscale = scale;
  a.out = hi;
  a.out_lo = lo;
  ProfScope ps(c, PROF_TC_SPLIT, 2.0 * nao * nb * no * no * npc, 2.0 * 2.0 * npc * N * nao);
  // FP16 scale from an upper bound of |T| (hi and lo keep their 22 bits for values within
  // 2^17 of the bound, so a loose bound costs nothing and saves a max pass over T)
  tbound_kernel<<<1, 256, 0, c->stream>>>(z.braS.as<unsigned>(), z.spin[s].Omax.as<unsigned>() + P0, npc, mx);
  count_launch();
  launch_t_scale(mx, sA, alpha, scale, c->stream);
  if (a.nkb <= ResT::MAX_KB && no <= ResT::BN && res_attr_ok()) {
    // bra tile resident, all i of a column in one 128-wide tile
    const CUtensorMap mO128 = make_map(z.spin[s].O.p, no, no, S2 * naux, ldj, ResT::BN, false);
    // store maps of the epilogue warps' parts: columns [0, 64) and [64, nocc)
    const int64_t n0c = std::min<int64_t>(no, 64), n1c = std::max<int64_t>(no - 64, 1);
    const CUtensorMap mT[4] = {make_t_store_map(hi, nao, N, npc, ldt, n0c), make_t_store_map(hi, nao, N, npc, ldt, n1c),
                               make_t_store_map(lo, nao, N, npc, ldt, n0c), make_t_store_map(lo, nao, N, npc, ldt, n1c)};
    launch_tgen_resident(c, mBt, mO128, mT, a);
  } else {
    launch_batched<Split2, EPI_SPLIT16>(c, mBt, mO, a);
  }
}

void lp_w_term2(cphf_ctx* c, OzState& z, int s, int64_t P0, int64_t npc, int64_t nb, double alpha, float* out,
                int* err) {
  const int64_t nao = c->nao, naux = c->naux, no = c->spin[s].nocc, N = no * nb;
  const int64_t ldk = z.ldk, ldj = z.spin[s].ldj;
  constexpr int S2 = Split2::S;
  const OzSpin& os = z.spin[s];
  z.Ws.ensure((size_t)S2 * npc * N * ldj * 2, c->counter());
  z.wsc.ensure(16, c->counter());
  unsigned* mx = z.wsc.as<unsigned>();
  float* wscale = reinterpret_cast<float*>(mx + 2);  // [0] = W's plane scale, [1] = alpha / [0]
  __half* ws = z.Ws.as<__half>();
  {
    // W-gen: FP16 planes of W_P[(j,a), i] * wscale into Ws[Pl][a][i][j] as one GEMM over the
    // chunk (rows (j, a), columns (i, Pl), K = nu); the scale from the upper bound
    // |W| <= max_(j,a) sum_nu |bra| * max_P |Z_P|, so no FP32 staging and no max pass
    ProfScope ps(c, PROF_TC_WGEN, 2.0 * N * no * nao * npc, 2.0 * S2 * (N + no * npc) * nao + 2.0 * S2 * npc * N * no);
    tbound_kernel<<<1, 256, 0, c->stream>>>(z.braWS.as<unsigned>(), os.Zmax.as<unsigned>() + P0, npc, mx);
    count_launch();
    launch_t_scale(mx, 1.f, (float)alpha, wscale, c->stream);
    const __half* zp = os.Z.as<__half>();
    const __half* bw = z.braw.as<__half>();
    tc_wgen_planes(c, bw, bw + N * ldk, N, zp, zp + naux * no * ldk, no * naux, no * P0, no * npc, nao, ldk,
                   z.ebraw.as<int>(), os.eZ.as<int>(), wscale, no, ldj, ldj * no, N * ldj, ws, ws + npc * N * ldj,
                   err);
  }
  {
    // term 2: out[mu, n] += alpha sum_{P, j} Z_P[mu, j] W_P[j, n] on the term-1 kernel's 256-wide
    // tiles (K = j per aux function in 64-wide blocks), rows scaled by Z^T's scales, every
    // element by alpha / wscale
    ProfScope ps(c, PROF_TC_TERM2, 2.0 * nao * N * no * npc, 2.0 * S2 * no * npc * (nao + N));
    const __half* zt = os.Zt.as<__half>();
    tc_planes_term(c, zt, zt + naux * nao * ldj, naux, P0, ws, ws + npc * N * ldj, npc, nao, N, no, ldj,
                   os.sZt.as<double>(), nullptr, out, nao, err, wscale + 1);
  }
}

// Split-FP16 contraction out[m, n] += rowscale[m] colscale[n] sum_k A[a_row0 + m, k] B[n, k]
// over FP16 hi / lo planes (plane stride rows x ld elements), K-major, FP32 atomics into out
// [m + ld_out n]; the K range is split over CTAs as the autotuner finds best.
template <class PR, class TOut>
void plane_gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0,
                int64_t M, int64_t N, int64_t K, const double* rowscale, const double* colscale, TOut* out,
                int64_t ld_out, int* err, int kb_per_cta, bool store, const RhoEpilogue* rho = nullptr) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  if (b_k0 % 8 != 0 || b_k0 < 0) throw Error(CPHF_ERR_ARG, "tensor-core contraction: B offset not 16-byte aligned");
  const CUtensorMap mA = make_map(A.p, A.kext, A.rows, PR::S, A.ld, BM, PR::BF16);
  const CUtensorMap mB = make_map(B.p, B.kext, B.rows, PR::S, B.ld, BM, PR::BF16);
  OzArgs a = base_args(z, (int)M, (int)N);
  a.err = err;
  a.out = out;
  a.nkb = (int)div_up(K, BK);
  a.total_kb = a.nkb;
  a.a_depth = 1;
  a.b_depth = 1;
  a.a_row0 = (int)a_row0;
  a.b_k0 = (int)b_k0;
  a.rowscale = rowscale;
  a.colscale = colscale;
  a.ld_out = ld_out;
  if (rho != nullptr) {
    if (PR::NACC != 1 || rho->nocc <= 0) throw Error(CPHF_ERR_ARG, "rho1 epilogue: split-FP16 contractions only");
    a.rho = rho->rho;
    a.rho_ao = rho->ao;
    a.ld_rho = rho->ld_rho;
    a.ld_ao = rho->ld_ao;
    a.rho_nocc = (int)rho->nocc;
  }
  if (kb_per_cta > 0) {
    a.kb_per_cta = PR::NACC == 4 ? std::min(kb_per_cta, KB_PER_CTA) : kb_per_cta;
    a.store = store && a.kb_per_cta >= a.total_kb;
    bool launched = false;
    if constexpr (PR::NACC == 1) {
      if (a.kb_per_cta <= 2 * SHORT_STAGES) {
        launch_split_raw<PR, 128, SHORT_STAGES>(c, mA, mB, a);
        launched = true;
      }
    }
    if (!launched) launch_split_raw<PR, 128>(c, mA, mB, a);
  } else {
    launch_split<PR, 128>(c, z, mA, mB, a);
  }
}

void lp_gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0, int64_t M,
             int64_t N, int64_t K, const double* rowscale, const double* colscale, float* out, int64_t ld_out,
             int* err, int kb_per_cta, bool store) {
  plane_gemm<Split2>(c, z, A, a_row0, B, b_k0, M, N, K, rowscale, colscale, out, ld_out, err, kb_per_cta, store);
}

void lp_gemm_rho(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0,
                 int64_t M, int64_t N, int64_t K, const double* rowscale, const double* colscale,
                 const RhoEpilogue& rho, int* err, int kb_per_cta) {
  plane_gemm<Split2>(c, z, A, a_row0, B, b_k0, M, N, K, rowscale, colscale, (float*)nullptr, 0, err, kb_per_cta, false,
                     &rho);
}

void oz_gemm(cphf_ctx* c, OzState& z, const PlaneMat& A, int64_t a_row0, const PlaneMat& B, int64_t b_k0, int64_t M,
             int64_t N, int64_t K, const double* rowscale, const double* colscale, double* out, int64_t ld_out,
             int* err, int kb_per_cta, bool store) {
  plane_gemm<Exact6>(c, z, A, a_row0, B, b_k0, M, N, K, rowscale, colscale, out, ld_out, err, kb_per_cta, store);
}

void oz_gemm_corr(cphf_ctx* c, OzState& z, int slices, const PlaneMat& A, int64_t a_row0, const PlaneMat& B,
                  int64_t b_k0, int64_t M, int64_t N, int64_t K, const double* rowscale, const double* colscale,
                  double* out, int64_t ld_out, int* err, int kb_per_cta, bool store) {
  if (slices == 3)
    plane_gemm<Exact6c3>(c, z, A, a_row0, B, b_k0, M, N, K, rowscale, colscale, out, ld_out, err, kb_per_cta, store);
  else
    plane_gemm<Exact6c>(c, z, A, a_row0, B, b_k0, M, N, K, rowscale, colscale, out, ld_out, err, kb_per_cta, store);
}

// Split-FP16 planes [t][r][ld] of FP32 rows r (K elements each, row stride rs), exponents to e_out.
void lp_slice_rows(cphf_ctx* c, const float* src, int64_t rows, int64_t K, int64_t rs, __half* dst, int64_t ld,
                   int* e_out) {
  ProfScope ps_slice(c, PROF_SLICE, 0.0, 4.0 * rows * K + 4.0 * rows * ld);
  slice_rows_kernel<Split2, float><<<grid_warps(rows, c->num_sms), 256, 0, c->stream>>>(
      src, rows, K, 0, rs, 0, 1, dst, ld, rows * ld, e_out);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

// The leading `slices` (3 or 4) of the same planes, for correction-precision contractions.
void oz_slice_rows_corr(cphf_ctx* c, int slices, const double* src, int64_t rows, int64_t K, int64_t rs,
                        __nv_bfloat16* dst, int64_t ld, int* e_out) {
  ProfScope ps_slice(c, PROF_SLICE, 0.0, 8.0 * rows * K + 2.0 * slices * rows * ld);
  if (slices == 3)
    slice_rows_kernel<Exact6c3, double><<<grid_warps(rows, c->num_sms), 256, 0, c->stream>>>(
        src, rows, K, 0, rs, 0, 1, dst, ld, rows * ld, e_out);
  else
    slice_rows_kernel<Exact6c, double><<<grid_warps(rows, c->num_sms), 256, 0, c->stream>>>(
        src, rows, K, 0, rs, 0, 1, dst, ld, rows * ld, e_out);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

// Exact BF16 slice planes [t][r][ld] of FP64 rows r (K elements each, row stride rs), exponents to e_out.
void oz_slice_rows(cphf_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, __nv_bfloat16* dst,
                   int64_t ld, int* e_out) {
  ProfScope ps_slice(c, PROF_SLICE, 0.0, 8.0 * rows * K + 2.0 * S * rows * ld);
  slice_rows_kernel<Exact6, double><<<grid_warps(rows, c->num_sms), 256, 0, c->stream>>>(
      src, rows, K, 0, rs, 0, 1, dst, ld, rows * ld, e_out);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

}  // namespace cphf
