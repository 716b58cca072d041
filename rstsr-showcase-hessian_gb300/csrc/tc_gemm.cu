// Tensor-core split-FP16 contraction of the RI-K term on sm_103a (tcgen05 + TMEM + TMA).
//
//   out[mu, n] += alpha * sum_P sum_nu B_P[mu, nu] T_P[nu, n],   T_P[nu, (i,a)] = sum_j bra[nu,j,a] O_P[j,i]
//
// which is term 1 of the exchange response, -sum_P (B_P bra_a) O_P (src/ri_jk/hess_r.rs:168-170).
//
// Precision: each FP64/FP32 operand x is scaled by a power of two s (|x s| <= 2^14) and
// split into two FP16 planes, x s = hi + lo (hi = fp16(x s), lo = fp16(x s - hi)), a
// 22-bit representation.  Three MMAs per K step, hi*hi + hi*lo + lo*hi, accumulate in
// FP32 in tensor memory; the dropped lo*lo term and the FP32 accumulation leave ~1e-6
// relative error, removed by the FP64 defect correction of the mixed solve.
//
// Kernel structure (one CTA per SM, 4 warps):
//   warp 0 lane 0  -- TMA producer: 3-D tiled loads (K = nu, row = mu or n, P) of the four
//                     planes into a 2-stage ring of 128B-swizzled shared-memory tiles (K = 64);
//   warp 1 lane 0  -- MMA issuer: tcgen05.mma.cta_group::1.kind::f16 (M=128, N=256, K=16),
//                     tcgen05.commit frees a stage when its MMAs retire;
//   warp 2         -- TMEM allocation (256 FP32 columns) and release;
//   warps 0-3      -- epilogue: tcgen05.ld of the 128 x 256 accumulator, scaled and
//                     atomically added to out (split over P ranges across CTAs).
// Every mbarrier wait is bounded; on expiry the kernel records an error flag and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "kernels.cuh"
#include "tc_gemm.cuh"
#include "tc_ptx.cuh"

namespace cphf {
namespace {
using namespace tcx;

constexpr int BM = 128, BN = 256, BK = 64;
constexpr int STAGES = 2;
constexpr int A_TILE = BM * BK * 2;  // bytes, FP16
constexpr int B_TILE = BN * BK * 2;
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;  // hi + lo planes of both operands
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*barriers*/ + 1024 /*alignment*/;
constexpr int TMEM_COLS = 256;

struct TcArgs {
  float* out;
  int64_t ld_out;   // out[mu + ld_out * n]
  int M, N;         // mu rows (nao), n columns
  int nkb;          // K blocks of 64 per aux function
  int np;           // aux functions in this chunk
  int p_per_cta;    // aux functions per CTA (P split)
  int pA0;          // global aux index of the chunk's first function (A coordinate)
  int m_tiles;
  const float* scale;  // device: alpha / (sA * sT), or null (1)
  const double* rowscale;  // per-row / per-column factors of the result (null: 1), the scales of
  const double* colscale;  // row- / column-scaled operand planes
  int* err;
};

__global__ void __launch_bounds__(128, 1)
    tc_term1_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                    const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, TcArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), accum = smem_u32(bars + 2 * STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_tile = blockIdx.x % args.m_tiles, n_tile = blockIdx.x / args.m_tiles;
  const int m0 = m_tile * BM, n0 = n_tile * BN;
  const int pbeg = blockIdx.y * args.p_per_cta;
  const int pend = min(args.np, pbeg + args.p_per_cta);
  const int total = (pend - pbeg) * args.nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
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
        const int P = pbeg + it / args.nkb;
        const int k0 = (it % args.nkb) * BK;
        uint8_t* st = smem + s * STAGE_BYTES;
        tma_load_3d(smem_u32(st), &mAh, full, k0, m0, args.pA0 + P);
        tma_load_3d(smem_u32(st + A_TILE), &mAl, full, k0, m0, args.pA0 + P);
        tma_load_3d(smem_u32(st + 2 * A_TILE), &mBh, full, k0, n0, P);
        tma_load_3d(smem_u32(st + 2 * A_TILE + B_TILE), &mBl, full, k0, n0, P);
      }
      // drain: the copies of the last round of every stage have landed before the CTA may exit
      for (int it = max(0, issued - STAGES); it < issued; ++it) {
        mbar_wait(full0 + 8 * (it % STAGES), (it / STAGES) & 1, nullptr);
      }
    } else if (warp == 1 && lane == 0) {
      // MMA issuer
      constexpr uint32_t idesc = instr_desc_f16(BM, BN, false);
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(full0 + 8 * s, ph, args.err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
        const uint64_t ah = smem_desc<128>(st), al = smem_desc<128>(st + A_TILE);
        const uint64_t bh = smem_desc<128>(st + 2 * A_TILE), bl = smem_desc<128>(st + 2 * A_TILE + B_TILE);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          const uint64_t dk = (uint64_t)((k * 32) >> 4);  // 16 FP16 = 32 B along K inside the swizzle atom
          mma_f16(tmem, ah + dk, bh + dk, idesc, (it > 0 || k > 0) ? 1u : 0u);
          mma_f16(tmem, ah + dk, bl + dk, idesc, 1u);
          mma_f16(tmem, al + dk, bh + dk, idesc, 1u);
        }
        mma_commit(empty0 + 8 * s);
      }
      mma_commit(accum);  // also covers an early exit: arrives when the issued MMAs retire
    }
    __syncwarp();
    // epilogue: all four warps, warp w owns TMEM lanes [32 w, 32 w + 32)
    // warp-uniform decision: tcgen05.ld is a whole-warp instruction
    const bool have = __all_sync(0xffffffffu, mbar_wait(accum, 0, args.err) && *(volatile int*)args.err == 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (have) {
      const int row = m0 + warp * 32 + lane;
      const float scale = (args.scale ? *args.scale : 1.f) *
                          ((args.rowscale && row < args.M) ? (float)args.rowscale[row] : 1.f);
      for (int c = 0; c < BN / 32; ++c) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
        // the chunk's 32 column factors: one load per lane, broadcast by shuffles
        const int nl = n0 + c * 32 + lane;
        const float csl = (args.colscale && nl < args.N) ? (float)args.colscale[nl] : 1.f;
        float cs[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) cs[j] = __shfl_sync(0xffffffffu, csl, j);
        if (row < args.M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c * 32 + j;
            if (n < args.N) atomicAdd(args.out + row + args.ld_out * (int64_t)n, scale * cs[j] * v[j]);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 2) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---- W generation: one persistent split-FP16 GEMM per aux chunk ---------------------------
//   W_P[(j,a), i] = sum_nu bra[nu, j, a] Z_P[nu, i]   (term 2's cderi_oxo_1, src/ri_jk/hess_r.rs:172-176,
//   with Z_P = B_P C_occ: mocc^T (B_P bra) reassociated as bra^T Z_P)
// for all P of the chunk as one GEMM: rows m = j + nocc a (A = bra's planes, K = nu), columns
// n = i + nocc Pl (B = Z's planes, whose rows (i, P) are contiguous), written as FP16 hi / lo
// planes of W * wscale (one power of two per chunk, from an upper bound of |W|) straight
// into the layout term 2 reads, out[j + ldj i + s_a a + s_p Pl] (K = j).
//   warp 0 lane 0 -- TMA producer over the CTA's tiles, 2-stage ring of the four planes;
//   warp 1        -- TMEM owner (2 x 256 columns); lane 0 issues the MMAs of tile t into
//                    accumulator t & 1 while the epilogue drains the other;
//   warps 2-9     -- epilogue: TMEM lane quarter warp & 3, column half (warp - 2) / 4.
// Tiles in a grouped raster: group_m row tiles walk every column tile with rows fastest, so a
// group's A tiles stay in L2 while B streams once per group.
struct WgArgs {
  __half* out_hi;
  __half* out_lo;
  int M, N;            // rows (nocc nb), columns (nocc npc)
  int nkb;             // K blocks of 64 (nu)
  int m_tiles, n_tiles, group_m;
  int b_row0;          // B row of column 0 (nocc P0)
  int no;              // j = m % no, a = m / no; i = n % no, Pl = n / no
  int ldj, s_a, s_p;   // 32-bit element offsets (the host checks the plane size)
  const int* e_row;    // exponent of A row m's planes (the product carries 2^(e_row + e_col - 2 EOFF))
  const int* e_col;    // exponent of B row b_row0 + n
  const float* wscale; // power of two
  int* err;
};
constexpr int WG_THREADS = 320, WG_EPI_WARPS = 8, WG_ACC = 256;
constexpr int SPLIT_EOFF = 14;  // FP16 planes: x 2^(14 - e), e the exponent of the row's max

__device__ __forceinline__ void wg_tile(const WgArgs& a, int t, int& m0, int& n0) {
  const int per_group = a.group_m * a.n_tiles;
  const int g = t / per_group, r = t % per_group;
  const int gm0 = g * a.group_m;
  const int gm = min(a.group_m, a.m_tiles - gm0);
  m0 = (gm0 + r % gm) * BM;
  n0 = (r / gm) * BN;
}

__global__ void __launch_bounds__(WG_THREADS, 1)
    tc_wgen_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                   const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, WgArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);
  const uint32_t accf0 = smem_u32(bars + 2 * STAGES), acce0 = smem_u32(bars + 2 * STAGES + 2);
  const uint32_t done = smem_u32(bars + 2 * STAGES + 4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles = args.m_tiles * args.n_tiles;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, WG_EPI_WARPS);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tmem_slot), 2 * WG_ACC);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    int it = 0, issued = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
      int m0, n0;
      wg_tile(args, t, m0, n0);
      for (int kb = 0; kb < args.nkb; ++kb, ++it) {
        const int s = it % STAGES;
        if (!mbar_wait(empty0 + 8 * s, ((it / STAGES) & 1) ^ 1, args.err)) { ok = false; break; }
        issued = it + 1;
        const uint32_t full = full0 + 8 * s;
        mbar_expect_tx(full, STAGE_BYTES);
        const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
        tma_load_3d(st, &mAh, full, kb * BK, m0, 0);
        tma_load_3d(st + A_TILE, &mAl, full, kb * BK, m0, 0);
        tma_load_3d(st + 2 * A_TILE, &mBh, full, kb * BK, args.b_row0 + n0, 0);
        tma_load_3d(st + 2 * A_TILE + B_TILE, &mBl, full, kb * BK, args.b_row0 + n0, 0);
      }
    }
    // the copies of the last round of every stage have landed before the CTA may exit
    for (int i = max(0, issued - STAGES); i < issued; ++i) mbar_wait(full0 + 8 * (i % STAGES), (i / STAGES) & 1, nullptr);
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = instr_desc_f16(BM, BN, false);
    int it = 0, lt = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++lt) {
      const int b = lt & 1;
      if (!mbar_wait(acce0 + 8 * b, ((lt >> 1) & 1) ^ 1, args.err)) break;
      fence_after_sync();
      const uint32_t acc = tmem + (uint32_t)(b * WG_ACC);
      for (int kb = 0; kb < args.nkb; ++kb, ++it) {
        const int s = it % STAGES;
        if (!mbar_wait(full0 + 8 * s, (it / STAGES) & 1, args.err)) { ok = false; break; }
        fence_after_sync();
        const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
        const uint64_t ah = smem_desc<128>(st), al = smem_desc<128>(st + A_TILE);
        const uint64_t bh = smem_desc<128>(st + 2 * A_TILE), bl = smem_desc<128>(st + 2 * A_TILE + B_TILE);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          const uint64_t dk = (uint64_t)((k * 32) >> 4);
          mma_f16(acc, ah + dk, bh + dk, idesc, (kb > 0 || k > 0) ? 1u : 0u);
          mma_f16(acc, ah + dk, bl + dk, idesc, 1u);
          mma_f16(acc, al + dk, bh + dk, idesc, 1u);
        }
        mma_commit(empty0 + 8 * s);
      }
      if (ok) mma_commit(accf0 + 8 * b);
    }
    // every issued MMA has retired before TMEM is released (also after an early exit)
    mma_commit(done);
    mbar_wait(done, 0, nullptr);
  } else if (warp >= 2) {
    const int q = warp & 3, h = (warp - 2) >> 2;
    // W's scale is a power of two: its exponent joins the row's and the column's
    const int ews = (int)((__float_as_uint(*args.wscale) >> 23) & 0xFF) - 127;
    // per tile: the row's exponent and the exponents of the lane's four columns, fetched one
    // tile ahead so that their load latency overlaps the previous tile's epilogue
    int m0n = 0, n0n = 0, erow_n = 0, ecl_n[4] = {0, 0, 0, 0};
    auto fetch = [&](int tt) {
      if (tt >= tiles) return;
      wg_tile(args, tt, m0n, n0n);
      const int m = m0n + q * 32 + lane;
      erow_n = m < args.M ? args.e_row[m] : 0;
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const int nl = n0n + h * 128 + cc * 32 + lane;
        ecl_n[cc] = nl < args.N ? args.e_col[args.b_row0 + nl] : 0;
      }
    };
    fetch(blockIdx.x);
    int lt = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++lt) {
      const int b = lt & 1;
      const int m0 = m0n, n0 = n0n;
      int ecl[4];
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) ecl[cc] = ecl_n[cc];
      const int m = m0 + q * 32 + lane;
      const bool row_ok = m < args.M;
      // the exponent of row m with the planes' offsets and W's scale (biased by 127)
      const int erow = erow_n - 2 * SPLIT_EOFF + ews + 127;
      fetch(t + gridDim.x);
      // warp-uniform decision: tcgen05.ld is a whole-warp instruction
      if (!__all_sync(0xffffffffu, mbar_wait(accf0 + 8 * b, (lt >> 1) & 1, args.err))) break;
      fence_after_sync();
      const int roff = row_ok ? (m % args.no) + (m / args.no) * args.s_a : 0;
      const bool rows_ok = __all_sync(0xffffffffu, row_ok);
#pragma unroll 1
      for (int cc = 0; cc < 4; ++cc) {
        const int c0 = n0 + h * 128 + cc * 32;
        float v[32];
        tmem_ld32(tmem + (uint32_t)(b * WG_ACC) + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 128 + cc * 32), v);
        // this lane's column: exponent and output offset, broadcast by shuffles
        const int nl = c0 + lane;
        const int ec = cc == 0 ? ecl[0] : cc == 1 ? ecl[1] : cc == 2 ? ecl[2] : ecl[3];  // registers, not local memory
        const int col = nl < args.N ? (nl % args.no) * args.ldj + (nl / args.no) * args.s_p : 0;
        const int jn = min(32, args.N - c0);
        // the factor 2^(e) with e = erow + ec - 127 as a bit pattern when it is a normal float
        // for the whole chunk (the common case), else clamped to the normal range: a nonzero
        // |v| >= 2^-48 (sums of FP16 products) with |v 2^e| <= 2^14 (the bound) keeps e <= 62,
        // and below 2^-126 v 2^e is under FP16's smallest subnormal either way, so the clamp
        // changes no stored plane
        int emn = ec, emx = ec;
        for (int o = 16; o > 0; o >>= 1) {
          emn = min(emn, __shfl_xor_sync(0xffffffffu, emn, o));
          emx = max(emx, __shfl_xor_sync(0xffffffffu, emx, o));
        }
        const bool fast = rows_ok && jn == 32 && __all_sync(0xffffffffu, erow + emn >= 1 && erow + emx <= 254);
        if (fast) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int off = roff + __shfl_sync(0xffffffffu, col, j);
            const float x = v[j] * __uint_as_float((unsigned)(erow + __shfl_sync(0xffffffffu, ec, j)) << 23);
            const __half hh = __float2half_rn(x);
            __stcs(args.out_hi + off, hh);
            __stcs(args.out_lo + off, __float2half_rn(x - __half2float(hh)));
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int ecj = __shfl_sync(0xffffffffu, ec, j);
            const int co = __shfl_sync(0xffffffffu, col, j);
            if (row_ok && j < jn) {
              const int e = min(max(erow + ecj, 1), 254);
              const float x = v[j] * __uint_as_float((unsigned)e << 23);
              const __half hh = __float2half_rn(x);
              __stcs(args.out_hi + (roff + co), hh);
              __stcs(args.out_lo + (roff + co), __float2half_rn(x - __half2float(hh)));
            }
          }
        }
      }
      fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce0 + 8 * b);
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 1) tmem_dealloc(tmem, 2 * WG_ACC);
}

// ---- FP16 plane splitting --------------------------------------------------------------
__device__ __forceinline__ void split_f16(double x, double s, __half* hi, __half* lo) {
  const double xs = x * s;
  const __half h = __double2half(xs);
  *hi = h;
  *lo = __double2half(xs - (double)__half2float(h));
}

// dense symmetric cderi (FP64 [P][mu][nu]) -> planes [P][mu][ldk] (nu contiguous)
__global__ void split_cderi_kernel(const double* __restrict__ Bd, int64_t nao, int64_t naux, int64_t ldk, double s,
                                   __half* __restrict__ hi, __half* __restrict__ lo) {
  const int64_t total = naux * nao * ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t nu = t % ldk;
    const int64_t r = t / ldk;  // P * nao + mu
    if (nu < nao) {
      const int64_t P = r / nao, mu = r % nao;
      split_f16(Bd[mu + nao * nu + nao * nao * P], s, hi + t, lo + t);
    } else {
      hi[t] = __float2half(0.f);
      lo[t] = __float2half(0.f);
    }
  }
}

__global__ void absmax_f64_kernel(const double* __restrict__ x, int64_t n, unsigned* out) {
  float m = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, (float)fabs(x[t]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// power-of-two scale bringing max |x| to at most 2^14; scale[0] = s, scale[1] = alpha / (sA * s)
__device__ __forceinline__ float pow2_scale(float mx) {
  if (!(mx > 0.f) || !isfinite(mx)) return 1.f;
  int e;
  frexpf(mx, &e);  // mx = f * 2^e, f in [0.5, 1)
  return ldexpf(1.f, 14 - e);
}

__global__ void t_scale_kernel(const unsigned* mx, float sA, float alpha, float* scale) {
  const float s = pow2_scale(__uint_as_float(*mx));
  scale[0] = s;
  scale[1] = alpha / (sA * s);
}

// ---- host side ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// 3-D FP16 tensor map: dims {K (= nao), rows, planes}, row stride ldk elements, box {64, rows, 1},
// 128B swizzle.
CUtensorMap make_map(const void* base, int64_t K, int64_t rows, int64_t depth, int64_t ldk, int box_rows) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  auto fn = encode_fn();
  if (!fn) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)(ldk * 2), (cuuint64_t)(ldk * 2 * rows)};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(CPHF_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

unsigned grid_for(int64_t total) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(div_up(total, 256), 1 << 20)); }

}  // namespace

void launch_t_scale(const unsigned* mx, float sA, float alpha, float* scale, cudaStream_t stream) {
  t_scale_kernel<<<1, 1, 0, stream>>>(mx, sA, alpha, scale);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

bool tc_available(cphf_ctx* c) {
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c->device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, c->device);
  if (major != 10 || encode_fn() == nullptr) return false;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(tc_term1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(tc_wgen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    attr_set = true;
  }
  return true;
}

void tc_prepare_cderi(cphf_ctx* c, DevBuf& hi, DevBuf& lo, int64_t& ldk) {
  const int64_t nao = c->nao, naux = c->naux;
  ldk = (nao + 7) / 8 * 8;
  // power-of-two scale from max |B|
  DevBuf mx;
  mx.ensure(sizeof(unsigned), nullptr);
  CPHF_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned), c->stream));
  absmax_f64_kernel<<<grid_for(nao * nao * naux), 256, 0, c->stream>>>(c->Bd.as<double>(), nao * nao * naux, mx.as<unsigned>());
  unsigned bits = 0;
  CPHF_CUDA(cudaMemcpyAsync(&bits, mx.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CPHF_CUDA(cudaStreamSynchronize(c->stream));
  float m;
  std::memcpy(&m, &bits, 4);
  int e = 0;
  std::frexp((double)m, &e);
  const double sA = (m > 0.f) ? std::ldexp(1.0, 14 - e) : 1.0;
  c->lowp->sA = sA;
  const size_t bytes = (size_t)naux * nao * ldk * 2;
  hi.ensure(bytes, c->counter());
  lo.ensure(bytes, c->counter());
  split_cderi_kernel<<<grid_for(naux * nao * ldk), 256, 0, c->stream>>>(c->Bd.as<double>(), nao, naux, ldk, sA,
                                                                       hi.as<__half>(), lo.as<__half>());
  count_launch(2);
  CPHF_CUDA(cudaGetLastError());
}

void tc_k_term1(cphf_ctx* c, const DevBuf& Bhi, const DevBuf& Blo, int64_t ldk, int64_t no, int64_t nb,
                float* out, DevBuf& Thi, DevBuf& Tlo, const TPlanes& tplanes) {
  LowpState& L = *c->lowp;
  const int64_t nao = c->nao, naux = c->naux;
  const int64_t N = no * nb;
  // aux functions per chunk: both T planes within the context's chunk budget, batched T
  // generation within grid limits
  int64_t np = std::max<int64_t>(1, L.budget / std::max<int64_t>(N * ldk * 4, 1));
  np = std::min<int64_t>(np, std::max<int64_t>(1, 65535 / std::max<int64_t>(nb, 1)));
  np = std::min<int64_t>(np, naux);
  const size_t plane = (size_t)np * N * ldk * 2;
  Thi.ensure(plane, c->counter());
  Tlo.ensure(plane, c->counter());
  // scale scratch: max |T| (float bits) and the two scale factors
  L.s_acc.ensure(64, c->counter());
  unsigned* mx = L.s_acc.as<unsigned>();
  float* scale = reinterpret_cast<float*>(mx + 4);
  L.err.ensure(sizeof(int), c->counter());
  const int m_tiles = (int)div_up(nao, BM), n_tiles = (int)div_up(N, BN);
  const int nkb = (int)div_up(nao, BK);
  const int ppc = 16;
  for (int64_t P0 = 0; P0 < naux; P0 += np) {
    const int64_t npc = std::min<int64_t>(np, naux - P0);
    // FP16 planes of T_P[nu, (i,a)] = sum_j bra[nu, j, a] O_P[j, i] and their scale from the
    // T generator (no FP32 T in HBM)
    tplanes(P0, npc, Thi.as<__half>(), Tlo.as<__half>(), mx, scale);
    const CUtensorMap mAh = make_map(Bhi.p, nao, nao, naux, ldk, BM);
    const CUtensorMap mAl = make_map(Blo.p, nao, nao, naux, ldk, BM);
    const CUtensorMap mBh = make_map(Thi.p, nao, N, npc, ldk, BN);
    const CUtensorMap mBl = make_map(Tlo.p, nao, N, npc, ldk, BN);
    TcArgs a;
    a.out = out;
    a.ld_out = nao;
    a.M = (int)nao;
    a.N = (int)N;
    a.nkb = nkb;
    a.np = (int)npc;
    a.p_per_cta = ppc;
    a.pA0 = (int)P0;
    a.m_tiles = m_tiles;
    a.scale = scale + 1;
    a.rowscale = nullptr;
    a.colscale = nullptr;
    a.err = L.err.as<int>();
    dim3 grid((unsigned)(m_tiles * n_tiles), (unsigned)div_up(npc, ppc));
    // algorithmic FLOPs of the contraction (the tensor pipe executes three split products);
    // bytes: the FP16 planes of both operands read once
    ProfScope ps(c, PROF_TC_KTERM, 2.0 * nao * N * nao * npc, 4.0 * nao * npc * (nao + N));
    tc_term1_kernel<<<grid, 128, SMEM_BYTES, c->stream>>>(mAh, mAl, mBh, mBl, a);
    count_launch();
    CPHF_CUDA(cudaGetLastError());
  }
}

void tc_planes_term(cphf_ctx* c, const __half* a_hi, const __half* a_lo, int64_t a_depth, int64_t a_off,
                    const __half* b_hi, const __half* b_lo, int64_t npc, int64_t M, int64_t N, int64_t K, int64_t ld,
                    const double* rowscale, const double* colscale, float* out, int64_t ld_out, int* err,
                    const float* scale) {
  if (M <= 0 || N <= 0 || K <= 0 || npc <= 0) return;
  const int m_tiles = (int)div_up(M, BM), n_tiles = (int)div_up(N, BN);
  const CUtensorMap mAh = make_map(a_hi, K, M, a_depth, ld, BM);
  const CUtensorMap mAl = make_map(a_lo, K, M, a_depth, ld, BM);
  const CUtensorMap mBh = make_map(b_hi, K, N, npc, ld, BN);
  const CUtensorMap mBl = make_map(b_lo, K, N, npc, ld, BN);
  TcArgs a;
  a.out = out;
  a.ld_out = ld_out;
  a.M = (int)M;
  a.N = (int)N;
  a.nkb = (int)div_up(K, BK);
  a.np = (int)npc;
  // one K range per tile unless the tiles alone leave SMs idle
  const int64_t tiles = (int64_t)m_tiles * n_tiles;
  const int64_t ranges = std::max<int64_t>(1, std::min<int64_t>(npc, div_up(2 * (int64_t)c->num_sms, tiles)));
  a.p_per_cta = (int)div_up(npc, ranges);
  a.pA0 = (int)a_off;
  a.m_tiles = m_tiles;
  a.scale = scale;
  a.rowscale = rowscale;
  a.colscale = colscale;
  a.err = err;
  dim3 grid((unsigned)tiles, (unsigned)div_up(npc, a.p_per_cta));
  tc_term1_kernel<<<grid, 128, SMEM_BYTES, c->stream>>>(mAh, mAl, mBh, mBl, a);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

void tc_wgen_planes(cphf_ctx* c, const __half* a_hi, const __half* a_lo, int64_t M, const __half* b_hi,
                    const __half* b_lo, int64_t b_rows, int64_t b_row0, int64_t N, int64_t K, int64_t ldk,
                    const int* e_row, const int* e_col, const float* wscale, int64_t no, int64_t ldj, int64_t s_a,
                    int64_t s_p, __half* out_hi, __half* out_lo, int* err) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  const int64_t last = (no - 1) + ldj * (no - 1) + s_a * ((M - 1) / no) + s_p * ((N - 1) / no);
  if (last >= (int64_t)INT32_MAX || b_row0 + N > (int64_t)INT32_MAX)
    throw Error(CPHF_ERR_ARG, "W generation: plane offsets exceed 32 bits");
  WgArgs a;
  a.out_hi = out_hi;
  a.out_lo = out_lo;
  a.M = (int)M;
  a.N = (int)N;
  a.nkb = (int)div_up(K, BK);
  a.m_tiles = (int)div_up(M, BM);
  a.n_tiles = (int)div_up(N, BN);
  a.group_m = std::min(a.m_tiles, 32);
  a.b_row0 = (int)b_row0;
  a.no = (int)no;
  a.ldj = (int)ldj;
  a.s_a = (int)s_a;
  a.s_p = (int)s_p;
  a.e_row = e_row;
  a.e_col = e_col;
  a.wscale = wscale;
  a.err = err;
  const CUtensorMap mAh = make_map(a_hi, K, M, 1, ldk, BM);
  const CUtensorMap mAl = make_map(a_lo, K, M, 1, ldk, BM);
  const CUtensorMap mBh = make_map(b_hi, K, b_rows, 1, ldk, BN);
  const CUtensorMap mBl = make_map(b_lo, K, b_rows, 1, ldk, BN);
  const int64_t tiles = (int64_t)a.m_tiles * a.n_tiles;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, c->num_sms);
  tc_wgen_kernel<<<grid, WG_THREADS, SMEM_BYTES, c->stream>>>(mAh, mAl, mBh, mBl, a);
  count_launch();
  CPHF_CUDA(cudaGetLastError());
}

}  // namespace cphf
