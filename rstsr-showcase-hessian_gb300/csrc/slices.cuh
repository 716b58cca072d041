// Operand representations of the tensor-core contractions and their slicing primitives
// (integer arithmetic on the FP64 / FP32 bit patterns), shared by the K-term kernels
// (tc_ozaki.cu) and the XC response (xc_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <type_traits>

namespace cphf {

// Operand representations: exact BF16 slices (FP64-accurate residual) and split FP16 hi/lo
// (the inner solves' operator).  EOFF: exponent offset of the stored planes (x 2^(EOFF - e)).
struct Exact6 {
  static constexpr int S = 6, NACC = 4, EOFF = 0, STAGES = 2;
  static constexpr bool BF16 = true;
  using Elem = __nv_bfloat16;
};
// The same exact BF16 slice planes read in correction precision: only slices 0 .. NS-1 of each
// operand and the products with t + u <= NS - 1, for operators applied to a small correction
// whose result only has to be accurate relative to the correction itself.  NS = 4: 10
// products, each operand cut at 2^-25 of its row / column maximum, dropped products below
// 2^-23 of the maxima's product; NS = 3: 6 products, 2^-19 and 2^-17.  Same planes, same exact
// accumulation bounds; with NS = 3 the fourth accumulator stays unused.
template <int NS>
struct ExactC {
  // split-K stages of 16 KB per plane pair: 3 x 64 KB (NS = 4) or 4 x 48 KB (NS = 3), so the
  // fewer products per stage still cover the loads' latency
  static constexpr int S = NS, NACC = 4, EOFF = 0, STAGES = NS == 3 ? 4 : 3;
  static constexpr bool BF16 = true;
  using Elem = __nv_bfloat16;
};
using Exact6c = ExactC<4>;
using Exact6c3 = ExactC<3>;
struct Split2 {
  static constexpr int S = 2, NACC = 1, EOFF = 14, STAGES = 6;
  static constexpr bool BF16 = false;
  using Elem = __half;
};

// ---- slicing (integer arithmetic on the bit patterns; the FP64 pipe is not used) ----------
// |x| as an ordered integer key (non-negative floats order like their bit patterns)
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long abs_key(float2 x) {
  return (unsigned long long)(__float_as_uint(x.x) & 0x7FFFFFFFu);
}
__device__ __forceinline__ unsigned long long abs_key(float x) {
  return (unsigned long long)(__float_as_uint(x) & 0x7FFFFFFFu);
}
template <class T>
__host__ __device__ constexpr bool float_key() { return !std::is_same<T, double>::value; }

// round(x 2^k) for |x| 2^k <= 2^36, from the FP64 bit pattern
__device__ __forceinline__ long long fix_round(double x, int k, bool& bad) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((bits >> 52) & 0x7FF);
  if (E == 0x7FF) { bad = true; return 0; }
  const long long M = E ? (long long)((bits & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : (long long)(bits & 0xFFFFFFFFFFFFFull);
  const int sh = 1075 - k - (E ? E : 1);  // x = M 2^(E - 1075)
  long long F = 0;
  if (sh <= 0) F = M << min(-sh, 10);
  else if (sh < 63) F = (M + (1ll << (sh - 1))) >> sh;
  return (bits >> 63) ? -F : F;
}
// same from the FP32 bit pattern
__device__ __forceinline__ long long fix_round(float x, int k, bool& bad) {
  const unsigned bits = __float_as_uint(x);
  const int E = (int)((bits >> 23) & 0xFF);
  if (E == 0xFF) { bad = true; return 0; }
  const long long M = E ? (long long)((bits & 0x7FFFFFu) | 0x800000u) : (long long)(bits & 0x7FFFFFu);
  const int sh = 150 - k - (E ? E : 1);   // x = M 2^(E - 150)
  long long F = 0;
  if (sh <= 0) F = M << min(-sh, 40);
  else if (sh < 63) F = (M + (1ll << (sh - 1))) >> sh;
  return (bits >> 31) ? -F : F;
}

// F = round(v 2^36), |F| <= 2^36, into the six digits q_t = round(R_t / 2^(30 - 6t)) of the
// running remainder, written as BF16 slices q_t 2^(-6(t+1)) (plane stride `plane`).
// NS < 6 writes only the leading NS digits (the planes a correction-precision product reads).
template <int NS = 6>
__device__ __forceinline__ void digits6(long long F, bool bad, __nv_bfloat16* dst, int64_t plane) {
  long long R = F;
#pragma unroll
  for (int t = 0; t < NS; ++t) {
    const int s = 30 - 6 * t;
    const long long q = s > 0 ? ((R + (1ll << (s - 1))) >> s) : R;
    R -= q << s;
    float v = (float)(int)q * __int_as_float((127 - 6 * (t + 1)) << 23);  // q 2^(-6(t+1)), exact
    if (bad) v = __int_as_float(0x7FC00000);                                // NaN / Inf propagate as NaN
    dst[t * plane] = __float2bfloat16_rn(v);
  }
}
template <int NS = 6>
__device__ __forceinline__ void slice6(double x, int e, __nv_bfloat16* dst, int64_t plane) {
  bool bad = false;
  const long long F = fix_round(x, 36 - e, bad);
  digits6<NS>(F, bad, dst, plane);
}
// Digits of an FP32 pair v = hi + lo (|v| < 2^e) in FP32 arithmetic, into d[0 .. NS): the
// balanced base-64 digits of F ~ v 2^(36 - e) (|F - v 2^(36 - e)| <= 1/2 + 2^-6), the same
// representation as the integer path above at a fraction of its instructions.  The scale
// comes as two normal powers of two f1 f2 = 2^(36 - e), so that no ldexpf is needed.  The high
// part alone gives the first three digits: its remainders r = r - q 2^s stay exact (multiples
// of its ulp with at most 24 significant bits); the low part (below the high part's ulp) joins
// once the remainder is below 2^17, where their sum keeps 2^-6 resolution; q_t = rint(r 2^-s)
// is balanced, |q_0| <= 64, |q_t| <= 32.
template <int NS>
__device__ __forceinline__ void digits_pair(float hi, float lo, float f1, float f2, float* d) {
  const bool bad = !isfinite(hi) || !isfinite(lo);
  float r = (hi * f1) * f2;
  const float l = (lo * f1) * f2;
#pragma unroll
  for (int t = 0; t < NS; ++t) {
    if (t == 3) r += l;
    const int sh = 30 - 6 * t;
    const float q = rintf(r * __int_as_float((127 - sh) << 23));  // r 2^-sh
    r = fmaf(-q, __int_as_float((127 + sh) << 23), r);
    d[t] = bad ? __int_as_float(0x7FC00000) : q * __int_as_float((127 - 6 * (t + 1)) << 23);
  }
}

// store one element's planes: exact BF16 slices, or split FP16 hi/lo of x 2^(14 - e)
template <class PR>
struct Put;
template <>
struct Put<Exact6> {
  template <class T>
  __device__ static void put(T x, int e, __nv_bfloat16* dst, int64_t plane) { slice6(x, e, dst, plane); }
};
template <int NS>
struct Put<ExactC<NS>> {  // only the planes a correction-precision product reads
  __device__ static void put(double x, int e, __nv_bfloat16* dst, int64_t plane) { slice6<NS>(x, e, dst, plane); }
};
template <>
struct Put<Split2> {
  __device__ static void put(float x, int e, __half* dst, int64_t plane) {
    const float v = ldexpf(x, Split2::EOFF - e);
    const __half h = __float2half_rn(v);
    dst[0] = h;
    dst[plane] = __float2half_rn(v - __half2float(h));
  }
};

// power of two strictly above max |x| (exponent e with max = f 2^e, f in [0.5, 1)); 0 for zero
__device__ __forceinline__ int key_exp(unsigned long long key, bool is_float) {
  if (is_float) {
    const int E = (int)((key >> 23) & 0xFF);
    if (key == 0 || E == 0xFF) return 0;
    int e;
    frexpf(__uint_as_float((unsigned)key), &e);
    return e;
  }
  const int E = (int)((key >> 52) & 0x7FF);
  if (key == 0 || E == 0x7FF) return 0;
  int e;
  frexp(__longlong_as_double((long long)key), &e);
  return e;
}

}  // namespace cphf
