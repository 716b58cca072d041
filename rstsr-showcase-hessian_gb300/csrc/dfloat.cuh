// Double-float arithmetic shared by the FP64-accurate SIMT GEMMs (gemm_simt.cu) and the
// grouped XC GEMMs (xc_grouped.cu).
#pragma once
#include <cuda_runtime.h>

namespace cphf {

// Double-float number for FP64-accurate products on the FP32 pipes.  A value is hi + lo
// (two floats).  The product of two such numbers keeps ah*bh exactly (FMA error term) plus
// the cross terms ah*bl + al*bh; accumulation is compensated summation (error-free
// two-sum of the high parts, Ogita-Rump-Oishi Dot2), so a K-term dot product carries
// about 2^-48 relative error per term instead of FP32's 2^-24.  Doubles are split with
// integer operations (no FP64 instruction per element).
struct dfloat {
  float hi, lo;
  dfloat() = default;
  __device__ __forceinline__ dfloat(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit dfloat(int v) : hi((float)v), lo(0.f) {}
  __device__ __forceinline__ explicit dfloat(double x) {
    const unsigned int h32 = (unsigned int)__double2hiint(x), l32 = (unsigned int)__double2loint(x);
    const unsigned int sign = h32 & 0x80000000u;
    const int e = (int)((h32 >> 20) & 0x7FFu);
    const int E = e - 1023 + 127;  // float biased exponent of hi
    if (e == 0 || E <= 0) {        // zero, or below the normal float range (|x| < 2^-126): negligible here
      hi = 0.f;
      lo = 0.f;
      return;
    }
    if (E >= 255) {  // beyond the float range: let it propagate as infinity
      hi = __int_as_float((int)(sign | 0x7F800000u));
      lo = 0.f;
      return;
    }
    const unsigned int mant23 = ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
    hi = __int_as_float((int)(sign | ((unsigned)E << 23) | mant23));
    // remaining 29 mantissa bits: value r * 2^(e - 1075)
    const unsigned int r = l32 & 0x1FFFFFFFu;
    const int El = e - 1075 + 127;
    if (r == 0u || El <= 0) {
      lo = 0.f;
    } else {
      const float rf = __uint2float_rn(r) * __int_as_float(El << 23);
      lo = sign ? -rf : rf;
    }
  }
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ bool operator!=(const dfloat& o) const { return hi != o.hi || lo != o.lo; }
  __device__ __forceinline__ dfloat& operator+=(const dfloat& b) {
    const float s = hi + b.hi;
    const float z = s - hi;
    const float t = (hi - (s - z)) + (b.hi - z);
    hi = s;
    lo = lo + (t + b.lo);
    return *this;
  }
};

__device__ __forceinline__ dfloat madd(const dfloat& a, const dfloat& b, const dfloat& c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = c.hi + p;
  const float z = s - c.hi;
  const float t = (c.hi - (s - z)) + (p - z);
  return dfloat(s, c.lo + (t + e));
}

__device__ __forceinline__ dfloat operator*(const dfloat& a, const dfloat& b) { return madd(a, b, dfloat(0)); }
__device__ __forceinline__ double madd(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ float madd(float a, float b, float c) { return fmaf(a, b, c); }

}  // namespace cphf
