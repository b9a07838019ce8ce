// Natural logarithm of an f32 that returns the same bits on the host and on
// the GPU.
//
// ConstantMedium::hit draws its free-flight distance as ln(U) / -density
// (clovers/src/objects/constant_medium.rs:102).  Library logf routines (CUDA's
// and the host libm's) are each accurate to about an ulp but round the last
// bit differently, which moves a medium hit between a GPU ray cast and the CPU
// oracle.  This routine evaluates ln(x) in IEEE double with a fixed sequence of
// correctly rounded + - * / operations and rounds once to f32; compiled with
// -fmad=false (GPU) and -ffp-contract=off (host) it gives identical results on
// both.  The double result is within a few double ulp of ln(x), so the f32
// result is within 0.5 ulp (+ 2^-27 ulp) of ln(x): correctly rounded except in
// rare near-halfway cases, and inside the 1-ulp bound CUDA states for logf.
//
// Method (argument reduction and the atanh series; e.g. J.-M. Muller,
// "Elementary Functions: Algorithms and Implementation", the chapter on
// logarithms): x = m 2^e with m in [sqrt(1/2), sqrt(2)), s = (m - 1)/(m + 1),
// ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), ln x = e ln 2 + ln m.
// |s| <= 3 - 2 sqrt(2) < 0.1716, so s^2 < 0.0295 and ten terms leave a
// truncation error below 2^-55 relative.  The coefficients are 2/(2k+1)
// rounded to the nearest double, written as hexadecimal literals so that both
// compilers read the same values.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define CLV_LOG_HD __host__ __device__ __forceinline__
#else
#define CLV_LOG_HD inline
#endif

namespace clv_math {

CLV_LOG_HD uint64_t log_bits_of(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
CLV_LOG_HD double log_double_of(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
CLV_LOG_HD float log_float_of(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, 4);
  return x;
#endif
}

// ln(x) for an f32 x: -inf at 0, NaN below 0 or for NaN, +inf at +inf.
CLV_LOG_HD float log_f32(float xf) {
  if (!(xf > 0.0f)) return xf == 0.0f ? log_float_of(0xFF800000u) : log_float_of(0x7FC00000u);
  if (xf > 3.40282347e+38f) return xf;  // +inf
  // x is finite and positive; as a double it is normal (f32 subnormals included)
  const uint64_t b = log_bits_of((double)xf);
  int e = (int)((b >> 52) & 0x7FF) - 1023;
  double m = log_double_of((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);  // [1, 2)
  if (m > 0x1.6a09e667f3bcdp+0) {  // sqrt(2): halve (exact) so that m < sqrt(2)
    m = m * 0.5;
    e = e + 1;
  }
  const double s = (m - 1.0) / (m + 1.0);  // m - 1 is exact (Sterbenz)
  const double z = s * s;
  double p = 0x1.af286bca1af28p-4;  // 2/19
  p = p * z + 0x1.e1e1e1e1e1e1ep-4;  // 2/17
  p = p * z + 0x1.1111111111111p-3;  // 2/15
  p = p * z + 0x1.3b13b13b13b14p-3;  // 2/13
  p = p * z + 0x1.745d1745d1746p-3;  // 2/11
  p = p * z + 0x1.c71c71c71c71cp-3;  // 2/9
  p = p * z + 0x1.2492492492492p-2;  // 2/7
  p = p * z + 0x1.999999999999ap-2;  // 2/5
  p = p * z + 0x1.5555555555555p-1;  // 2/3
  p = p * z + 2.0;
  const double lnm = s * p;
  const double ln2 = 0x1.62e42fefa39efp-1;  // ln 2 rounded to the nearest double
  return (float)((double)e * ln2 + lnm);
}

}  // namespace clv_math
