// swc_fpconv.h -- FP32 <-> FP64 conversions built from integer operations.
//
// On GB300 the FP64 pipe (which also executes the F2F conversions between FP32 and
// FP64) issues about 2 operations per clock per SM, 1/64 of the FP32 rate, so in the
// mixed engine's memory-bound passes the conversions, not the memory, set the time.
// Both formats are IEEE-754 binary: a conversion between normal numbers re-biases the
// exponent (127 <-> 1023) and shifts the mantissa (23 <-> 52 bits), which the integer
// pipes do at full rate. Zeros are handled too; subnormal, infinite and NaN operands
// (never met on the engine's hot paths) take the hardware conversion, so the result
// is always the one the cast gives: exact for widening, round-to-nearest-even for
// narrowing. Host builds (the unit test) use the same arithmetic through memcpy. The
// FP64 reciprocal at the end builds on them.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SWC_HD __host__ __device__ __forceinline__
#else
#define SWC_HD inline
#endif

namespace swc {

SWC_HD uint32_t f32_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
SWC_HD float f32_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}
SWC_HD void f64_words(double x, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  hi = (uint32_t)__double2hiint(x);
  lo = (uint32_t)__double2loint(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  hi = (uint32_t)(u >> 32);
  lo = (uint32_t)u;
#endif
}
SWC_HD double f64_from_words(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t u = ((uint64_t)hi << 32) | lo;
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

// The hardware conversions for the rare operands, as volatile asm on the device so the
// compiler keeps them behind their branch instead of executing them speculatively.
SWC_HD double widen_slow(float x) {
#if defined(__CUDA_ARCH__)
  double d;
  asm volatile("cvt.f64.f32 %0, %1;" : "=d"(d) : "f"(x));
  return d;
#else
  return (double)x;
#endif
}
SWC_HD float narrow_slow(double x) {
#if defined(__CUDA_ARCH__)
  float f;
  asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(x));
  return f;
#else
  return (float)x;
#endif
}

// Exact FP32 -> FP64.
SWC_HD double widen_f32(float x) {
  const uint32_t u = f32_bits(x);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e != 0u && e != 0xffu) {  // normal: exponent bias 127 -> 1023, mantissa 23 -> 52 bits
    const uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return f64_from_words(hi, (u & 0x7u) << 29);
  }
  if ((u & 0x7fffffffu) == 0u) return f64_from_words(u, 0u);  // +-0
  return widen_slow(x);
}

// FP64 -> FP32, round to nearest, ties to even.
SWC_HD float narrow_f64(double x) {
  uint32_t hi, lo;
  f64_words(x, hi, lo);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e >= 897u && e <= 1150u) {  // the result's biased exponent e - 896 is in [1, 254]
    const uint32_t m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1fffffffu;  // the 29 dropped mantissa bits
    uint32_t base = ((e - 896u) << 23) | m23;
    base += (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) ? 1u : 0u;  // a carry may reach infinity
    return f32_from_bits((hi & 0x80000000u) | base);
  }
  if ((hi & 0x7fffffffu) == 0u && lo == 0u) return f32_from_bits(hi);  // +-0
  return narrow_slow(x);
}

// 1/x in FP64 by Newton-Raphson iteration for the reciprocal, r <- r + r (1 - x r):
// each step squares the seed's relative error, and the error term 1 - x r and the
// update are one fused multiply-add each. From a seed within 2^-20 of 1/x, two steps
// leave FP64's own rounding (within an ulp of 1/x): four FP64 FMAs.
SWC_HD double rcp_f64_from_seed(double x, double r) {
#if defined(__CUDA_ARCH__)
  double t = __fma_rn(-x, r, 1.0);
  r = __fma_rn(r, t, r);
  t = __fma_rn(-x, r, 1.0);
  return __fma_rn(r, t, r);
#else
  double t = __builtin_fma(-x, r, 1.0);
  r = __builtin_fma(r, t, r);
  t = __builtin_fma(-x, r, 1.0);
  return __builtin_fma(r, t, r);
#endif
}

// 1/x for an FP64 x of either sign whose magnitude lies within FP32's normal range
// with a margin (2^-124 .. 2^124): the seed is FP32's reciprocal of x narrowed on the
// integer pipes (on the device the approximate reciprocal, within 2 ulp: about 2^-21
// with the narrowing), widened back, then two Newton-Raphson steps. Other x (zero,
// tiny, huge, non-finite) take the IEEE division. On GB300, whose FP64 pipe runs at
// 1/64 of the FP32 rate, this is fewer FP64 operations than the IEEE division's
// sequence; the result is within an ulp of it, not always the same bits.
SWC_HD double rcp_f64(double x) {
  uint32_t hi, lo;
  f64_words(x, hi, lo);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e < 899u || e > 1147u) return 1.0 / x;
  const float xf = narrow_f64(x);
#if defined(__CUDA_ARCH__)
  const float sf = __fdividef(1.0f, xf);
#else
  const float sf = 1.0f / xf;
#endif
  return rcp_f64_from_seed(x, widen_f32(sf));
}

}  // namespace swc
