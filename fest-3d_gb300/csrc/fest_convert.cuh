// fest_convert.cuh - FP32 <-> FP64 conversions in integer arithmetic, for
// the mixed-precision sweep.  GB300 converts between FP32 and FP64 in its
// FP64 unit, which runs at a small fraction of the FP32 rate; these do the
// same with integer operations.  f2d is exact for normal numbers, zero,
// infinities and NaN (FP32 subnormals, below 1.2e-38, become zero); d2f
// rounds to nearest even like a conversion instruction for results in the
// normal FP32 range (results below it become signed zero).  Host and
// device: the host build exists so that the CPU tests can check them
// against the compiler's conversions.
#pragma once
#include <cuda_runtime.h>
#include <string.h>

namespace fest {

__host__ __device__ __forceinline__ unsigned f32_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}
__host__ __device__ __forceinline__ float f32_from(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}
__host__ __device__ __forceinline__ double f64_from(unsigned hi, unsigned lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const unsigned long long b = ((unsigned long long)hi << 32) | lo;
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}
__host__ __device__ __forceinline__ void f64_words(double x, unsigned& hi, unsigned& lo) {
#ifdef __CUDA_ARCH__
  hi = (unsigned)__double2hiint(x);
  lo = (unsigned)__double2loint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof b);
  hi = (unsigned)(b >> 32);
  lo = (unsigned)b;
#endif
}

__host__ __device__ __forceinline__ double f2d(float x) {
  const unsigned u = f32_bits(x);
  const unsigned e = (u >> 23) & 0xffu, s = u & 0x80000000u, m = u & 0x7fffffu;
  unsigned hi = s, lo = 0u;
  if (e == 0xffu) { hi = s | 0x7ff00000u | (m >> 3); lo = m << 29; }
  else if (e != 0u) { hi = s | ((e + 896u) << 20) | (m >> 3); lo = m << 29; }
  return f64_from(hi, lo);
}
__host__ __device__ __forceinline__ float d2f(double x) {
  unsigned hi, lo;
  f64_words(x, hi, lo);
  const unsigned s = hi & 0x80000000u, ed = (hi >> 20) & 0x7ffu;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;  // the 29 bits dropped
  if (ed == 0x7ffu) return f32_from(s | 0x7f800000u | (mant != 0u || rest != 0u ? 0x400000u : 0u));
  const int e = (int)ed - 896;  // FP32 biased exponent
  if (e <= 0) return f32_from(s);
  if (e >= 255) return f32_from(s | 0x7f800000u);
  unsigned bits = s | ((unsigned)e << 23) | mant;
  bits += (rest > 0x10000000u || (rest == 0x10000000u && (mant & 1u))) ? 1u : 0u;  // may carry into inf
  return f32_from(bits);
}

}  // namespace fest
