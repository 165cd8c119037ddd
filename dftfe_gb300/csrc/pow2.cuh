// Exact scaling by powers of two and FP32 -> FP64 widening done on the bit patterns
// (IEEE 754 binary32 / binary64 layouts), so that streaming passes stay off the FP64 pipe:
// GB300 issues about two FP64 FMAs per clock per SM, and one FP64 multiply per entry of a
// 1.7e9-entry block costs ~2.8 ms, more than the block's bytes take at HBM speed.
// Zeros take a fast path; subnormal, infinite and NaN inputs and results outside the normal
// range fall back to ldexp, so every helper returns exactly x * 2^k rounded once.
#pragma once

#include <cstdint>

namespace chefsi {

// The rare cases run out of line behind a branch: inlined, the compiler evaluates them for
// every entry under a predicate, on the FP64 pipe.
static __device__ __noinline__ double ldexp_slow(double x, int k) { return ldexp(x, k); }
static __device__ __noinline__ float ldexpf_slow(float x, int k) {
  return static_cast<float>(ldexp(static_cast<double>(x), k));
}

// x * 2^k (exact when the result is a normal double)
__device__ __forceinline__ double ldexp_exact(double x, int k) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
  if ((u << 1) == 0) return x;  // +-0
  const int e = static_cast<int>((u >> 52) & 0x7ff);
  const int ne = e + k;
  if (__builtin_expect(e == 0 || e == 0x7ff || ne <= 0 || ne >= 0x7ff, 0)) return ldexp_slow(x, k);
  return __longlong_as_double(
      static_cast<long long>((u & 0x800fffffffffffffull) | (static_cast<unsigned long long>(ne) << 52)));
}

// x * 2^k rounded to FP32 once (equals (float)((double)x * 2^k))
__device__ __forceinline__ float ldexpf_exact(float x, int k) {
  const uint32_t u = __float_as_uint(x);
  if ((u << 1) == 0) return x;
  const int e = static_cast<int>((u >> 23) & 0xff);
  const int ne = e + k;
  if (__builtin_expect(e == 0 || e == 0xff || ne <= 0 || ne >= 0xff, 0)) return ldexpf_slow(x, k);
  return __uint_as_float((u & 0x807fffffu) | (static_cast<uint32_t>(ne) << 23));
}

// (double)x * 2^k, exact: the FP32 exponent is re-biased (1023 - 127 = 896) and the 23
// mantissa bits move to the top of the 52
__device__ __forceinline__ double widen_ldexp(float x, int k) {
  const uint32_t u = __float_as_uint(x);
  const unsigned long long sign = static_cast<unsigned long long>(u >> 31) << 63;
  if ((u << 1) == 0) return __longlong_as_double(static_cast<long long>(sign));
  const int e = static_cast<int>((u >> 23) & 0xff);
  const int ne = e + 896 + k;
  if (__builtin_expect(e == 0 || e == 0xff || ne <= 0 || ne >= 0x7ff, 0))
    return ldexp_slow(static_cast<double>(x), k);
  return __longlong_as_double(static_cast<long long>(
      sign | (static_cast<unsigned long long>(ne) << 52) | (static_cast<unsigned long long>(u & 0x7fffffu) << 29)));
}

static __device__ __noinline__ float narrow_slow(double x, int k) {
  return static_cast<float>(ldexp(x, k));
}

// (float)(x * 2^k), one rounding. When x and x 2^k both lie in FP32's normal range
// (unbiased exponent in [-125, 126]), rounding commutes with the scaling: f = fp32(x) is a
// normal FP32 of exponent e or e + 1 and f 2^k is the exponent field plus k. Everything else
// (zeros, subnormal or out-of-range values) takes the exact out-of-line path.
__device__ __forceinline__ float narrow_ldexp(double x, int k) {
  const int e = ((__double2hiint(x) >> 20) & 0x7ff) - 1023;
  const float f = __double2float_rn(x);
  if (__builtin_expect(e < -125 || e > 126 || e + k < -125 || e + k > 126, 0)) {
    if ((static_cast<unsigned long long>(__double_as_longlong(x)) << 1) == 0) return f;  // +-0
    return narrow_slow(x, k);
  }
  return __uint_as_float(__float_as_uint(f) + (static_cast<uint32_t>(k) << 23));
}

// |x| as an order-preserving integer key (non-negative doubles order like their bit patterns)
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull;
}

}  // namespace chefsi
