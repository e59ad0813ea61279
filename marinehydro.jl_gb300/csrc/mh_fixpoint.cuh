// mh_fixpoint.cuh -- polynomial evaluation in 64-bit fixed point on the integer pipe.
//
// GB300 executes FP64 at two lanes per SM per clock, against 64-128 for 32-bit integer and
// FP32 work, so the Wu wave term (hundreds of FP64 operations per panel pair) is bound by
// the FP64 pipe alone.  Its polynomials on bounded intervals -- the Liang-Wu-Noblesse fits
// in rho in [0, 1), the Struve fits, the Bessel interpolants -- need no floating point:
// with the variable as a 64-bit fraction z and the coefficients and partial sums as 64-bit
// integers v 2^-F, one Horner step is v <- c + floor(v z), a 64 x 64 -> high-64 integer
// multiply and an add, exact up to the one truncation of 2^-F.  With F = 44 (Wu fits,
// |partial sums| < 2^18) or 59-61 (Struve, Bessel) that truncation is below the FP64
// rounding of the same partial sums, so the results are at least as accurate as the FP64
// evaluation they replace.  Conversions between double and fixed point are done on the
// bits (exponent field, shifts, leading-zero count), also without the FP64 pipe.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mh {
namespace fx {

// round(c 2^frac) for a coefficient literal c (compile time; c 2^frac is exact in binary,
// |c 2^frac| < 2^62)
constexpr long long q(double c, int frac) {
  double s = c;
  for (int i = 0; i < frac; ++i) s *= 2.0;
  const double a = s < 0 ? -s : s;
  const long long r = a >= 4503599627370496.0 ? (long long)a : (long long)(a + 0.5);  // 2^52
  return s < 0 ? -r : r;
}

// floor(v t / 2^64): signed v, unsigned fraction t (the high word of the 128-bit product;
// for v < 0 the unsigned product of v + 2^64 is t too large)
__device__ __forceinline__ long long mulhi_su(long long v, unsigned long long t) {
  const unsigned long long h = __umul64hi((unsigned long long)v, t);
  return (long long)(h - (v < 0 ? t : 0ull));
}

// floor(x 2^64) for x in [0, 1) (0 below 2^-1022)
__device__ __forceinline__ unsigned long long unit_q64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0ull;
  const unsigned long long m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - 1011;  // x 2^64 = m 2^(e - 1075 + 64)
  return sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
}

// floor(x 2^63) for x in [0, 1] (x = 1 included; 0 below 2^-1022): Horner steps with this
// fraction take z = x / 2, so coefficient i carries a factor 2^i
__device__ __forceinline__ unsigned long long unit_q63(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0ull;
  const unsigned long long m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - 1012;
  return sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
}

// trunc(x 2^s) as a signed integer, for |x| 2^s < 2^62 (0 below 2^-1022)
__device__ __forceinline__ long long to_q(double x, int s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0ll;
  const unsigned long long m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - 1075 + s;
  const unsigned long long a = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
  return (b >> 63) ? -(long long)a : (long long)a;
}

// v 2^-frac as a double, rounded to nearest (ties away from zero); |v| < 2^63, results
// below the normal range flush to zero
__device__ __forceinline__ double to_double(long long v, int frac) {
  const unsigned long long sign = (unsigned long long)v & 0x8000000000000000ull;
  unsigned long long m = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int msb = 63 - __clzll(m);
  long long e = (long long)msb - frac + 1023;
  if (msb > 52) {
    const int sh = msb - 52;
    m = (m + (1ull << (sh - 1))) >> sh;
    if (m >> 53) { m >>= 1; ++e; }
  } else {
    m <<= (52 - msb);
  }
  const unsigned long long bits = sign | ((unsigned long long)e << 52) | (m & 0x000FFFFFFFFFFFFFull);
  return (v == 0 || e <= 0) ? 0.0 : __longlong_as_double((long long)bits);
}

// sum_i c[i] t^i for t in [0, 1) as unit_q64(t); coefficients and result v 2^-F
template <int N>
__device__ __forceinline__ long long horner_u(const long long (&c)[N], unsigned long long t) {
  long long v = c[N - 1];
#pragma unroll
  for (int i = N - 2; i >= 0; --i) v = c[i] + mulhi_su(v, t);
  return v;
}

// sum_i c[i] z^i for z in [-1/2, 1/2) given as z 2^64 (coefficients in a constant bank or
// registers)
template <int N>
__device__ __forceinline__ long long horner_s(const long long (&c)[N], long long z) {
  long long v = c[N - 1];
#pragma unroll
  for (int i = N - 2; i >= 0; --i) v = c[i] + __mul64hi(v, z);
  return v;
}

// the same with the coefficients read from global memory (a row of a table)
template <int N>
__device__ __forceinline__ long long horner_s_ld(const long long* __restrict__ c, long long z) {
  long long v = __ldg(c + N - 1);
#pragma unroll
  for (int i = N - 2; i >= 0; --i) v = __ldg(c + i) + __mul64hi(v, z);
  return v;
}

}  // namespace fx
}  // namespace mh
