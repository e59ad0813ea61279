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
// bits (exponent field, shifts, leading-zero count), also without the FP64 pipe; so are the
// reciprocal, exp and log below.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mh_special_tables.cuh"

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

// 1/x for a normal x > 0, on the integer pipe: the FP32 reciprocal (one MUFU operation) of
// the leading 24 mantissa bits as the seed, two Newton steps y <- y (2 - m y) in 64-bit fixed
// point (mantissa m in [1, 2) as m 2^63, y in (1/2, 1) as y 2^64; the seed's 2^-22 error
// squares to below the fixed point's 2^-62), rounded to 53 bits: within one ulp of the
// correctly rounded quotient, without the FP64 pipe.  x = 0 gives +inf, as 1.0 / 0.0 does.
__device__ __forceinline__ double recip(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long frac = b & 0x000FFFFFFFFFFFFFull;
  if (e == 0) return __longlong_as_double(0x7FF0000000000000ll);
  if (frac == 0) return __longlong_as_double((long long)((unsigned long long)(2046 - e) << 52));  // 2^(1023 - e)
  const unsigned long long M = (frac | (1ull << 52)) << 11;
  float yf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(__int_as_float(0x3F800000 | (int)(frac >> 29))));
  const unsigned int yb = __float_as_uint(yf);  // in [1/2 - 2^-24, 1]
  unsigned long long Y = yb >= 0x3F800000u
                             ? ~0ull
                             : (unsigned long long)((yb & 0x7FFFFFu) | 0x800000u) << (40 + (int)(yb >> 23) - 126);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const unsigned long long E = 0ull - __umul64hi(M, Y);  // (2 - m y) 2^63
    Y = __umul64hi(Y, E) << 1;                             // y (2 - m y) 2^64 <= 2^64 / m
  }
  const int p = 63 - __clzll(Y);  // 62 or 63
  const int sh = p - 52;
  unsigned long long mant = (Y >> sh) + ((Y >> (sh - 1)) & 1ull);
  int ex = p + 1982 - e;  // 1/x = (Y 2^-64) 2^(1023 - e)
  if (mant >> 53) { mant >>= 1; ++ex; }
  if (ex <= 0) return 0.0;
  return __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0x000FFFFFFFFFFFFFull)));
}

// e^x for x <= 0 on the integer pipe (0 for x <= -745.25 and where the result is below the
// normal range).  y = x log2(e) from a 128-bit product of x 2^s (s = 60 for |x| < 8, else
// 53: exact) and log2(e) 2^63, so y's fraction f carries 64 bits; 2^f = 2^(j/32) 2^(g/32)
// with j the top five bits of f, 2^(g/32) a degree-7 series and both factors as integers
// c 2^62 (tables fxq); relative error below 3e-17 before the final rounding (emulated bit
// for bit against mpmath by gen_special_tables.py).
__device__ __forceinline__ double exp_nonpos(double x) {
  const unsigned long long ax = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  if (ax >= 0x40874A0000000000ull) return 0.0;  // |x| >= 745.25
  const int s = ax < 0x4020000000000000ull ? 60 : 53;  // |x| < 8
  const long long X = to_q(x, s);
  const long long hi = mulhi_su(X, fxq::kLog2eQ63);
  const unsigned long long lo = (unsigned long long)X * fxq::kLog2eQ63;
  const long long n = hi >> (s - 1);  // floor(y)
  const unsigned long long F = ((unsigned long long)hi << (65 - s)) | (lo >> (s - 1));  // frac(y) 2^64
  const int j = (int)(F >> 59);
  const unsigned long long G = F << 5;
  long long v = fxq::kExp2Poly[fxq::kExpDeg];
#pragma unroll
  for (int i = fxq::kExpDeg - 1; i >= 0; --i) v = fxq::kExp2Poly[i] + mulhi_su(v, G);
  const long long R = (long long)__umul64hi((unsigned long long)__ldg(fxq::kExp2Tab + j), (unsigned long long)v);
  return to_double(R, 60 - (int)n);  // R = 2^f 2^60
}

// log(w) for a normal w > 0 on the integer pipe (-inf for 0): w = m 2^n, m in [1, 2);
// n ln 2 + log(m) with log(m) from a degree-10 interpolant on the 1/32-interval of m (table
// fxq::kLogTab, c 2^62), summed as a 128-bit integer in units of 2^-64 and rounded to 2^-53:
// absolute error below 8e-17, which is what the Wu term needs (log enters as
// log(...) + gamma - 2 dd^2).
__device__ __forceinline__ double log_pos(double w) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(w);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return __longlong_as_double((long long)0xFFF0000000000000ull);
  const unsigned long long frac = b & 0x000FFFFFFFFFFFFFull;
  const long long* __restrict__ row = fxq::kLogTab + (int)(frac >> 47) * fxq::kLogTerms;
  const unsigned long long U = frac << 17;
  long long v = __ldg(row + fxq::kLogTerms - 1);
#pragma unroll
  for (int i = fxq::kLogTerms - 2; i >= 0; --i) v = __ldg(row + i) + mulhi_su(v, U);
  // n ln2 2^64 + v 2^2 as a signed 128-bit (hi, lo), |total| < 2^74
  const long long nn = e - 1023;
  long long hi = mulhi_su(nn, fxq::kLn2Q64);
  unsigned long long lo = (unsigned long long)nn * fxq::kLn2Q64;
  const unsigned long long add = (unsigned long long)(v << 2);
  const unsigned long long lo2 = lo + add;
  hi += (v < 0 ? -1 : 0) + (lo2 < lo ? 1 : 0);
  // round to 2^-53 and convert (|total 2^-11| < 2^63)
  const unsigned long long lo3 = lo2 + 1024ull;
  hi += lo3 < lo2 ? 1 : 0;
  const long long q = (long long)(((unsigned long long)hi << 53) | (lo3 >> 11));
  return to_double(q, 53);
}

// sqrt(x) for x >= 0 on the integer pipe (0 for x below the normal range): x = m 2^(2h),
// m in [1, 4); the FP32 reciprocal square root (one MUFU operation) of m's leading bits as
// the seed, two Newton steps y <- y (3 - m y^2) / 2 in 64-bit fixed point (m 2^62, y 2^63),
// then sqrt(m) = m y rounded to 53 bits: within one ulp of the correctly rounded root.
__device__ __forceinline__ double sqrt_pos(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0.0;
  const unsigned long long frac = b & 0x000FFFFFFFFFFFFFull;
  const int odd = (e - 1023) & 1;  // the exponent made even: m = 1.f 2^odd
  const unsigned long long M = ((frac | (1ull << 52)) << 9) << odd;  // m 2^61 (m < 4: < 2^63)
  float yf;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(__int_as_float(((127 + odd) << 23) | (int)(frac >> 29))));
  const unsigned int yb = __float_as_uint(yf);  // in (1/2 - 2^-22, 1 + 2^-22)
  unsigned long long Y = yb >= 0x3F800000u
                             ? (1ull << 63)
                             : (unsigned long long)((yb & 0x7FFFFFu) | 0x800000u) << (40 + (int)(yb >> 23) - 126 - 1);
  const unsigned long long M62 = M << 1;  // m 2^62 (< 2^64)
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const unsigned long long Y2 = __umul64hi(Y, Y);        // y^2 2^62
    const unsigned long long T = __umul64hi(M62, Y2);      // m y^2 2^60
    const unsigned long long E = 3ull * (1ull << 60) - T;   // (3 - m y^2) 2^60
    Y = __umul64hi(Y, E) << 3;                             // y (3 - m y^2) / 2  2^63
  }
  const unsigned long long S = __umul64hi(M62, Y);  // m y 2^61 = sqrt(m) 2^61, in [2^61, 2^62)
  const int p = 63 - __clzll(S);
  const int sh = p - 52;
  unsigned long long mant = (S >> sh) + ((S >> (sh - 1)) & 1ull);
  int ex = ((e - 1023 - odd) >> 1) + 1023 + (p - 61);
  if (mant >> 53) { mant >>= 1; ++ex; }
  return __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0x000FFFFFFFFFFFFFull)));
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
