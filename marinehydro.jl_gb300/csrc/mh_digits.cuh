// mh_digits.cuh -- exact digit splitting of FP64 values for the tensor-core FP64 products
// (mh_ozaki.cu, mh_zgemv_tc.cu), in integer arithmetic on the FP64 bit fields.
//
// A row (or column) of values with largest biased exponent emax (|v| < 2^E, E = emax - 1022)
// is scaled to a 55-bit fixed point X = round(v 2^(55 - E)) and cut into eight balanced
// base-128 digits d_0 .. d_7 in [-64, 64], X = sum_p d_p 128^(7 - p) (the GEMV), or seven
// balanced base-256 digits in [-128, 128] (the LU update); each digit is exact in BF16.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mh {
namespace dg {

constexpr int kDigits = 8;

// biased exponent field of v (0 for zero and subnormals)
__device__ __forceinline__ int biased_exp(double v) {
  return (int)((__double_as_longlong(v) >> 52) & 0x7FF);
}

// the scale exponent E of a row or column from its largest biased exponent
__device__ __forceinline__ int scale_of(int emax_biased) { return emax_biased > 0 ? emax_biased - 1022 : 0; }

// round(v 2^(55 - E)), rounding half away from zero; zero and subnormal entries give 0
__device__ __forceinline__ long long fixed55(double v, int emax_biased) {
  const long long bits = __double_as_longlong(v);
  const int ev = (int)((bits >> 52) & 0x7FF);
  if (ev == 0) return 0;
  const long long m = (bits & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL;
  const int s = ev - emax_biased + 2;  // <= 2
  long long X;
  if (s >= 0) X = m << s;
  else if (s > -63) X = (m + (1LL << (-s - 1))) >> (-s);
  else X = 0;
  return bits < 0 ? -X : X;
}

// the balanced digits of X, most significant first, with 32-bit arithmetic:
// X = hi 2^28 + lo, lo in [0, 2^28) gives digits 7..4 and a carry, hi (|hi| < 2^27) 3..0
__device__ __forceinline__ void digits(long long X, int (&d)[kDigits]) {
  int lo = (int)(X & 0xFFFFFFF);
  int hi = (int)(X >> 28);
#pragma unroll
  for (int p = kDigits - 1; p >= 4; --p) {
    const int c = lo + 64;
    d[p] = (c & 127) - 64;
    lo = c >> 7;
  }
  hi += lo;
#pragma unroll
  for (int p = 3; p >= 1; --p) {
    const int c = hi + 64;
    d[p] = (c & 127) - 64;
    hi = c >> 7;
  }
  d[0] = hi;
}

// two BF16 values of small integers (|d| <= 64) in one 32-bit word, the first in the low half
__device__ __forceinline__ uint32_t bf16x2(int d0, int d1) {
  const float f0 = __int_as_float(0x4B400000 + d0) - 12582912.0f;
  const float f1 = __int_as_float(0x4B400000 + d1) - 12582912.0f;
  return __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
}

// Eight consecutive K values (one 16-byte row chunk of the canonical K-major layout) of one
// row: their 16 digit planes (re/im x 8 digits) as packed BF16 pairs, pk[part][digit][0..3].
__device__ __forceinline__ void split8(const double2 (&v)[8], int emax, uint32_t (&pk)[2][kDigits][4]) {
#pragma unroll
  for (int c = 0; c < 8; c += 2) {
    int a0[kDigits], a1[kDigits], b0[kDigits], b1[kDigits];
    digits(fixed55(v[c].x, emax), a0);
    digits(fixed55(v[c + 1].x, emax), a1);
    digits(fixed55(v[c].y, emax), b0);
    digits(fixed55(v[c + 1].y, emax), b1);
#pragma unroll
    for (int p = 0; p < kDigits; ++p) {
      pk[0][p][c >> 1] = bf16x2(a0[p], a1[p]);
      pk[1][p][c >> 1] = bf16x2(b0[p], b1[p]);
    }
  }
}

// Seven balanced base-256 digits in [-128, 128] of the same X (|X| < 2^55), most significant
// first: X = sum_p d_p 256^(6 - p).  X = hi 2^24 + lo, lo in [0, 2^24) gives digits 6..4 and
// a carry, hi (|hi| < 2^31) digits 3..0.  Each is exact in BF16 (eight significant bits).
constexpr int kDigits7 = 7;
__device__ __forceinline__ void digits7(long long X, int (&d)[kDigits7]) {
  int lo = (int)(X & 0xFFFFFF);
  int hi = (int)(X >> 24);
#pragma unroll
  for (int p = kDigits7 - 1; p >= 4; --p) {
    const int c = lo + 128;
    d[p] = (c & 255) - 128;
    lo = c >> 8;
  }
  hi += lo;
#pragma unroll
  for (int p = 3; p >= 1; --p) {
    const int c = hi + 128;
    d[p] = (c & 255) - 128;
    hi = c >> 8;
  }
  d[0] = hi;
}

// split8 with seven base-256 digit planes
__device__ __forceinline__ void split7(const double2 (&v)[8], int emax, uint32_t (&pk)[2][kDigits7][4]) {
#pragma unroll
  for (int c = 0; c < 8; c += 2) {
    int a0[kDigits7], a1[kDigits7], b0[kDigits7], b1[kDigits7];
    digits7(fixed55(v[c].x, emax), a0);
    digits7(fixed55(v[c + 1].x, emax), a1);
    digits7(fixed55(v[c].y, emax), b0);
    digits7(fixed55(v[c + 1].y, emax), b1);
#pragma unroll
    for (int p = 0; p < kDigits7; ++p) {
      pk[0][p][c >> 1] = bf16x2(a0[p], a1[p]);
      pk[1][p][c >> 1] = bf16x2(b0[p], b1[p]);
    }
  }
}

}  // namespace dg
}  // namespace mh
