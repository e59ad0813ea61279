// mh_bessel01.cuh -- J0, J1, Y0, Y1 of one argument in one evaluation, for the Wu wave term
// (wu.jl:203, 335, 396, 431 call SpecialFunctions.jl's besselj0/j1, bessely0/y1 at the same
// argument): bessel01 in FP64, bessel01f in FP32 for the surrogate path's FP32 Wu term.
//
// Below x = 8 each function is a polynomial (degree 11 in FP64, 6 in FP32) on its half-unit
// interval, read from a table by the interval index, so the lanes of a warp follow one
// instruction stream whatever their arguments; above x = 8 Hankel's modulus-phase form
// shares one sincos between all four.  In FP64 the polynomials are evaluated in fixed point
// on the integer pipe.  The coefficients come from gen_special_tables.py
// (Chebyshev interpolation of mpmath's functions; the method and its measured error, below
// 1e-16 absolute in FP64 and 4e-8 in FP32, are described there).  Absolute, not relative,
// accuracy: near a zero of a function its relative error grows, as it does for any
// evaluation of it in floating point.
#pragma once

#include <cuda_runtime.h>

#include "mh_fixpoint.cuh"
#include "mh_special_tables.cuh"

namespace mh {
namespace bes {

template <int N, typename T>
__device__ __forceinline__ T horner_ld(const T* __restrict__ c, T t) {
  T v = __ldg(c + N - 1);
#pragma unroll
  for (int i = N - 2; i >= 0; --i) v = fma(v, t, __ldg(c + i));
  return v;
}

template <int N, typename T>
__device__ __forceinline__ T horner_c(const T (&c)[N], T t) {
  T v = c[N - 1];
#pragma unroll
  for (int i = N - 2; i >= 0; --i) v = fma(v, t, c[i]);
  return v;
}

}  // namespace bes

// J0(x), J1(x) for x >= 0; Y0(x), Y1(x) for x >= 3 (below 3 the Y outputs are not defined
// and must not be used).  The polynomials run in 64-bit fixed point on the integer pipe
// (mh_fixpoint.cuh, tables besq): below 8, X = floor(x 2^60) gives the interval q = X >> 59
// and z = 2 (x - q/2 - 1/4) as (X - q 2^59 - 2^58) 2^5 exactly; above 8 the Hankel
// polynomials take z = (u - 1/2) / 2 from the FP64 u = (8/x)^2.  Absolute error below 1e-17
// (the integer evaluation, emulated bit for bit by the generator, against mpmath).
__device__ __forceinline__ void bessel01(double x, double& J0, double& J1, double& Y0, double& Y1) {
  using namespace bes;
  if (x < 8.0) {
    long long X = fx::to_q(x, 60);
    X = X < 0 ? 0 : X;
    const int q = (int)(X >> 59);  // X < 2^63: q <= 15
    const long long z = (X - (((long long)q << 59) + (1ll << 58))) << 5;
    J0 = fx::to_double(fx::horner_s_ld<kLowTerms>(besq::kJ0 + q * kLowTerms, z), besq::kFrac);
    J1 = fx::to_double(fx::horner_s_ld<kLowTerms>(besq::kJ1 + q * kLowTerms, z), besq::kFrac);
    const int qy = q < 6 ? 0 : q - 6;
    const long long zy = q < 6 ? 0 : z;
    Y0 = fx::to_double(fx::horner_s_ld<kLowTerms>(besq::kY0 + qy * kLowTerms, zy), besq::kFrac);
    Y1 = fx::to_double(fx::horner_s_ld<kLowTerms>(besq::kY1 + qy * kLowTerms, zy), besq::kFrac);
  } else {
    const double f = rsqrt(3.14159265358979323846 * x);  // 1 / sqrt(pi x)
    const double s = 8.0 * 3.14159265358979323846 * f * f;  // 8 / x
    const long long z = fx::to_q(s * s - 0.5, 63);
    const double P0 = fx::to_double(fx::horner_s(besq::kP0, z), besq::kFrac);
    const double Q0 = s * fx::to_double(fx::horner_s(besq::kQ0, z), besq::kFrac);
    const double P1 = fx::to_double(fx::horner_s(besq::kP1, z), besq::kFrac);
    const double Q1 = s * fx::to_double(fx::horner_s(besq::kQ1, z), besq::kFrac);
    double sn, cs;
    sincos(x, &sn, &cs);
    // cos(x - pi/4) = (cos x + sin x) / sqrt 2, sin(x - pi/4) = (sin x - cos x) / sqrt 2; the
    // sqrt 2 cancels against sqrt(2 / (pi x)); the order-1 phase is that minus pi/2
    const double a = cs + sn, b = sn - cs;
    J0 = f * (P0 * a - Q0 * b);
    Y0 = f * (P0 * b + Q0 * a);
    J1 = f * (P1 * b + Q1 * a);
    Y1 = f * (Q1 * b - P1 * a);
  }
}

// The same in FP32 (tables of gen_special_tables.py at FP32 accuracy)
__device__ __forceinline__ void bessel01f(float x, float& J0, float& J1, float& Y0, float& Y1) {
  using namespace besf;
  if (x < 8.0f) {
    int q = (int)(2.0f * x);
    q = q < 0 ? 0 : (q > 15 ? 15 : q);
    const float t = x - (0.5f * q + 0.25f);
    J0 = bes::horner_ld<kLowTerms>(kJ0 + q * kLowTerms, t);
    J1 = bes::horner_ld<kLowTerms>(kJ1 + q * kLowTerms, t);
    const int qy = q < 6 ? 0 : q - 6;
    const float ty = q < 6 ? 0.0f : t;
    Y0 = bes::horner_ld<kLowTerms>(kY0 + qy * kLowTerms, ty);
    Y1 = bes::horner_ld<kLowTerms>(kY1 + qy * kLowTerms, ty);
  } else {
    const float f = rsqrtf(3.14159265f * x);
    const float s = 8.0f * 3.14159265f * f * f;
    const float u = s * s - 0.5f;
    const float P0 = bes::horner_c(kP0, u), Q0 = s * bes::horner_c(kQ0, u);
    const float P1 = bes::horner_c(kP1, u), Q1 = s * bes::horner_c(kQ1, u);
    float sn, cs;
    sincosf(x, &sn, &cs);
    const float a = cs + sn, b = sn - cs;
    J0 = f * (P0 * a - Q0 * b);
    Y0 = f * (P0 * b + Q0 * a);
    J1 = f * (P1 * b + Q1 * a);
    Y1 = f * (Q1 * b - P1 * a);
  }
}

}  // namespace mh
