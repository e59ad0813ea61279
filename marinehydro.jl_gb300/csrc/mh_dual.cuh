// mh_dual.cuh -- forward-mode dual numbers for the reverse (adjoint) kernels.
//
// Dn<M> carries a value and M partial derivatives.  The adjoint kernels evaluate
// the pair Green functions on Dn to obtain the exact derivatives of the code path
// the primal kernels run (the Wu polynomial/Struve fits, the Birk panel
// integral), the way the reference differentiates them with ForwardDiff / Enzyme
// (ad_rules.jl:79-294).  Derivatives of the special functions:
//   d j0 = -j1, d j1 = j0 - j1/x, d y0 = -y1, d y1 = y0 - y1/x,
//   d atan2(y, x) = (x dy - y dx) / (x^2 + y^2).
#pragma once

#include <cuda_runtime.h>

#include "mh_bessel01.cuh"

namespace mh {

template <int M>
struct Dn {
  double v;
  double d[M];
  __device__ Dn() : v(0.0) {
#pragma unroll
    for (int q = 0; q < M; ++q) d[q] = 0.0;
  }
  __device__ Dn(double x) : v(x) {
#pragma unroll
    for (int q = 0; q < M; ++q) d[q] = 0.0;
  }
  __device__ static Dn var(double x, int slot) {
    Dn r(x);
    if (slot >= 0 && slot < M) r.d[slot] = 1.0;
    return r;
  }
};

template <int M> __device__ __forceinline__ double val(const Dn<M>& a) { return a.v; }
__device__ __forceinline__ double val(double a) { return a; }

// double overloads, so that templated code written for Dn also compiles for double
// (and unqualified calls inside namespace mh keep finding the CUDA math functions)
__device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
__device__ __forceinline__ double log(double x) { return ::log(x); }
__device__ __forceinline__ double exp(double x) { return ::exp(x); }
__device__ __forceinline__ double atan2(double y, double x) { return ::atan2(y, x); }
__device__ __forceinline__ double hypot(double x, double y) { return ::hypot(x, y); }

// chain: r = f(a) with f'(a) = s
template <int M> __device__ __forceinline__ Dn<M> chain1(const Dn<M>& a, double fv, double s) {
  Dn<M> r(fv);
#pragma unroll
  for (int q = 0; q < M; ++q) r.d[q] = s * a.d[q];
  return r;
}

template <int M> __device__ __forceinline__ Dn<M> operator+(const Dn<M>& a, const Dn<M>& b) {
  Dn<M> r(a.v + b.v);
#pragma unroll
  for (int q = 0; q < M; ++q) r.d[q] = a.d[q] + b.d[q];
  return r;
}
template <int M> __device__ __forceinline__ Dn<M> operator-(const Dn<M>& a, const Dn<M>& b) {
  Dn<M> r(a.v - b.v);
#pragma unroll
  for (int q = 0; q < M; ++q) r.d[q] = a.d[q] - b.d[q];
  return r;
}
template <int M> __device__ __forceinline__ Dn<M> operator-(const Dn<M>& a) { return chain1(a, -a.v, -1.0); }
template <int M> __device__ __forceinline__ Dn<M> operator*(const Dn<M>& a, const Dn<M>& b) {
  Dn<M> r(a.v * b.v);
#pragma unroll
  for (int q = 0; q < M; ++q) r.d[q] = a.d[q] * b.v + a.v * b.d[q];
  return r;
}
// Divisions take one FP64 reciprocal (a multi-instruction sequence on the FP64 pipe) and
// multiply by it; the value is then within an ulp of the correctly rounded quotient, which
// is immaterial for the derivatives these kernels produce.
template <int M> __device__ __forceinline__ Dn<M> operator/(const Dn<M>& a, const Dn<M>& b) {
  const double inv = 1.0 / b.v, rv = a.v * inv;
  Dn<M> r(rv);
#pragma unroll
  for (int q = 0; q < M; ++q) r.d[q] = (a.d[q] - rv * b.d[q]) * inv;
  return r;
}
template <int M> __device__ __forceinline__ Dn<M> operator+(const Dn<M>& a, double b) { return chain1(a, a.v + b, 1.0); }
template <int M> __device__ __forceinline__ Dn<M> operator+(double b, const Dn<M>& a) { return chain1(a, b + a.v, 1.0); }
template <int M> __device__ __forceinline__ Dn<M> operator-(const Dn<M>& a, double b) { return chain1(a, a.v - b, 1.0); }
template <int M> __device__ __forceinline__ Dn<M> operator-(double b, const Dn<M>& a) { return chain1(a, b - a.v, -1.0); }
template <int M> __device__ __forceinline__ Dn<M> operator*(const Dn<M>& a, double b) { return chain1(a, a.v * b, b); }
template <int M> __device__ __forceinline__ Dn<M> operator*(double b, const Dn<M>& a) { return chain1(a, b * a.v, b); }
template <int M> __device__ __forceinline__ Dn<M> operator/(const Dn<M>& a, double b) {
  const double inv = 1.0 / b;
  return chain1(a, a.v * inv, inv);
}
template <int M> __device__ __forceinline__ Dn<M> operator/(double b, const Dn<M>& a) {
  const double inv = 1.0 / a.v, rv = b * inv;
  return chain1(a, rv, -rv * inv);
}
template <int M> __device__ __forceinline__ Dn<M>& operator+=(Dn<M>& a, const Dn<M>& b) { a = a + b; return a; }
template <int M> __device__ __forceinline__ Dn<M>& operator-=(Dn<M>& a, const Dn<M>& b) { a = a - b; return a; }

template <int M> __device__ __forceinline__ Dn<M> sqrt(const Dn<M>& a) {
  const double s = ::sqrt(a.v);
  return chain1(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
template <int M> __device__ __forceinline__ Dn<M> log(const Dn<M>& a) { return chain1(a, ::log(a.v), 1.0 / a.v); }
template <int M> __device__ __forceinline__ Dn<M> exp(const Dn<M>& a) {
  const double e = ::exp(a.v);
  return chain1(a, e, e);
}
template <int M> __device__ __forceinline__ Dn<M> atan2(const Dn<M>& y, const Dn<M>& x) {
  const double den = x.v * x.v + y.v * y.v;
  Dn<M> r(::atan2(y.v, x.v));
  if (den > 0.0) {
#pragma unroll
    for (int q = 0; q < M; ++q) r.d[q] = (x.v * y.d[q] - y.v * x.d[q]) / den;
  }
  return r;
}
template <int M> __device__ __forceinline__ Dn<M> hypot(const Dn<M>& x, const Dn<M>& y) {
  const double h = ::hypot(x.v, y.v);
  Dn<M> r(h);
  if (h > 0.0) {
#pragma unroll
    for (int q = 0; q < M; ++q) r.d[q] = (x.v * x.d[q] + y.v * y.d[q]) / h;
  }
  return r;
}
// J0, J1 (and Y0, Y1 for x >= 3) from one joint evaluation (mh_bessel01.cuh), with
// J0' = -J1, J1' = J0 - J1/x (1/2 at 0), Y0' = -Y1, Y1' = Y0 - Y1/x
__device__ __forceinline__ void bessel01_t(double x, double& J0, double& J1, double& Y0, double& Y1) {
  bessel01(x, J0, J1, Y0, Y1);
}
template <int M>
__device__ __forceinline__ void bessel01_t(const Dn<M>& a, Dn<M>& J0, Dn<M>& J1, Dn<M>& Y0, Dn<M>& Y1) {
  const double x = a.v;
  double j0v, j1v, y0v, y1v;
  bessel01(x, j0v, j1v, y0v, y1v);
  const double inv_x = x != 0.0 ? 1.0 / x : 0.0;
  J0 = chain1(a, j0v, -j1v);
  J1 = chain1(a, j1v, x != 0.0 ? j0v - j1v * inv_x : 0.5);
  Y0 = chain1(a, y0v, -y1v);
  Y1 = chain1(a, y1v, y0v - y1v * inv_x);
}

}  // namespace mh
