// mh_greens.cuh -- device Green-function kernels of the MarineHydro.jl hot path (FP64).
//
// Each function restates the reference function cited beside it (paths within the
// MarineHydro.jl tree).  Elementary functions are CUDA's (exp, log, atan2, sqrt, hypot,
// sincos), except in the Wu term, whose exp, log and reciprocals run on the integer pipe
// (mh_fixpoint.cuh); the Bessel functions J0, J1, Y0, Y1 (mh_bessel01.cuh, Chebyshev and Hankel
// forms), the complex exponential integral and the Gauss-Kronrod rule are written from
// published methods (DLMF 10.17.3, 6.6.2, 6.9.1; Kronrod's 15-point nodes, QUADPACK qk15).
#pragma once

#include <cuda_runtime.h>

#include "mh_bessel01.cuh"
#include "mh_fixpoint.cuh"
#include "mh_internal.cuh"

namespace mh {

// ------------------------------- complex ------------------------------------
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double zabs(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double2 zdiv(double2 a, double2 b) {
  // Smith's algorithm (scaled) for a / b
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  } else {
    double r = b.x / b.y, den = b.y + b.x * r;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
}
__device__ __forceinline__ double2 zexp(double2 a) {
  double s, c;
  sincos(a.y, &s, &c);
  double e = exp(a.x);
  return make_double2(e * c, e * s);
}
__device__ __forceinline__ double2 zlog(double2 a) { return make_double2(log(hypot(a.x, a.y)), atan2(a.y, a.x)); }

// ------------------------------- Birk Rankine -------------------------------
constexpr double kBirkZTol = 1e-14;   // rankine_vectorized.jl:24
constexpr double kBirkDkTol = 1e-14;  // rankine_vectorized.jl:25

// _abs_ad (rankine_vectorized.jl:30): -0.0 stays -0.0
__device__ __forceinline__ double abs_ad(double x) { return x < 0.0 ? -x : x; }
// _atan_ratio (rankine_vectorized.jl:42-45)
__device__ __forceinline__ double atan_ratio(double num, double den) {
  double flipped = den < 0.0 ? -num : num;
  return atan2(flipped, abs_ad(den));
}

// birk_phi_and_velocity (rankine_vectorized.jl:241-267); lc = 4 local corners (x, y),
// edge = their 4 edge lengths (per panel, precomputed; the same hypot of the corner offsets)
__device__ inline void birk_phi_and_velocity(double x, double y, double z, const double* lc, const double* edge,
                                             double& phi, double v[3]) {
  double sx[4], sy[4], r[4], e[4], h[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    sx[k] = x - lc[2 * k];
    sy[k] = y - lc[2 * k + 1];
    r[k] = sqrt(sx[k] * sx[k] + sy[k] * sy[k] + z * z);
    e[k] = sx[k] * sx[k] + z * z;
    h[k] = sx[k] * sy[k];
  }
  const bool inplane = fabs(z) <= kBirkZTol;  // _inplane_atan (:49-54)
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int kn = (k + 1) & 3;
    double dx = lc[2 * kn] - lc[2 * k];
    double dy = lc[2 * kn + 1] - lc[2 * k + 1];
    const double dk = edge[k];
    if (!(dk <= kBirkDkTol)) {
      double rsum = r[k] + r[kn];
      double log_term = log((rsum - dk) / (rsum + dk));
      double lt_dk = log_term / dk;
      double vzk = 0.0;
      if (!inplane)
        vzk = atan_ratio(dy * e[k] - dx * h[k], dx * z * r[k]) - atan_ratio(dy * e[kn] - dx * h[kn], dx * z * r[kn]);
      s0 += (sx[k] * dy - sy[k] * dx) * lt_dk + z * vzk;
      s1 += dy * lt_dk;
      s2 += -dx * lt_dk;
      s3 += vzk;
    }
  }
  phi = kMinusInv4Pi * s0;
  v[0] = kMinusInv4Pi * s1;
  v[1] = kMinusInv4Pi * s2;
  v[2] = kMinusInv4Pi * s3;
}

// _vrankine_from_geom (rankine_vectorized.jl:273-287): integral of 1/r over panel P
// seen from `pt`, and its gradient with respect to the source.
__device__ inline void vrankine_from_geom(const double pt[3], const PanelRec& P, double& phi, double g[3]) {
  double rb0 = pt[0] - P.c[0], rb1 = pt[1] - P.c[1], rb2 = pt[2] - P.c[2];
  double r = sqrt(rb0 * rb0 + rb1 * rb1 + rb2 * rb2);
  if (r > 7 * P.radius) {
    // a/r and a r_vec/r^3 from one FP64 division (within an ulp or two of the quotients)
    const double inv_r = 1.0 / r;
    const double s = P.area * inv_r * inv_r * inv_r;
    phi = P.area * inv_r;
    g[0] = rb0 * s;
    g[1] = rb1 * s;
    g[2] = rb2 * s;
    return;
  }
  double d0 = pt[0] - P.qgc[0], d1 = pt[1] - P.qgc[1], d2 = pt[2] - P.qgc[2];
  double fx = P.T[0] * d0 + P.T[1] * d1 + P.T[2] * d2;
  double fy = P.T[3] * d0 + P.T[4] * d1 + P.T[5] * d2;
  double fz = P.T[6] * d0 + P.T[7] * d1 + P.T[8] * d2;
  double phb, vl[3];
  birk_phi_and_velocity(fx, fy, fz, P.lc, P.edge, phb, vl);
#pragma unroll
  for (int i = 0; i < 3; ++i) g[i] = kFourPi * (P.T[i] * vl[0] + P.T[3 + i] * vl[1] + P.T[6 + i] * vl[2]);
  phi = -kFourPi * phb;
}

// ---------------------------- Delhommeau Rankine ----------------------------
__device__ __forceinline__ double sign_ad(double x) { return x < 0.0 ? -1.0 : 1.0; }

// integral(::DelhommeauRankine) (rankine.jl:33-71) and the gradient of
// both_integral_and_integral_gradient (rankine.jl:73-131); v12: 4 raw corners.
__device__ inline void delhommeau_rankine(const double pt[3], const PanelRec& P, const double* v12, int wrt_first,
                                          double& integral, double g[3]) {
  double rb[3] = {pt[0] - P.c[0], pt[1] - P.c[1], pt[2] - P.c[2]};
  double r = sqrt(rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]);
  const double* nrm = P.n;
  if (r > 7 * P.radius) {
    double r3 = r * r * r;
    integral = P.area / r;
    for (int c = 0; c < 3; ++c) g[c] = (1 / r3 * rb[c]) * P.area;
  } else {
    integral = 0.0;
    g[0] = g[1] = g[2] = 0.0;
    double GZ = rb[0] * nrm[0] + rb[1] * nrm[1] + rb[2] * nrm[2];
    double RR[4], DRX[4][3];
    for (int i = 0; i < 4; ++i) {
      double d[3] = {pt[0] - v12[3 * i], pt[1] - v12[3 * i + 1], pt[2] - v12[3 * i + 2]};
      RR[i] = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      for (int c = 0; c < 3; ++c) DRX[i][c] = d[c] / RR[i];
    }
    for (int iv = 0; iv < 4; ++iv) {
      int in = (iv + 1) & 3;
      double ctn[3] = {v12[3 * in] - v12[3 * iv], v12[3 * in + 1] - v12[3 * iv + 1], v12[3 * in + 2] - v12[3 * iv + 2]};
      double seg = sqrt(ctn[0] * ctn[0] + ctn[1] * ctn[1] + ctn[2] * ctn[2]);
      if (!(seg >= 1e-3 * P.radius)) continue;
      double u[3] = {ctn[0] / seg, ctn[1] / seg, ctn[2] / seg};
      double GYX[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2], nrm[0] * u[1] - nrm[1] * u[0]};
      double pv[3] = {pt[0] - v12[3 * iv], pt[1] - v12[3 * iv + 1], pt[2] - v12[3 * iv + 2]};
      double GY = pv[0] * GYX[0] + pv[1] * GYX[1] + pv[2] * GYX[2];
      double ANT = 2 * GY * seg;
      double rs = RR[in] + RR[iv];
      double DNT = rs * rs - seg * seg + 2 * abs_ad(GZ) * rs;
      double ANL = rs + seg, DNL = rs - seg;
      double ALDEN = log(ANL / DNL);
      double AT = fabs(GZ) >= 1e-4 * P.radius ? atan2(ANT, DNT) : 0.0;  // _delhommeau_atan
      integral -= 2 * abs_ad(GZ) * AT;
      if (fabs(GY) > 1e-5) integral += GY * ALDEN;
      double q1 = GY * (DNL - ANL), q2 = 2 * abs_ad(GZ), den2 = ANT * ANT + DNT * DNT;
      for (int c = 0; c < 3; ++c) {
        double ANLX = DRX[in][c] + DRX[iv][c];
        double ANTX = 2 * seg * GYX[c];
        double DNTX = 2 * (rs + abs_ad(GZ)) * ANLX + 2 * sign_ad(GZ) * rs * nrm[c];
        double term = ALDEN * GYX[c] - 2 * sign_ad(GZ) * AT * nrm[c] + q1 / (ANL * DNL) * ANLX -
                      q2 * (ANTX * DNT - DNTX * ANT) / den2;
        g[c] = g[c] - term;
      }
    }
  }
  if (wrt_first) { g[0] = -g[0]; g[1] = -g[1]; g[2] = -g[2]; }
}

// ------------------------------------ Wu -----------------------------------
// Polynomial fits A-D and dA-dC of Liang, Wu & Noblesse (wu.jl:131-197, 235-329), lowest
// degree first, all seven at one rho in [0, 1), in 64-bit fixed point on the integer pipe
// (mh_fixpoint.cuh): coefficients and partial sums are integers v 2^-44 (the partial sums
// stay below 2^18 on [0, 1)), so each Horner step truncates at 5.7e-14 absolute where FP64
// rounds partial sums up to 2e5 at 2.9e-11 (worst error of a fit 4e-13 here, up to 3e-11 in
// the reference's FP64 order); the coefficients are the FP64 values of the literals, as in
// the reference, exactly.
struct WuFits {
  double A, B, C, D, dA, dB, dC;
};

__device__ __forceinline__ void wu_fits(double rho, WuFits& f) {
  constexpr int F = 44;
  constexpr long long kA[10] = {fx::q(1.21, F), fx::q(-13.328, F), fx::q(215.896, F), fx::q(-1763.96, F),
                                fx::q(8418.94, F), fx::q(-24314.21, F), fx::q(42002.57, F), fx::q(-41592.9, F),
                                fx::q(21859.0, F), fx::q(-4838.6, F)};
  constexpr long long kB[10] = {fx::q(0.938, F), fx::q(5.737, F), fx::q(-67.92, F), fx::q(796.534, F),
                                fx::q(-4780.77, F), fx::q(17137.74, F), fx::q(-36618.81, F), fx::q(44894.06, F),
                                fx::q(-29030.24, F), fx::q(7671.22, F)};
  constexpr long long kC[8] = {fx::q(1.268, F), fx::q(-9.747, F), fx::q(209.653, F), fx::q(-1397.89, F),
                               fx::q(5155.67, F), fx::q(-9844.35, F), fx::q(9136.4, F), fx::q(-3272.62, F)};
  constexpr long long kD[10] = {fx::q(0.632, F), fx::q(-40.97, F), fx::q(667.16, F), fx::q(-6072.07, F),
                                fx::q(31127.39, F), fx::q(-96293.05, F), fx::q(181856.75, F), fx::q(-205690.43, F),
                                fx::q(128170.2, F), fx::q(-33744.6, F)};
  constexpr long long kdA[10] = {fx::q(2.948, F), fx::q(-24.53, F), fx::q(249.69, F), fx::q(-754.85, F),
                                 fx::q(-1187.71, F), fx::q(16370.75, F), fx::q(-48811.41, F), fx::q(68220.87, F),
                                 fx::q(-46688.0, F), fx::q(12622.25, F)};
  constexpr long long kdB[10] = {fx::q(1.11, F), fx::q(2.894, F), fx::q(-76.765, F), fx::q(1565.35, F),
                                 fx::q(-11336.19, F), fx::q(44270.15, F), fx::q(-97014.11, F), fx::q(118879.26, F),
                                 fx::q(-76209.82, F), fx::q(19923.28, F)};
  constexpr long long kdC[6] = {fx::q(14.19, F), fx::q(-148.24, F), fx::q(847.8, F), fx::q(-2318.58, F),
                                fx::q(3168.35, F), fx::q(-1590.27, F)};
  const unsigned long long t = fx::unit_q64(rho);
  f.A = fx::to_double(fx::horner_u(kA, t), F);
  f.B = fx::to_double(fx::horner_u(kB, t), F);
  f.C = fx::to_double(fx::horner_u(kC, t), F);
  f.D = fx::to_double(fx::horner_u(kD, t), F);
  f.dA = fx::to_double(fx::horner_u(kdA, t), F);
  f.dB = fx::to_double(fx::horner_u(kdB, t), F);
  f.dC = fx::to_double(fx::horner_u(kdC, t), F);
}

// StruveH0 and StruveH1 fits (wu.jl:368-435); also returns J0/J1.  The four Bessel
// functions of the argument come from one joint evaluation (mh_bessel01.cuh).  The
// polynomials in yy in [0, 1] run in fixed point (v 2^-59 below 3, 2^-55 above, variable
// yy / 2, so coefficient i carries 2^i); the rational fits' quotients stay FP64.
// inv_xx = 1 / xx (used above 3).
__device__ inline void struve_bessel(double xx, double inv_xx, double& H0, double& H1, double& J0, double& J1) {
  double Y0, Y1;
  bessel01(xx, J0, J1, Y0, Y1);
  constexpr int F = 59;
  if (xx <= 3.0) {
    const double x3 = xx * (1.0 / 3.0);
    const unsigned long long t = fx::unit_q63(x3 * x3);
    constexpr long long kH0[6] = {fx::q(1.909859164, F), fx::q(-1.909855001, F + 1), fx::q(0.687514637, F + 2),
                                  fx::q(-0.126164557, F + 3), fx::q(0.013828813, F + 4),
                                  fx::q(-0.000876918, F + 5)};
    // H1 = yy (1.909859286 + ...): the factor yy as one more Horner step with c = 0
    constexpr long long kH1[7] = {0, fx::q(1.909859286, F + 1), fx::q(-1.145914713, F + 2),
                                  fx::q(0.294656958, F + 3), fx::q(-0.042070508, F + 4),
                                  fx::q(0.003785727, F + 5), fx::q(-0.000207183, F + 6)};
    H0 = fx::to_double(fx::horner_u(kH0, t), F) * x3;
    H1 = fx::to_double(fx::horner_u(kH1, t), F);
  } else {
    constexpr int G = 55;  // partial sums up to 2^7
    const double t3 = 3.0 * inv_xx;
    const unsigned long long t = fx::unit_q63(t3 * t3);
    constexpr long long kC1[4] = {fx::q(0.99999906, G + 1), fx::q(4.77228920, G + 2), fx::q(3.85542044, G + 3),
                                  fx::q(0.32303607, G + 4)};  // 2 (a0 + a1 yy + ...)
    constexpr long long kC2[4] = {fx::q(1.0, G), fx::q(4.88331068, G + 1), fx::q(4.28957333, G + 2),
                                  fx::q(0.52120508, G + 3)};
    constexpr long long kD1[4] = {fx::q(1.00000004, G + 1), fx::q(3.92205313, G + 2), fx::q(2.64893033, G + 3),
                                  fx::q(0.27450895, G + 4)};
    constexpr long long kD2[4] = {fx::q(1.0, G), fx::q(3.81095112, G + 1), fx::q(2.26216956, G + 2),
                                  fx::q(0.10885141, G + 3)};
    const double c1 = fx::to_double(fx::horner_u(kC1, t), G);
    const double c2 = kPi * xx * fx::to_double(fx::horner_u(kC2, t), G);
    const double d1 = fx::to_double(fx::horner_u(kD1, t), G);
    const double d2 = kPi * fx::to_double(fx::horner_u(kD2, t), G);
    const double inv = fx::recip(c2 * d2);
    H0 = c1 * d2 * inv + Y0;
    H1 = d1 * c2 * inv + Y1;
  }
}

// _wu_wave_term_and_derivs (wu.jl:28-37) with GF_Func_L0/Lp/W/Ls/Lsp/Wh (wu.jl:201-366)
// FP64 division is a multi-instruction sequence on GB300's FP64 pipe, which bounds this
// kernel; 1/dd, 1/(dd - vv), 1/(1 + dd^3) and 1/hh come from one reciprocal of their
// product, taken on the integer pipe (fx::recip, within an ulp) like the other reciprocals
// and the square roots of the term, and are multiplied out (rho gets one residual
// correction on top: an ulp of rho moves the fits A-D by up to 1e-13).  inv_hh: 1/hh for hh > 1e-6 (the only pairs
// whose horizontal gradient factor k^2/hh is used, wu.jl:118-121), else 0.
__device__ inline void wu_wave_term_and_derivs(double hh, double vv, double2& GF, double2& dGh, double2& dGv,
                                               double* inv_hh = nullptr) {
  double dd = fx::sqrt_pos(hh * hh + vv * vv);
  double dd2 = dd * dd, dd3 = dd * dd * dd;
  // 1/dd, 1/(dd - vv), 1/(1 + dd^3) and 1/hh from one division of their product (all
  // factors are positive, dd - vv >= dd >= hh with vv <= 0, and moderate: below 1e6 in the
  // reduced coordinates, so the product stays far inside the FP64 range)
  const double dmv = dd - vv, opd3 = 1.0 + dd3;
  const bool has_h = fabs(hh) > 1e-6;
  const double hf = has_h ? hh : 1.0;
  const double prod3 = dd * dmv * opd3;
  const double inv_all = fx::recip(prod3 * hf);
  const double inv_all3 = inv_all * hf;  // 1 / (dd dmv opd3)
  const double inv_dd = dmv * opd3 * inv_all3;
  const double inv_dmv = dd * opd3 * inv_all3;
  const double inv_1dd3 = dd * dmv * inv_all3;
  const double inv_h = has_h ? prod3 * inv_all : 0.0;
  if (inv_hh) *inv_hh = inv_h;
  double alpha = -vv * inv_dd;
  double beta = hh * inv_dd;
  // rho = dd / (1 + dd): the integer-pipe reciprocal and one residual correction, which
  // leaves rho within a rounding of the correctly rounded quotient
  const double opdd = 1 + dd;
  const double r1 = fx::recip(opdd);
  double rho = dd * r1;
  rho = fma(fma(-rho, opdd, dd), r1, rho);
  double omr = 1.0 - rho;
  double omr3 = omr * omr * omr;
  double ev = fx::exp_nonpos(vv);
  double H0, H1, J0, J1;
  struve_bessel(hh, inv_h, H0, H1, J0, J1);
  // GF_Func_Lp
  WuFits fit;
  wu_fits(rho, fit);
  double RR = (1.0 - beta) * fit.A;
  RR -= beta * fit.B;
  RR -= alpha * fit.C * fx::recip(1.0 + 6.0 * alpha * rho * (1.0 - rho));
  RR += beta * (1.0 - beta) * fit.D;
  double Lp = rho * omr3 * RR;
  // GF_Func_L0
  const double gama = 0.5772156649;
  double PP = fx::log_pos(0.5 * (dd - vv)) + gama - 2.0 * dd2;
  PP = ev * PP;
  PP = PP + dd2 - vv;
  double L0 = 2.0 * PP * inv_1dd3 + 2.0 * Lp;
  const double twopi = 2 * kPi;
  GF = make_double2(-L0 - (twopi * H0) * ev, -((twopi * -J0) * ev));
  // GF_Func_Lsp
  double RS = beta * fit.dA;
  RS -= (1.0 - alpha) * fit.dB;
  RS += beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * fit.dC;
  double Lsp = rho * omr3 * RS;
  // GF_Func_Ls
  double PS = (beta + hh) * inv_dmv;
  PS = PS - 2.0 * beta + 2.0 * ev * dd - hh;
  double QS = fx::exp_nonpos(-dd) * (1.0 - beta);
  QS = QS * (1.0 + dd * inv_1dd3);
  double Ls = 2.0 * PS * inv_1dd3 - 4.0 * QS + 2.0 * Lsp;
  dGh = make_double2(-Ls - (twopi * (2 / kPi - H1)) * ev, -((twopi * J1) * ev));
  dGv = make_double2(GF.x + 2 * inv_dd, GF.y);
}

// _wu_reduced_hh_vv (wu.jl:7-18) == with_reduced_coordinates (abstract_greens_function.jl:117-138)
__device__ __forceinline__ void reduced_coords(const double x[3], const double xi[3], double k, double& hh,
                                               double& vv) {
  double d2 = (x[0] - xi[0]) * (x[0] - xi[0]) + (x[1] - xi[1]) * (x[1] - xi[1]);
  const double purt = 1e-18;
  double dis = (d2 == 0) ? sqrt(d2 + purt * purt) - purt : fx::sqrt_pos(d2);
  hh = k * dis;
  vv = k * (x[2] + xi[2]);
}

// _wu_sd (wu.jl:112-127): s, d for one pair before the -1/4pi scale
__device__ inline void wu_sd(const double x[3], const double xi[3], const double nv[3], double area2, double k,
                             double dx1, double dx2, double2& s, double2& d) {
  double hh, vv;
  reduced_coords(x, xi, k, hh, vv);
  double2 GF, Gh, Gv;
  wu_wave_term_and_derivs(hh, vv, GF, Gh, Gv);
  double dr1 = 0.0, dr2 = 0.0;
  if (fabs(hh) > 1e-6) {
    dr1 = k * k / hh * dx1;
    dr2 = k * k / hh * dx2;
  }
  double g0r = k * (dr1 * Gh.x), g0i = k * (dr1 * Gh.y);
  double g1r = k * (dr2 * Gh.x), g1i = k * (dr2 * Gh.y);
  double g2r = k * (k * Gv.x), g2i = k * (k * Gv.y);
  s = make_double2((k * GF.x) * area2, (k * GF.y) * area2);
  d = make_double2((nv[0] * g0r + nv[1] * g1r + nv[2] * g2r) * area2, (nv[0] * g0i + nv[1] * g1i + nv[2] * g2i) * area2);
}

// ------------------------- exact Guevel-Delhommeau --------------------------
// 1/n for the power series of E1 (every entry the correctly rounded quotient, as 1.0 / n)
struct InvN {
  double v[400];
};
__constant__ static const InvN kInvN = [] {
  InvN t{};
  for (int n = 1; n < 400; ++n) t.v[n] = 1.0 / (double)n;
  return t;
}();

// a / b for a real numerator: a conj(b) / |b|^2, one division (|b| stays far inside the
// FP64 range in the continued fraction below: its terms are b_i = z + 2i + 1 and their
// quotients)
__device__ __forceinline__ double2 rdivz(double a, double2 b) {
  const double s = a / (b.x * b.x + b.y * b.y);
  return make_double2(b.x * s, -b.y * s);
}

// e^z E1(z): power series of E1 (DLMF 6.6.2) where its cancellation loss
// exp(|z| + Re z) is below e^4, else the even continued fraction of DLMF 6.9.1
// by the modified Lentz method.  Iteration counts are bounded.  `ez` = e^z (the
// integrands have it already).  Convergence and underflow tests compare squared
// magnitudes (no hypot in the loops); 1/n comes from a table.
__device__ inline double2 exp_e1(double2 z, double2 ez) {
  const double az = hypot(z.x, z.y);
  if (az + z.x < 4.0) {
    double2 term = make_double2(1.0, 0.0), sum = make_double2(0.0, 0.0);
    const double2 mz = make_double2(-z.x, -z.y);
    for (int n = 1; n < 400; ++n) {
      const double inv = kInvN.v[n];
      term = zscale(inv, zmul(term, mz));
      const double2 add = zscale(inv, term);
      sum = zadd(sum, add);
      if (add.x * add.x + add.y * add.y <= 1e-34 * (sum.x * sum.x + sum.y * sum.y)) break;
    }
    const double euler_gamma = 0.57721566490153286061;
    const double2 lz = make_double2(log(az), atan2(z.y, z.x));
    const double2 e1 = make_double2(-euler_gamma - lz.x - sum.x, -lz.y - sum.y);
    return zmul(ez, e1);
  }
  const double tiny = 1e-300;
  double2 b = make_double2(z.x + 1.0, z.y);
  double2 f = b;
  double2 C = f, D = make_double2(0.0, 0.0);
  for (int i = 1; i < 400; ++i) {
    const double a = -(double)i * (double)i;
    b.x += 2.0;
    D = make_double2(b.x + a * D.x, b.y + a * D.y);
    if (fabs(D.x) + fabs(D.y) < tiny) D = make_double2(tiny, 0.0);
    const double2 q = rdivz(a, C);
    C = make_double2(b.x + q.x, b.y + q.y);
    if (fabs(C.x) + fabs(C.y) < tiny) C = make_double2(tiny, 0.0);
    D = rdivz(1.0, D);
    const double2 delta = zmul(C, D);
    f = zmul(f, delta);
    const double dx = delta.x - 1.0;
    if (dx * dx + delta.y * delta.y < 1e-32) break;
  }
  return rdivz(1.0, f);
}
__device__ inline double2 exp_e1(double2 z) { return exp_e1(z, zexp(z)); }

// integrands of _dimless_wave_term / _d_dimless_wave_term_dr
// (exact_Guevel_Delhommeau.jl:16-23, 36-43)
template <bool DR>
__device__ __forceinline__ double2 egd_integrand(double theta, double r, double z) {
  double ct = cos(theta);
  double2 zeta = make_double2(z, r * ct);
  double2 ez = zexp(zeta);
  double2 g = exp_e1(zeta, ez);
  // j = e^zeta (E1(zeta)/pi + i) = g/pi + i e^zeta
  const double inv_pi = 1.0 / kPi;
  double2 j = make_double2(g.x * inv_pi - ez.y, g.y * inv_pi + ez.x);
  if (!DR) return make_double2(j.x, ez.x);
  double2 inv = rdivz(inv_pi, zeta);  // 1 / (pi zeta); |zeta| >= -z > 0 below the free surface
  double2 w = make_double2(j.x - inv.x, j.y - inv.y);
  // Re(i ct w) = -ct Im(w); Re(i ct e^zeta) = -ct Im(e^zeta)
  return make_double2(-ct * w.y, -ct * ez.y);
}

__constant__ static const double kGKx[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                                           0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                                           0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                                           0.207784955007898467600689403773245, 0.0};
__constant__ static const double kGKwk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                            0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                            0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                            0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
__constant__ static const double kGKwg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                                            0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

template <bool DR>
__device__ inline void gk15(double a, double b, double r, double z, double2& val, double& err) {
  double c = 0.5 * (a + b), h = 0.5 * (b - a);
  double2 fc = egd_integrand<DR>(c, r, z);
  double2 Ik = zscale(kGKwk[7], fc), Ig = zscale(kGKwg[3], fc);
#pragma unroll 1
  for (int j = 0; j < 7; ++j) {
    double dx = h * kGKx[j];
    double2 f1 = egd_integrand<DR>(c - dx, r, z), f2 = egd_integrand<DR>(c + dx, r, z);
    double2 fs = zadd(f1, f2);
    Ik = zadd(Ik, zscale(kGKwk[j], fs));
    if (j & 1) Ig = zadd(Ig, zscale(kGKwg[j >> 1], fs));
  }
  val = zscale(h, Ik);
  double2 dif = zsub(Ik, Ig);
  err = hypot(dif.x * h, dif.y * h);
}

constexpr int kGKStack = 48;        // depth-first refinement stack (segments)
constexpr int kGKMaxEvals = 8192;   // GK15 evaluations per integral, a hard bound

// 4 * adaptive GK(7,15) over [0, pi/2] (exact_Guevel_Delhommeau.jl:8-13, 25, 45) to a
// total error estimate <= max(atol, rtol |I|).  The phase r cos(theta) of the integrand
// turns through r radians over the interval, so the interval is first cut into
// ceil(r / 4) equal segments (at most 1024, about 2/3 of an oscillation each); each is
// then refined depth-first by bisection until its GK error estimate is below its
// share of the tolerance, tol * length / (pi/2), with tol from a first pass over the
// initial segments.  The per-thread state is a short stack, so large r costs time,
// not memory.
template <bool DR>
__device__ inline double2 egd_adaptive(double r, double z, double rtol, double atol) {
  const double L = kPi / 2;
  const int m0 = (int)fmin(1024.0, fmax(1.0, ceil(r / 4.0)));
  const double h0 = L / m0;
  // first pass: the integral and the tolerance it implies
  double2 coarse = make_double2(0.0, 0.0);
  double v0e = 0.0;
  double2 v0 = make_double2(0.0, 0.0);
  for (int s = 0; s < m0; ++s) {
    double2 v;
    double e;
    gk15<DR>(s * h0, s == m0 - 1 ? L : (s + 1) * h0, r, z, v, e);
    coarse = zadd(coarse, v);
    if (s == 0) { v0 = v; v0e = e; }
  }
  int evals = m0;
  const double tol = fmax(atol, rtol * hypot(coarse.x, coarse.y));
  double2 total = make_double2(0.0, 0.0);
  double sa[kGKStack], sb[kGKStack], se[kGKStack];
  double2 sv[kGKStack];
  for (int s = 0; s < m0; ++s) {
    int top = 0;
    sa[0] = s * h0;
    sb[0] = s == m0 - 1 ? L : (s + 1) * h0;
    if (m0 == 1) {
      sv[0] = v0;
      se[0] = v0e;
    } else {
      gk15<DR>(sa[0], sb[0], r, z, sv[0], se[0]);
      ++evals;
    }
    top = 1;
    while (top > 0) {
      --top;
      const double a = sa[top], b = sb[top];
      const double2 v = sv[top];
      const double e = se[top];
      if (e <= tol * (b - a) / L || top + 2 > kGKStack || evals + 2 > kGKMaxEvals) {
        total = zadd(total, v);
        continue;
      }
      const double mid = 0.5 * (a + b);
      double2 v1, v2;
      double e1, e2;
      gk15<DR>(a, mid, r, z, v1, e1);
      gk15<DR>(mid, b, r, z, v2, e2);
      evals += 2;
      sa[top] = mid; sb[top] = b; sv[top] = v2; se[top] = e2; ++top;
      sa[top] = a; sb[top] = mid; sv[top] = v1; se[top] = e1; ++top;
    }
  }
  return zscale(4.0, total);
}

// ---- warp-cooperative form: one warp per (r, z), both integrals at once -------------
// The same quadrature rule and tolerance test, organised for the SIMT machine: the 15
// Kronrod nodes of two segments run on 30 lanes, G and dG/dr come from the same
// exp(zeta), E1(zeta) evaluation at each node, and the depth-first refinement stack
// lives in shared memory, written by lane 0 and read by the whole warp.  A segment is
// accepted when both integrals meet their share of the tolerance.
constexpr int kGKWarpStack = 48;   // entries of 8 doubles: a, b, G (2), dG/dr (2), err G, err dG/dr

// both integrands at theta (the two egd_integrand<> forms sharing E1)
__device__ __forceinline__ void egd_integrands(double theta, double r, double z, double f[4]) {
  const double ct = cos(theta);
  const double2 zeta = make_double2(z, r * ct);
  const double2 ez = zexp(zeta);
  const double2 g = exp_e1(zeta, ez);
  const double inv_pi = 1.0 / kPi;
  const double2 j = make_double2(g.x * inv_pi - ez.y, g.y * inv_pi + ez.x);
  f[0] = j.x;
  f[1] = ez.x;
  const double2 inv = rdivz(inv_pi, zeta);  // 1 / (pi zeta); |zeta| >= -z > 0 below the free surface
  const double2 w = make_double2(j.x - inv.x, j.y - inv.y);
  f[2] = -ct * w.y;
  f[3] = -ct * ez.y;
}

// Kronrod node, Kronrod weight and Gauss weight of this lane (lanes 15 and 31 idle)
__device__ __forceinline__ void gk_lane_node(int lane, double& t, double& wk, double& wg) {
  const int j = lane & 15;
  t = 0.0; wk = 0.0; wg = 0.0;
  if (j == 15) return;
  if (j < 7) {
    t = -kGKx[j]; wk = kGKwk[j]; wg = (j & 1) ? kGKwg[j >> 1] : 0.0;
  } else if (j == 7) {
    wk = kGKwk[7]; wg = kGKwg[3];
  } else {
    const int m = 14 - j;
    t = kGKx[m]; wk = kGKwk[m]; wg = (m & 1) ? kGKwg[m >> 1] : 0.0;
  }
}

// GK(7,15) of both integrands over [aA, bA] (lanes 0-15) and [aB, bB] (lanes 16-31);
// every lane returns both results
__device__ __forceinline__ void gk15_pair_warp(double aA, double bA, double aB, double bB, double r, double z,
                                               double vA[4], double& eGA, double& eRA, double vB[4], double& eGB,
                                               double& eRB) {
  const int lane = threadIdx.x & 31;
  double t, wk, wg;
  gk_lane_node(lane, t, wk, wg);
  const double a = lane < 16 ? aA : aB, b = lane < 16 ? bA : bB;
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  double f[4];
  egd_integrands(c + h * t, r, z, f);
  double K[4], Gs[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) { K[q] = wk * f[q]; Gs[q] = wg * f[q]; }
#pragma unroll
  for (int off = 8; off > 0; off >>= 1) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      K[q] += __shfl_xor_sync(0xffffffffu, K[q], off);
      Gs[q] += __shfl_xor_sync(0xffffffffu, Gs[q], off);
    }
  }
  double KA[4], GA[4], KB[4], GB[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    KA[q] = __shfl_sync(0xffffffffu, K[q], 0);
    GA[q] = __shfl_sync(0xffffffffu, Gs[q], 0);
    KB[q] = __shfl_sync(0xffffffffu, K[q], 16);
    GB[q] = __shfl_sync(0xffffffffu, Gs[q], 16);
  }
  const double hA = 0.5 * (bA - aA), hB = 0.5 * (bB - aB);
#pragma unroll
  for (int q = 0; q < 4; ++q) { vA[q] = hA * KA[q]; vB[q] = hB * KB[q]; }
  eGA = hypot(hA * (KA[0] - GA[0]), hA * (KA[1] - GA[1]));
  eRA = hypot(hA * (KA[2] - GA[2]), hA * (KA[3] - GA[3]));
  eGB = hypot(hB * (KB[0] - GB[0]), hB * (KB[1] - GB[1]));
  eRB = hypot(hB * (KB[2] - GB[2]), hB * (KB[3] - GB[3]));
}

// G = _dimless_wave_term(r, z) and dG/dr = _d_dimless_wave_term_dr(r, z) by the whole warp
// (all 32 lanes call it with the same r, z; `sw` is this warp's 8 * kGKWarpStack doubles of
// shared memory).  Same segmentation and tolerance rule as egd_adaptive.
__device__ inline void egd_warp(double r, double z, double rtol, double atol, double* sw, double2& G, double2& Gr) {
  const int lane = threadIdx.x & 31;
  const double L = kPi / 2;
  const int m0 = (int)fmin(1024.0, fmax(1.0, ceil(r / 4.0)));
  const double h0 = L / m0;
  // first pass: the integrals over the initial segments and the tolerances they imply
  double cg[4] = {0.0, 0.0, 0.0, 0.0};
  double v1[4] = {0.0, 0.0, 0.0, 0.0}, e1G = 0.0, e1R = 0.0;
  int evals = 0;
  for (int s = 0; s < m0; s += 2) {
    const int s2 = s + 1 < m0 ? s + 1 : s;
    double vA[4], vB[4], eGA, eRA, eGB, eRB;
    gk15_pair_warp(s * h0, s == m0 - 1 ? L : (s + 1) * h0, s2 * h0, s2 == m0 - 1 ? L : (s2 + 1) * h0, r, z, vA, eGA,
                   eRA, vB, eGB, eRB);
    ++evals;
#pragma unroll
    for (int q = 0; q < 4; ++q) cg[q] += vA[q] + (s2 != s ? vB[q] : 0.0);
    if (s == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) v1[q] = vA[q];
      e1G = eGA;
      e1R = eRA;
    }
  }
  const double tolG = fmax(atol, rtol * hypot(cg[0], cg[1]));
  const double tolR = fmax(atol, rtol * hypot(cg[2], cg[3]));
  double tot[4] = {0.0, 0.0, 0.0, 0.0};
  int top = 0;
  auto push = [&](double a, double b, const double v[4], double eG, double eR) {
    if (lane == 0) {
      double* e = sw + 8 * top;
      e[0] = a; e[1] = b; e[2] = v[0]; e[3] = v[1]; e[4] = v[2]; e[5] = v[3]; e[6] = eG; e[7] = eR;
    }
    ++top;
  };
  for (int s = 0; s < m0; s += 2) {
    const int s2 = s + 1 < m0 ? s + 1 : s;
    if (m0 == 1) {
      push(0.0, L, v1, e1G, e1R);
    } else {
      double vA[4], vB[4], eGA, eRA, eGB, eRB;
      const double aA = s * h0, bA = s == m0 - 1 ? L : (s + 1) * h0;
      const double aB = s2 * h0, bB = s2 == m0 - 1 ? L : (s2 + 1) * h0;
      gk15_pair_warp(aA, bA, aB, bB, r, z, vA, eGA, eRA, vB, eGB, eRB);
      ++evals;
      if (s2 != s) push(aB, bB, vB, eGB, eRB);
      push(aA, bA, vA, eGA, eRA);
    }
    __syncwarp();
    while (top > 0) {
      --top;
      const double* e = sw + 8 * top;
      const double a = e[0], b = e[1], eG = e[6], eR = e[7];
      const double v[4] = {e[2], e[3], e[4], e[5]};
      __syncwarp();  // every lane has read the entry before it can be overwritten
      const double frac = (b - a) / L;
      if ((eG <= tolG * frac && eR <= tolR * frac) || top + 2 > kGKWarpStack || evals + 1 > kGKMaxEvals) {
#pragma unroll
        for (int q = 0; q < 4; ++q) tot[q] += v[q];
        continue;
      }
      const double mid = 0.5 * (a + b);
      double vA[4], vB[4], eGA, eRA, eGB, eRB;
      gk15_pair_warp(a, mid, mid, b, r, z, vA, eGA, eRA, vB, eGB, eRB);
      ++evals;
      push(mid, b, vB, eGB, eRB);
      push(a, mid, vA, eGA, eRA);  // the left half is refined first
      __syncwarp();
    }
  }
  G = make_double2(4.0 * tot[0], 4.0 * tot[1]);
  Gr = make_double2(4.0 * tot[2], 4.0 * tot[3]);
}

// both_greens_and_gradient_greens(::ExactGuevelDelhommeau) with
// with_reduced_coordinates_derivative (exact_Guevel_Delhommeau.jl:52-59;
// abstract_greens_function.jl:140-185); outputs already multiplied by the area
// (integral / integral_gradient, exact_Guevel_Delhommeau.jl:61-69).
__device__ inline void egd_integrals(const double x[3], const double xi[3], double k, double area, int wrt_first,
                                     double rtol, double atol, double2& I, double2 g[3]) {
  double r, z;
  reduced_coords(x, xi, k, r, z);
  double2 GF = egd_adaptive<false>(r, z, rtol, atol);
  double2 dGdr = egd_adaptive<true>(r, z, rtol, atol);
  double2 dGdz = make_double2(GF.x + 2 / hypot(r, z), GF.y);
  double d1 = 0.0, d2 = 0.0;
  if (fabs(r) > 1e-6) {
    if (wrt_first) { d1 = k * k / r * (x[0] - xi[0]); d2 = k * k / r * (x[1] - xi[1]); }
    else { d1 = k * k / r * (xi[0] - x[0]); d2 = k * k / r * (xi[1] - x[1]); }
  }
  I = make_double2((k * GF.x) * area, (k * GF.y) * area);
  g[0] = make_double2((k * (d1 * dGdr.x)) * area, (k * (d1 * dGdr.y)) * area);
  g[1] = make_double2((k * (d2 * dGdr.x)) * area, (k * (d2 * dGdr.y)) * area);
  g[2] = make_double2((k * (k * dGdz.x)) * area, (k * (k * dGdz.y)) * area);
}

}  // namespace mh
