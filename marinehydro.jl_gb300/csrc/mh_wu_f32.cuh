// mh_wu_f32.cuh -- the Wu wave term and its derivatives in FP32, for the learned surrogate
// path (Wu fits + network correction toward the exact Guevel-Delhommeau term).
//
// The surrogate's own error against the exact term is ~1e-3 of the coefficients, so the Wu
// base it corrects needs no FP64: on GB300 FP64 runs at ~1/70 of the FP32 rate, and in FP64
// this base is what bounds the surrogate assembly.  The arithmetic is that of
// wu_wave_term_and_derivs (mh_greens.cuh, restating wu.jl:28-37, 201-435) with three
// changes that keep FP32 rounding from being amplified:
//   * the seven polynomial fits A-D, dA-dC are evaluated in the Chebyshev basis of
//     2 rho - 1 (the same polynomials, coefficients below 15 instead of up to 2e5 of
//     alternating sign; gen_special_tables.py) by Clenshaw's recurrence;
//   * J0, J1, Y0, Y1 come from the FP32 joint evaluator bessel01f;
//   * 1/dd and 1/(1 + dd^3) are formed once.
// Measured against the FP64 term: below 2e-6 of max(|G|, 1) over the surrogate's box.
#pragma once

#include <cuda_runtime.h>

#include "mh_bessel01.cuh"
#include "mh_special_tables.cuh"

namespace mh {
namespace wuf {

// sum_j c_j T_j(s), |s| <= 1
template <int N>
__device__ __forceinline__ float clenshaw(const float (&c)[N], float s) {
  const float s2 = s + s;
  float b1 = 0.0f, b2 = 0.0f;
#pragma unroll
  for (int j = N - 1; j >= 1; --j) {
    const float b0 = fmaf(s2, b1, c[j] - b2);
    b2 = b1;
    b1 = b0;
  }
  return fmaf(s, b1, c[0] - b2);
}

}  // namespace wuf

__device__ inline void wu_wave_term_and_derivs_f32(float hh, float vv, float2& GF, float2& dGh, float2& dGv) {
  using namespace wuf;
  const float pi = 3.14159265f, twopi = 6.28318531f;
  const float dd = sqrtf(fmaf(hh, hh, vv * vv));
  const float inv_dd = 1.0f / dd;
  const float alpha = -vv * inv_dd;
  const float beta = hh * inv_dd;
  const float rho = dd / (1.0f + dd);
  const float s = fmaf(2.0f, rho, -1.0f);
  const float dd2 = dd * dd, dd3 = dd2 * dd;
  const float omr = 1.0f - rho;
  const float omr3 = omr * omr * omr;
  const float ev = expf(vv);
  float J0, J1, Y0, Y1, H0, H1;
  bessel01f(hh, J0, J1, Y0, Y1);
  // StruveH0 and StruveH1 fits (wu.jl:368-435)
  if (hh <= 3.0f) {
    const float x3 = hh * (1.0f / 3.0f);
    const float yy = x3 * x3;
    const float h0 = 1.909859164f + (-1.909855001f + (0.687514637f + (-0.126164557f + (0.013828813f + -0.000876918f * yy) * yy) * yy) * yy) * yy;
    H0 = h0 * x3;
    H1 = (1.909859286f + (-1.145914713f + (0.294656958f + (-0.042070508f + (0.003785727f + -0.000207183f * yy) * yy) * yy) * yy) * yy) * yy;
  } else {
    const float t3 = 3.0f / hh;
    const float yy = t3 * t3;
    const float c1 = 2.0f * (0.99999906f + (4.77228920f + (3.85542044f + 0.32303607f * yy) * yy) * yy);
    const float c2 = pi * hh * (1.0f + (4.88331068f + (4.28957333f + 0.52120508f * yy) * yy) * yy);
    H0 = c1 / c2 + Y0;
    const float d1 = 2.0f * (1.00000004f + (3.92205313f + (2.64893033f + 0.27450895f * yy) * yy) * yy);
    const float d2 = pi * (1.0f + (3.81095112f + (2.26216956f + 0.10885141f * yy) * yy) * yy);
    H1 = d1 / d2 + Y1;
  }
  // GF_Func_Lp
  float RR = (1.0f - beta) * clenshaw(kChebA, s);
  RR -= beta * clenshaw(kChebB, s);
  RR -= alpha * clenshaw(kChebC, s) / (1.0f + 6.0f * alpha * rho * omr);
  RR += beta * (1.0f - beta) * clenshaw(kChebD, s);
  const float Lp = rho * omr3 * RR;
  // GF_Func_L0
  const float gama = 0.5772156649f;
  float PP = logf(0.5f * (dd - vv)) + gama - 2.0f * dd2;
  PP = ev * PP + dd2 - vv;
  const float inv_1dd3 = 1.0f / (1.0f + dd3);
  const float L0 = 2.0f * PP * inv_1dd3 + 2.0f * Lp;
  GF = make_float2(-L0 - (twopi * H0) * ev, (twopi * J0) * ev);
  // GF_Func_Lsp
  float RS = beta * clenshaw(kChebdA, s);
  RS -= (1.0f - alpha) * clenshaw(kChebdB, s);
  RS += beta * (1.0f - beta) * rho * (1.0f - 2.0f * rho) * clenshaw(kChebdC, s);
  const float Lsp = rho * omr3 * RS;
  // GF_Func_Ls
  float PS = (beta + hh) / (dd - vv);
  PS = PS - 2.0f * beta + 2.0f * ev * dd - hh;
  const float QS = expf(-dd) * (1.0f - beta) * (1.0f + dd * inv_1dd3);
  const float Ls = 2.0f * PS * inv_1dd3 - 4.0f * QS + 2.0f * Lsp;
  dGh = make_float2(-Ls - (twopi * (2.0f / pi - H1)) * ev, -((twopi * J1) * ev));
  dGv = make_float2(GF.x + 2.0f * inv_dd, GF.y);
}

}  // namespace mh
