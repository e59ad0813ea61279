// mh_adjoint.cu -- reverse (adjoint) kernels of the assembly: gradient of a
// real objective with respect to every panel's centre, normal, area and corner
// vertices, recomputing the Green-function derivatives pair by pair instead of
// storing them (the reference differentiates the assembly loops with Enzyme /
// ForwardDiff, matrix_assembly.jl:341-342, with the Birk kernel rules of
// ad_rules.jl:79-294).
//
// Objective weights.  With J = sum Re(W^S_ij dS_ij + W^D_ij dD_ij) over pairs,
// the caller supplies, per wavenumber, the weight factors as vectors
//   W^S_ij = c sum_h lS_h[i] rS_h[j],   W^D_ij = -c sum_h lD_h[i] rD_h[j]
// (rank-nh outer products, never formed), and for the wavenumber-independent
// Rankine part the real, frequency-summed matrices RS = Re sum W^S, RD = Re sum W^D.
// Direct BEM (phi = D^-1 S b, lam = D^-T w for the force weights w): lS = lD = lam,
// rS = b, rD = phi.  Indirect BEM (sigma = K^-1 b, phi = S sigma, lam = K^-T S^T w):
// lS = w, rS = rD = sigma, lD = lam -- the _mulvec and _linearsolve rules
// (ad_rules.jl:300-414) applied to the two formulations of solve (matrix_assembly.jl:436-449).
// The pair kernels are templated on the formulation: the indirect D differentiates the
// field point and carries the field panel's normal.
//
// Per-panel gradient accumulators (device, FP64, atomically summed):
//   gc[n][3] centre, gn[n][3] normal, ga[n] area, gv[n][12] Birk corner vertices.
#include <cuda_runtime.h>

#include "mh_dual.cuh"
#include "mh_greens.cuh"
#include "mh_internal.cuh"

namespace mh {

namespace {

constexpr int kRows = 128;
constexpr int kCols = 8;
constexpr int kMaxH = 4;  // right-hand sides per frequency in the adjoint weights

struct GradPtrs {
  double* gc;
  double* gn;
  double* ga;
  double* gv;
};

template <typename R> struct CR { R x, y; };

// ---------------------------------------------------------------------------
// Wu wave term on a generic scalar (the same operations as wu_wave_term_and_derivs)
// ---------------------------------------------------------------------------
template <typename R> __device__ R pA(R t) {
  R v = (21859.0 + -4838.6 * t) * t;
  v = (-41592.9 + v) * t; v = (42002.57 + v) * t; v = (-24314.21 + v) * t; v = (8418.94 + v) * t;
  v = (-1763.96 + v) * t; v = (215.896 + v) * t; v = (-13.328 + v) * t;
  return 1.21 + v;
}
template <typename R> __device__ R pB(R t) {
  R v = (-29030.24 + 7671.22 * t) * t;
  v = (44894.06 + v) * t; v = (-36618.81 + v) * t; v = (17137.74 + v) * t; v = (-4780.77 + v) * t;
  v = (796.534 + v) * t; v = (-67.92 + v) * t; v = (5.737 + v) * t;
  return 0.938 + v;
}
template <typename R> __device__ R pC(R t) {
  R v = (9136.4 + -3272.62 * t) * t;
  v = (-9844.35 + v) * t; v = (5155.67 + v) * t; v = (-1397.89 + v) * t; v = (209.653 + v) * t;
  v = (-9.747 + v) * t;
  return 1.268 + v;
}
template <typename R> __device__ R pD(R t) {
  R v = (128170.2 + -33744.6 * t) * t;
  v = (-205690.43 + v) * t; v = (181856.75 + v) * t; v = (-96293.05 + v) * t; v = (31127.39 + v) * t;
  v = (-6072.07 + v) * t; v = (667.16 + v) * t; v = (-40.97 + v) * t;
  return 0.632 + v;
}
template <typename R> __device__ R pdA(R t) {
  R v = (-46688.0 + 12622.25 * t) * t;
  v = (68220.87 + v) * t; v = (-48811.41 + v) * t; v = (16370.75 + v) * t; v = (-1187.71 + v) * t;
  v = (-754.85 + v) * t; v = (249.69 + v) * t; v = (-24.53 + v) * t;
  return 2.948 + v;
}
template <typename R> __device__ R pdB(R t) {
  R v = (-76209.82 + 19923.28 * t) * t;
  v = (118879.26 + v) * t; v = (-97014.11 + v) * t; v = (44270.15 + v) * t; v = (-11336.19 + v) * t;
  v = (1565.35 + v) * t; v = (-76.765 + v) * t; v = (2.894 + v) * t;
  return 1.11 + v;
}
template <typename R> __device__ R pdC(R t) {
  R v = (3168.35 + -1590.27 * t) * t;
  v = (-2318.58 + v) * t; v = (847.8 + v) * t; v = (-148.24 + v) * t;
  return 14.19 + v;
}

template <typename R>
__device__ void wu_terms_t(R hh, R vv, CR<R>& GF, CR<R>& Gh, CR<R>& Gv) {
  R dd = sqrt(hh * hh + vv * vv);
  const R inv_dd = 1.0 / dd;
  R alpha = -vv * inv_dd;
  R beta = hh * inv_dd;
  R rho = dd / (1.0 + dd);
  R dd2 = dd * dd, dd3 = dd * dd * dd;
  R omr = 1.0 - rho;
  R omr3 = omr * omr * omr;
  R ev = exp(vv);
  R J0, J1, Y0, Y1, H0, H1;
  bessel01_t(hh, J0, J1, Y0, Y1);
  if (val(hh) <= 3.0) {
    R yy = (hh / 3.0) * (hh / 3.0);
    R h0 = 1.909859164 + (-1.909855001 + (0.687514637 + (-0.126164557 + (0.013828813 + -0.000876918 * yy) * yy) * yy) * yy) * yy;
    H0 = h0 * (hh / 3.0);
    H1 = (1.909859286 + (-1.145914713 + (0.294656958 + (-0.042070508 + (0.003785727 + -0.000207183 * yy) * yy) * yy) * yy) * yy) * yy;
  } else {
    R yy = (3.0 / hh) * (3.0 / hh);
    R c1 = 2.0 * (0.99999906 + (4.77228920 + (3.85542044 + 0.32303607 * yy) * yy) * yy);
    R c2 = kPi * hh * (1.0 + (4.88331068 + (4.28957333 + 0.52120508 * yy) * yy) * yy);
    H0 = c1 / c2 + Y0;
    R d1 = 2.0 * (1.00000004 + (3.92205313 + (2.64893033 + 0.27450895 * yy) * yy) * yy);
    R d2 = kPi * (1.0 + (3.81095112 + (2.26216956 + 0.10885141 * yy) * yy) * yy);
    H1 = d1 / d2 + Y1;
  }
  R RR = (1.0 - beta) * pA(rho);
  RR -= beta * pB(rho);
  RR -= alpha * pC(rho) / (1.0 + 6.0 * alpha * rho * (1.0 - rho));
  RR += beta * (1.0 - beta) * pD(rho);
  R Lp = rho * omr3 * RR;
  const double gama = 0.5772156649;
  R PP = log(0.5 * (dd - vv)) + gama - 2.0 * dd2;
  PP = ev * PP;
  PP = PP + dd2 - vv;
  const R inv_1dd3 = 1.0 / (1.0 + dd3);
  R L0 = 2.0 * PP * inv_1dd3 + 2.0 * Lp;
  const double twopi = 2 * kPi;
  GF.x = -L0 - (twopi * H0) * ev;
  GF.y = -((twopi * -J0) * ev);
  R RS = beta * pdA(rho);
  RS -= (1.0 - alpha) * pdB(rho);
  RS += beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * pdC(rho);
  R Lsp = rho * omr3 * RS;
  R PS = (beta + hh) / (dd - vv);
  PS = PS - 2.0 * beta + 2.0 * ev * dd - hh;
  R QS = exp(-dd) * (1.0 - beta);
  QS = QS * (1.0 + dd * inv_1dd3);
  R Ls = 2.0 * PS * inv_1dd3 - 4.0 * QS + 2.0 * Lsp;
  Gh.x = -Ls - (twopi * (2 / kPi - H1)) * ev;
  Gh.y = -((twopi * J1) * ev);
  Gv.x = GF.x + 2.0 * inv_dd;
  Gv.y = GF.y;
}

// ---------------------------------------------------------------------------
// Birk panel pipeline on a generic scalar: geometry from the 4 corners and the
// near-field panel integral (rankine_vectorized.jl:79-137, 241-287)
// ---------------------------------------------------------------------------
template <typename R> __device__ R abs_ad_t(R x) { return val(x) < 0.0 ? -x : x; }
template <typename R> __device__ R atan_ratio_t(R num, R den) {
  R flipped = val(den) < 0.0 ? -num : num;
  return atan2(flipped, abs_ad_t(den));
}

template <typename R>
__device__ void birk_near_t(const R p[3], const R v[12], R& phi, R g[3]) {
  R mid[4][3], mgc[3], s[3], tt[3], nn[3], t[3];
  for (int i = 0; i < 4; ++i) {
    int ip = (i + 1) & 3;
    for (int c = 0; c < 3; ++c) mid[i][c] = (v[3 * i + c] + v[3 * ip + c]) / 2.0;
  }
  for (int c = 0; c < 3; ++c) {
    mgc[c] = (mid[1][c] + mid[3][c]) / 2.0;
    s[c] = mid[1][c] - mid[3][c];
    tt[c] = mid[2][c] - mid[0][c];
  }
  R ns = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  for (int c = 0; c < 3; ++c) s[c] = s[c] / ns;
  nn[0] = s[1] * tt[2] - s[2] * tt[1];
  nn[1] = s[2] * tt[0] - s[0] * tt[2];
  nn[2] = s[0] * tt[1] - s[1] * tt[0];
  R nl = sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
  for (int c = 0; c < 3; ++c) nn[c] = nn[c] / nl;
  t[0] = nn[1] * s[2] - nn[2] * s[1];
  t[1] = nn[2] * s[0] - nn[0] * s[2];
  t[2] = nn[0] * s[1] - nn[1] * s[0];
  R tl = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  for (int c = 0; c < 3; ++c) t[c] = t[c] / tl;
  R tc[4][2];
  for (int k = 0; k < 4; ++k) {
    R d0 = v[3 * k] - mgc[0], d1 = v[3 * k + 1] - mgc[1], d2 = v[3 * k + 2] - mgc[2];
    tc[k][0] = d0 * s[0] + d1 * s[1] + d2 * s[2];
    tc[k][1] = d0 * t[0] + d1 * t[1] + d2 * t[2];
  }
  R Ar(0.0), Mx(0.0), My(0.0);
  for (int k = 0; k < 4; ++k) {
    int kn = (k + 1) & 3;
    R xk = tc[k][0], yk = tc[k][1], xk1 = tc[kn][0], yk1 = tc[kn][1];
    Ar = Ar + (yk1 - yk) * (xk + xk1) / 2.0;
    Mx = Mx + (xk1 - xk) * (yk * yk + yk * yk1 + yk1 * yk1) / 6.0;
    My = My + (yk1 - yk) * (xk * xk + xk * xk1 + xk1 * xk1) / 6.0;
  }
  R clx = My / Ar, cly = -Mx / Ar;
  R qgc[3], lc[8];
  for (int c = 0; c < 3; ++c) qgc[c] = mgc[c] + clx * s[c] + cly * t[c];
  for (int k = 0; k < 4; ++k) {
    lc[2 * k] = tc[k][0] - clx;
    lc[2 * k + 1] = tc[k][1] - cly;
  }
  // field point in the local frame
  R d0 = p[0] - qgc[0], d1 = p[1] - qgc[1], d2 = p[2] - qgc[2];
  R x = s[0] * d0 + s[1] * d1 + s[2] * d2;
  R y = t[0] * d0 + t[1] * d1 + t[2] * d2;
  R z = nn[0] * d0 + nn[1] * d1 + nn[2] * d2;
  R sx[4], sy[4], r[4], e[4], h[4];
  for (int k = 0; k < 4; ++k) {
    sx[k] = x - lc[2 * k];
    sy[k] = y - lc[2 * k + 1];
    r[k] = sqrt(sx[k] * sx[k] + sy[k] * sy[k] + z * z);
    e[k] = sx[k] * sx[k] + z * z;
    h[k] = sx[k] * sy[k];
  }
  const bool inplane = fabs(val(z)) <= kBirkZTol;
  R s0(0.0), s1(0.0), s2(0.0), s3(0.0);
  for (int k = 0; k < 4; ++k) {
    const int kn = (k + 1) & 3;
    R dx = lc[2 * kn] - lc[2 * k];
    R dy = lc[2 * kn + 1] - lc[2 * k + 1];
    R dk = hypot(dx, dy);
    if (!(val(dk) <= kBirkDkTol)) {
      R rsum = r[k] + r[kn];
      R log_term = log((rsum - dk) / (rsum + dk));
      R lt_dk = log_term / dk;
      R vzk;
      if (!inplane) {
        vzk = atan_ratio_t(dy * e[k] - dx * h[k], dx * z * r[k]) - atan_ratio_t(dy * e[kn] - dx * h[kn], dx * z * r[kn]);
      } else {
        // In-plane field point (|z| <= tol): value 0 as in the primal, and the tangent the
        // reference keeps (_zero_primal_keep_tangent, rankine_vectorized.jl:36-37): at z = 0
        // the atan pair moves only with z, at the rate d(vz)/dz of the Birk Hessian
        // (hzz = lambda rsum / (rk rk1 rho), velocity_hessian, rankine_vectorized.jl:200-235).
        // Written this way it stays finite where the atan form is 0/0 (field point on the
        // line of an edge).
        const double sxk = val(sx[k]), syk = val(sy[k]), sxn = val(sx[kn]), syn = val(sy[kn]);
        const double rk = val(r[k]), rn = val(r[kn]), zv = val(z);
        const double lam = sxk * syn - sxn * syk;
        const double rho = rk * rn + sxk * sxn + syk * syn + zv * zv;
        const double rate = (rho > 0.0) ? lam * (rk + rn) / (rk * rn * rho) : 0.0;
        vzk = (z - zv) * rate;
      }
      s0 = s0 + ((sx[k] * dy - sy[k] * dx) * lt_dk + z * vzk);
      s1 = s1 + dy * lt_dk;
      s2 = s2 - dx * lt_dk;
      s3 = s3 + vzk;
    }
  }
  R phb = kMinusInv4Pi * s0;
  R vl0 = kMinusInv4Pi * s1, vl1 = kMinusInv4Pi * s2, vl2 = kMinusInv4Pi * s3;
  g[0] = kFourPi * (s[0] * vl0 + t[0] * vl1 + nn[0] * vl2);
  g[1] = kFourPi * (s[1] * vl0 + t[1] * vl1 + nn[1] * vl2);
  g[2] = kFourPi * (s[2] * vl0 + t[2] * vl1 + nn[2] * vl2);
  phi = -kFourPi * phb;
}

// near-field derivatives of (phi, g) w.r.t. the field point (3) and the corners (12):
// four forward sweeps of 4 directions each
__device__ void birk_near_jacobian(const double p[3], const double* v12, double dphi[15], double dg[3][15],
                                   double& phi, double g[3]) {
  for (int chunk = 0; chunk < 4; ++chunk) {
    Dn<4> P[3], V[12], ph, G[3];
    for (int c = 0; c < 3; ++c) P[c] = Dn<4>::var(p[c], c - 4 * chunk);
    for (int q = 0; q < 12; ++q) V[q] = Dn<4>::var(v12[q], 3 + q - 4 * chunk);
    birk_near_t(P, V, ph, G);
    if (chunk == 0) {
      phi = ph.v;
      g[0] = G[0].v; g[1] = G[1].v; g[2] = G[2].v;
    }
    for (int q = 0; q < 4; ++q) {
      int slot = 4 * chunk + q;
      if (slot >= 15) break;
      dphi[slot] = ph.d[q];
      for (int c = 0; c < 3; ++c) dg[c][slot] = G[c].d[q];
    }
  }
}

// sum of NV values over the CTA's threads (thread 0 gets the total)
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red /*NV * 4*/) {
#pragma unroll
  for (int q = 0; q < NV; ++q) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) red[q * 4 + warp] = v[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = red[q * 4] + red[q * 4 + 1] + red[q * 4 + 2] + red[q * 4 + 3];
  }
}

// ---------------------------------------------------------------------------
// static (Rankine + image, Birk) adjoint, real weights.  Direct: D = a (n_j . g) with g the
// source gradient of the panel integral at the field point (or its image).  Indirect: the
// field-point gradient of the same integral, -M g (M = diag(1, 1, -1) for the image point),
// with the field panel's normal: D = a (nv . g), nv = -M n_i.
// ---------------------------------------------------------------------------
template <bool DIRECT>
__global__ void __launch_bounds__(kRows) static_adjoint_kernel(AssemblyParams p, const double* __restrict__ RS,
                                                               const double* __restrict__ RD, GradPtrs gp) {
  __shared__ PanelRec sp[kCols];
  __shared__ double red[19 * 4];
  const int64_t n = p.n;
  const int64_t i0 = blockIdx.x * (int64_t)kRows;
  const int64_t i = i0 + threadIdx.x;
  const int64_t j0 = blockIdx.y * (int64_t)kCols;
  const int ncol = (int)((n - j0) < kCols ? (n - j0) : kCols);
  {
    const double2* src = reinterpret_cast<const double2*>(p.P + j0);
    double2* dst = reinterpret_cast<double2*>(sp);
    for (int q = threadIdx.x; q < ncol * 16; q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  const bool active = i < n;
  double ci[3] = {0, 0, 0}, ni[3] = {0, 0, 0};
  if (active)
    for (int c = 0; c < 3; ++c) { ci[c] = p.P[i].c[c]; ni[c] = p.P[i].n[c]; }
  const bool need_R = (p.gfs & MH_GF_RANKINE) != 0;
  const bool need_I = (p.gfs & (MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE)) != 0;
  const double image_sign = ((p.gfs & MH_GF_RANKINE_REFLECTED) ? 1.0 : 0.0) -
                            ((p.gfs & MH_GF_RANKINE_REFLECTED_NEGATIVE) ? 1.0 : 0.0);
  double gci[3] = {0, 0, 0}, gni[3] = {0, 0, 0};
  for (int jj = 0; jj < ncol; ++jj) {
    const int64_t j = j0 + jj;
    const PanelRec& Pj = sp[jj];
    // column accumulators: gc_j (3), gn_j (3), ga_j (1), gv_j (12)
    double col[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) col[q] = 0.0;
    if (active) {
      const double ws = RS[i + j * n], wd = RD[i + j * n];
      for (int img = 0; img < 2; ++img) {
        if (img == 0 && !need_R) continue;
        if (img == 1 && !need_I) continue;
        const double sgn = img ? image_sign : 1.0;
        const double pt[3] = {ci[0], ci[1], img ? -ci[2] : ci[2]};
        const double zf = img ? -1.0 : 1.0;  // d pt / d ci_z
        const double a = kMinusInv4Pi * sgn;
        double nv[3];
        if (DIRECT) { nv[0] = Pj.n[0]; nv[1] = Pj.n[1]; nv[2] = Pj.n[2]; }
        else { nv[0] = -ni[0]; nv[1] = -ni[1]; nv[2] = -zf * ni[2]; }
        double rb[3] = {pt[0] - Pj.c[0], pt[1] - Pj.c[1], pt[2] - Pj.c[2]};
        double r = sqrt(rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]);
        double g[3];  // source gradient of the integral (far field: A rb / r^3)
        if (r > 7 * Pj.radius) {
          // S = a A/r ; D = a A (nv . rb)/r^3
          const double r3 = r * r * r, r5 = r3 * r * r, A = Pj.area;
          const double nr = nv[0] * rb[0] + nv[1] * rb[1] + nv[2] * rb[2];
          for (int c = 0; c < 3; ++c) {
            const double dS = a * A * (-rb[c] / r3);
            const double dD = a * A * (nv[c] / r3 - 3.0 * nr * rb[c] / r5);
            const double gtot = ws * dS + wd * dD;  // d/d pt_c
            gci[c] += (c == 2 ? zf : 1.0) * gtot;
            col[c] -= gtot;  // d/d c_j = - d/d pt
            g[c] = A * rb[c] / r3;
          }
          col[6] += ws * a / r + wd * a * nr / r3;  // d/d A_j
        } else {
          double dphi[15], dg[3][15], phi;
          birk_near_jacobian(pt, p.V + 12 * j, dphi, dg, phi, g);
          for (int q = 0; q < 15; ++q) {
            const double dS = a * dphi[q];
            const double dD = a * (nv[0] * dg[0][q] + nv[1] * dg[1][q] + nv[2] * dg[2][q]);
            const double gtot = ws * dS + wd * dD;
            if (q < 3) gci[q] += (q == 2 ? zf : 1.0) * gtot;
            else col[7 + (q - 3)] += gtot;
          }
        }
        // d/d normal: the source's (direct) or the field panel's through nv = -M n_i (indirect)
        for (int c = 0; c < 3; ++c) {
          if (DIRECT) col[3 + c] += wd * a * g[c];
          else gni[c] -= wd * a * (c == 2 ? zf : 1.0) * g[c];
        }
      }
    }
    block_sum<19>(col, red);
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c) {
        atomicAdd(gp.gc + 3 * j + c, col[c]);
        atomicAdd(gp.gn + 3 * j + c, col[3 + c]);
      }
      atomicAdd(gp.ga + j, col[6]);
      for (int q = 0; q < 12; ++q) atomicAdd(gp.gv + 12 * j + q, col[7 + q]);
    }
  }
  if (active)
    for (int c = 0; c < 3; ++c) {
      atomicAdd(gp.gc + 3 * i + c, gci[c]);
      if (!DIRECT) atomicAdd(gp.gn + 3 * i + c, gni[c]);
    }
}

// ---------------------------------------------------------------------------
// wave adjoint (Wu or exact Delhommeau), one wavenumber, complex rank-nh weights
// ---------------------------------------------------------------------------
struct WaveWeights {
  const double2* lS;  // n x nh:  W^S_ij = c sum_h lS_h[i] rS_h[j]
  const double2* rS;
  const double2* lD;  //          W^D_ij = -c sum_h lD_h[i] rD_h[j]
  const double2* rD;
  int nh;
  double2 c;          // objective factor of this frequency
};

__device__ __forceinline__ double2 cmulz(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

constexpr int kWaveWu = 1, kWaveExact = 2;

// index of the unordered pair i <= j in the packed upper triangle
__device__ __forceinline__ int64_t packed_pair(int64_t i, int64_t j) { return j * (j + 1) / 2 + i; }

// The exact term and its first and second derivatives in (r, z) = (hh, vv) as duals, from
// G and dG/dr at the pair: dG/dz = G + 2/d (d = |(r, z)|, the relation the primal uses,
// exact_Guevel_Delhommeau.jl:52-59), so G_zz = G_z - 2 z/d^3 and G_rz = G_r - 2 r/d^3; the
// wave term is harmonic below the free surface, so G_rr = -G_r/r - G_zz.  For r <= 1e-6
// (where the primal zeroes every horizontal term) G_rr only ever meets zero weights and is
// set to 0.
__device__ void egd_terms_from_values(double2 G, double2 Gr, double r, double z, CR<Dn<2>>& GF, CR<Dn<2>>& Gh,
                                      CR<Dn<2>>& Gv) {
  const double d = hypot(r, z);
  const double id3 = 1.0 / (d * d * d);
  const double2 Gz = make_double2(G.x + 2 / d, G.y);
  const double2 Gzz = make_double2(Gz.x - 2.0 * z * id3, Gz.y);
  const double2 Grz = make_double2(Gr.x - 2.0 * r * id3, Gr.y);
  const double2 Grr = fabs(r) > 1e-6 ? make_double2(-Gr.x / r - Gzz.x, -Gr.y / r - Gzz.y) : make_double2(0.0, 0.0);
  GF.x.v = G.x;   GF.x.d[0] = Gr.x;  GF.x.d[1] = Gz.x;
  GF.y.v = G.y;   GF.y.d[0] = Gr.y;  GF.y.d[1] = Gz.y;
  Gh.x.v = Gr.x;  Gh.x.d[0] = Grr.x; Gh.x.d[1] = Grz.x;
  Gh.y.v = Gr.y;  Gh.y.d[0] = Grr.y; Gh.y.d[1] = Grz.y;
  Gv.x.v = Gz.x;  Gv.x.d[0] = Grz.x; Gv.x.d[1] = Gzz.x;
  Gv.y.v = Gz.y;  Gv.y.d[0] = Grz.y; Gv.y.d[1] = Gzz.y;
}

// contribution of one oriented pair (field f, source s) to the gradient:
// S = sc k a_s GF, D = sc a_s k^2 (u Gh + n3 Gv) with u = (n1 dx + n2 dy)/dis,
// (dx, dy) = source - field horizontal offset.
struct PairGrad {
  double gcf[3], gcs[3], gns[3], gas;
};

__device__ void wave_pair_grad(double k, double dx, double dy, double dis, double as, const double ns[3],
                               const CR<Dn<2>>& GF, const CR<Dn<2>>& Gh, const CR<Dn<2>>& Gv, double2 WS,
                               double2 WD, PairGrad& o) {
  const double sc = kMinusInv4Pi;
  const double hh = k * dis;
  // d/dhh and d/dvv of GF, Gh, Gv as complex numbers
  const double2 GFh = make_double2(GF.x.d[0], GF.y.d[0]), GFv = make_double2(GF.x.d[1], GF.y.d[1]);
  const double2 Ghh = make_double2(Gh.x.d[0], Gh.y.d[0]), Ghv = make_double2(Gh.x.d[1], Gh.y.d[1]);
  const double2 Gvh = make_double2(Gv.x.d[0], Gv.y.d[0]), Gvv = make_double2(Gv.x.d[1], Gv.y.d[1]);
  const double2 Ghx = make_double2(Gh.x.v, Gh.y.v), Gvx = make_double2(Gv.x.v, Gv.y.v);
  const double2 GFx = make_double2(GF.x.v, GF.y.v);
  const bool horiz = fabs(hh) > 1e-6;      // the primal zeroes the horizontal term below
  const double ux = horiz ? dx / dis : 0.0, uy = horiz ? dy / dis : 0.0;
  const double u = ns[0] * ux + ns[1] * uy;
  const double k2 = k * k;
  // S
  double2 dS_dhh = make_double2(sc * k * as * GFh.x, sc * k * as * GFh.y);
  double2 dS_dvv = make_double2(sc * k * as * GFv.x, sc * k * as * GFv.y);
  double2 dS_da = make_double2(sc * k * GFx.x, sc * k * GFx.y);
  // D
  auto lin = [](double a, double2 x, double b, double2 y) { return make_double2(a * x.x + b * y.x, a * x.y + b * y.y); };
  double2 Dcore = lin(u, Ghx, ns[2], Gvx);
  double2 dD_dhh = lin(sc * as * k2 * u, Ghh, sc * as * k2 * ns[2], Gvh);
  double2 dD_dvv = lin(sc * as * k2 * u, Ghv, sc * as * k2 * ns[2], Gvv);
  double2 dD_da = make_double2(sc * k2 * Dcore.x, sc * k2 * Dcore.y);
  double2 dD_dn0 = make_double2(sc * as * k2 * ux * Ghx.x, sc * as * k2 * ux * Ghx.y);
  double2 dD_dn1 = make_double2(sc * as * k2 * uy * Ghx.x, sc * as * k2 * uy * Ghx.y);
  double2 dD_dn2 = make_double2(sc * as * k2 * Gvx.x, sc * as * k2 * Gvx.y);
  // du / d(dx, dy)
  double du_dx = 0.0, du_dy = 0.0;
  if (horiz) {
    du_dx = (ns[0] - u * ux) / dis;
    du_dy = (ns[1] - u * uy) / dis;
  }
  // dhh / d(dx, dy).  hh = k |(dx, dy)| has a kink at dis = 0; inside the band where the
  // primal treats the pair as vertically aligned (hh <= 1e-6, which also catches centres
  // whose horizontal offset is rounding noise of order 1e-16) no direction is preferred and
  // the derivative is taken as 0, the central difference of the kink.
  const double dh_dx = horiz ? k * ux : 0.0, dh_dy = horiz ? k * uy : 0.0;
  auto re = [](double2 w, double2 d) { return w.x * d.x - w.y * d.y; };
  // d/d(dx): S via hh; D via hh and u
  double2 dD_ddx = make_double2(dD_dhh.x * dh_dx + sc * as * k2 * du_dx * Ghx.x,
                                dD_dhh.y * dh_dx + sc * as * k2 * du_dx * Ghx.y);
  double2 dD_ddy = make_double2(dD_dhh.x * dh_dy + sc * as * k2 * du_dy * Ghx.x,
                                dD_dhh.y * dh_dy + sc * as * k2 * du_dy * Ghx.y);
  double2 dS_ddx = make_double2(dS_dhh.x * dh_dx, dS_dhh.y * dh_dx);
  double2 dS_ddy = make_double2(dS_dhh.x * dh_dy, dS_dhh.y * dh_dy);
  const double gdx = re(WS, dS_ddx) + re(WD, dD_ddx);
  const double gdy = re(WS, dS_ddy) + re(WD, dD_ddy);
  const double gvv = re(WS, dS_dvv) + re(WD, dD_dvv);  // vv = k (z_f + z_s): d/dz = k each
  o.gcs[0] = gdx; o.gcs[1] = gdy; o.gcs[2] = k * gvv;
  o.gcf[0] = -gdx; o.gcf[1] = -gdy; o.gcf[2] = k * gvv;
  o.gns[0] = re(WD, dD_dn0); o.gns[1] = re(WD, dD_dn1); o.gns[2] = re(WD, dD_dn2);
  o.gas = re(WS, dS_da) + re(WD, dD_da);
}

// One thread per unordered pair (i <= j), both orientations.  DIRECT: the pair (field f,
// source s) enters D through the source normal and the offset s - f; indirect: through the
// field normal and the offset f - s.  WAVE: the Wu fits on duals, or the exact term from the
// packed values gv[2q] = G, gv[2q + 1] = dG/dr of pair q.
template <bool DIRECT, int WAVE>
__global__ void __launch_bounds__(kRows) wave_adjoint_kernel(AssemblyParams p, double k, WaveWeights w,
                                                             const double2* __restrict__ gv, GradPtrs gp) {
  __shared__ PanelRec sp[kCols];
  __shared__ double2 slS[kCols][kMaxH], srS[kCols][kMaxH], slD[kCols][kMaxH], srD[kCols][kMaxH];
  __shared__ double red[7 * 4];
  const int64_t n = p.n;
  const int64_t i0 = blockIdx.x * (int64_t)kRows;
  const int64_t j0 = blockIdx.y * (int64_t)kCols;
  if (i0 > j0 + kCols - 1) return;  // strictly below the diagonal
  const int64_t i = i0 + threadIdx.x;
  const int ncol = (int)((n - j0) < kCols ? (n - j0) : kCols);
  {
    const double2* src = reinterpret_cast<const double2*>(p.P + j0);
    double2* dst = reinterpret_cast<double2*>(sp);
    for (int q = threadIdx.x; q < ncol * 16; q += blockDim.x) dst[q] = src[q];
    for (int q = threadIdx.x; q < ncol * w.nh; q += blockDim.x) {
      int jj = q % ncol, h = q / ncol;
      slS[jj][h] = w.lS[(j0 + jj) + h * n];
      srS[jj][h] = w.rS[(j0 + jj) + h * n];
      slD[jj][h] = w.lD[(j0 + jj) + h * n];
      srD[jj][h] = w.rD[(j0 + jj) + h * n];
    }
  }
  __syncthreads();
  const bool active = i < n;
  double ci[3] = {0, 0, 0}, ni[3] = {0, 0, 0}, ai = 0.0;
  double2 lSi[kMaxH], rSi[kMaxH], lDi[kMaxH], rDi[kMaxH];
  if (active) {
    for (int c = 0; c < 3; ++c) { ci[c] = p.P[i].c[c]; ni[c] = p.P[i].n[c]; }
    ai = p.P[i].area;
    for (int h = 0; h < w.nh; ++h) {
      lSi[h] = w.lS[i + h * n]; rSi[h] = w.rS[i + h * n];
      lDi[h] = w.lD[i + h * n]; rDi[h] = w.rD[i + h * n];
    }
  }
  const double2 cS = w.c, cD = make_double2(-w.c.x, -w.c.y);
  double gci[3] = {0, 0, 0}, gni[3] = {0, 0, 0}, gai = 0.0;
  for (int jj = 0; jj < ncol; ++jj) {
    const int64_t j = j0 + jj;
    const PanelRec& Pj = sp[jj];
    double col[7] = {0, 0, 0, 0, 0, 0, 0};  // gc_j (3), gn_j (3), ga_j
    if (active && i <= j) {
      double hh, vv;
      reduced_coords(ci, Pj.c, k, hh, vv);
      CR<Dn<2>> GF, Gh, Gv;
      if (WAVE == kWaveWu) {
        wu_terms_t(Dn<2>::var(hh, 0), Dn<2>::var(vv, 1), GF, Gh, Gv);
      } else {
        const int64_t q = packed_pair(i, j);
        egd_terms_from_values(gv[2 * q], gv[2 * q + 1], hh, vv, GF, Gh, Gv);
      }
      const double dx = Pj.c[0] - ci[0], dy = Pj.c[1] - ci[1];
      const double dis = sqrt(dx * dx + dy * dy);
      // weights of (i, j) and (j, i)
      double2 WSij = make_double2(0, 0), WDij = WSij, WSji = WSij, WDji = WSij;
      for (int h = 0; h < w.nh; ++h) {
        WSij = zadd(WSij, cmulz(lSi[h], srS[jj][h]));
        WDij = zadd(WDij, cmulz(lDi[h], srD[jj][h]));
        WSji = zadd(WSji, cmulz(slS[jj][h], rSi[h]));
        WDji = zadd(WDji, cmulz(slD[jj][h], rDi[h]));
      }
      WSij = cmulz(cS, WSij);
      WSji = cmulz(cS, WSji);
      WDij = cmulz(cD, WDij);
      WDji = cmulz(cD, WDji);
      PairGrad g1;  // field i, source j
      if (DIRECT) {
        wave_pair_grad(k, dx, dy, dis, Pj.area, Pj.n, GF, Gh, Gv, WSij, WDij, g1);
        for (int c = 0; c < 3; ++c) { gci[c] += g1.gcf[c]; col[c] += g1.gcs[c]; col[3 + c] += g1.gns[c]; }
      } else {
        wave_pair_grad(k, -dx, -dy, dis, Pj.area, ni, GF, Gh, Gv, WSij, WDij, g1);
        for (int c = 0; c < 3; ++c) { gci[c] += g1.gcs[c]; col[c] += g1.gcf[c]; gni[c] += g1.gns[c]; }
      }
      col[6] += g1.gas;
      if (i != j) {
        PairGrad g2;  // field j, source i
        if (DIRECT) {
          wave_pair_grad(k, -dx, -dy, dis, ai, ni, GF, Gh, Gv, WSji, WDji, g2);
          for (int c = 0; c < 3; ++c) { col[c] += g2.gcf[c]; gci[c] += g2.gcs[c]; gni[c] += g2.gns[c]; }
        } else {
          wave_pair_grad(k, dx, dy, dis, ai, Pj.n, GF, Gh, Gv, WSji, WDji, g2);
          for (int c = 0; c < 3; ++c) { col[c] += g2.gcs[c]; gci[c] += g2.gcf[c]; col[3 + c] += g2.gns[c]; }
        }
        gai += g2.gas;
      }
    }
    block_sum<7>(col, red);
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c) {
        atomicAdd(gp.gc + 3 * j + c, col[c]);
        atomicAdd(gp.gn + 3 * j + c, col[3 + c]);
      }
      atomicAdd(gp.ga + j, col[6]);
    }
  }
  if (active) {
    for (int c = 0; c < 3; ++c) {
      atomicAdd(gp.gc + 3 * i + c, gci[c]);
      atomicAdd(gp.gn + 3 * i + c, gni[c]);
    }
    atomicAdd(gp.ga + i, gai);
  }
}

// G and dG/dr of the exact term for every unordered pair (i <= j) at wavenumber k, packed
// (pair q = j (j + 1)/2 + i at out[2q], out[2q + 1]), one warp per pair, with the primal's
// rules: the adaptive quadrature at the assembly's tolerance, the closed form at r = 0.
constexpr int kEgdWarps = 4;
__global__ void __launch_bounds__(32 * kEgdWarps) egd_pair_values_kernel(AssemblyParams p, double k, int64_t npairs,
                                                                         double2* __restrict__ out) {
  __shared__ double sw[kEgdWarps][8 * kGKWarpStack];
  const int warp = threadIdx.x >> 5;
  const int64_t q = blockIdx.x * (int64_t)kEgdWarps + warp;
  if (q >= npairs) return;  // warp-uniform
  int64_t j = (int64_t)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
  while (j * (j + 1) / 2 > q) --j;
  while ((j + 1) * (j + 2) / 2 <= q) ++j;
  const int64_t i = q - j * (j + 1) / 2;
  double r, z;
  reduced_coords(p.P[i].c, p.P[j].c, k, r, z);
  double2 G, Gr;
  if (r == 0.0) {
    if ((threadIdx.x & 31) != 0) return;
    const double2 f = egd_integrand<false>(0.0, 0.0, z);
    G = make_double2(2.0 * kPi * f.x, 2.0 * kPi * f.y);
    Gr = make_double2(0.0, 0.0);
  } else {
    egd_warp(r, z, p.quad_rtol, p.quad_atol, sw[warp], G, Gr);
    if ((threadIdx.x & 31) != 0) return;
  }
  out[2 * q] = G;
  out[2 * q + 1] = Gr;
}

// dS/dk and dD/dk of the exact term from the packed values: S = sc a k G(k dis, k Z) and
// D = sc a k^2 (u G_r + n_3 G_z) (u = n . offset / dis, zero for r <= 1e-6), so with
// (r, z) = k (dis, Z):  dS/dk = sc a (G + r G_r + z G_z),
// dD/dk = sc a k (2 (u G_r + n_3 G_z) + u (r G_rr + z G_rz) + n_3 (r G_rz + z G_zz)).
template <bool DIRECT>
__global__ void __launch_bounds__(kRows) egd_dk_kernel(AssemblyParams p, double k, const double2* __restrict__ gv,
                                                       double2* __restrict__ dS, double2* __restrict__ dD) {
  __shared__ PanelRec sp[kCols];
  const int64_t n = p.n;
  const int64_t i0 = blockIdx.x * (int64_t)kRows;
  const int64_t j0 = blockIdx.y * (int64_t)kCols;
  const int64_t i = i0 + threadIdx.x;
  const int ncol = (int)((n - j0) < kCols ? (n - j0) : kCols);
  {
    const double2* src = reinterpret_cast<const double2*>(p.P + j0);
    double2* dst = reinterpret_cast<double2*>(sp);
    for (int q = threadIdx.x; q < ncol * 16; q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  if (i >= n) return;
  double ci[3], ni[3];
  for (int c = 0; c < 3; ++c) { ci[c] = p.P[i].c[c]; ni[c] = p.P[i].n[c]; }
  for (int jj = 0; jj < ncol; ++jj) {
    const int64_t j = j0 + jj;
    const PanelRec& Pj = sp[jj];
    double r, z;
    reduced_coords(ci, Pj.c, k, r, z);
    const int64_t q = i <= j ? packed_pair(i, j) : packed_pair(j, i);
    CR<Dn<2>> GF, Gh, Gv;
    egd_terms_from_values(gv[2 * q], gv[2 * q + 1], r, z, GF, Gh, Gv);
    const double dx1 = DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0];
    const double dx2 = DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1];
    double nv[3];
    if (p.has_fixed) { nv[0] = p.fixed[0]; nv[1] = p.fixed[1]; nv[2] = p.fixed[2]; }
    else if (DIRECT) { nv[0] = Pj.n[0]; nv[1] = Pj.n[1]; nv[2] = Pj.n[2]; }
    else { nv[0] = ni[0]; nv[1] = ni[1]; nv[2] = ni[2]; }
    const double u = fabs(r) > 1e-6 ? k / r * (nv[0] * dx1 + nv[1] * dx2) : 0.0;
    const double a = kMinusInv4Pi * Pj.area;
    const double n3 = nv[2];
    dS[i + j * n] = make_double2(a * (GF.x.v + r * GF.x.d[0] + z * GF.x.d[1]),
                                 a * (GF.y.v + r * GF.y.d[0] + z * GF.y.d[1]));
    const double ux = fabs(r) > 1e-6 ? 1.0 : 0.0;  // the horizontal term is absent for r <= 1e-6
    dD[i + j * n] = make_double2(
        a * k * (2.0 * (u * Gh.x.v + n3 * Gv.x.v) + ux * u * (r * Gh.x.d[0] + z * Gh.x.d[1]) +
                 n3 * (r * Gv.x.d[0] + z * Gv.x.d[1])),
        a * k * (2.0 * (u * Gh.y.v + n3 * Gv.y.v) + ux * u * (r * Gh.y.d[0] + z * Gh.y.d[1]) +
                 n3 * (r * Gv.y.d[0] + z * Gv.y.d[1])));
  }
}

// out[i + j n] = alpha sum_h U[i + h n] conj(V[j + h n])  (a rank-nh outer product, N x N)
__global__ void outer_adj_kernel(int64_t n, int nh, const double2* __restrict__ U, const double2* __restrict__ V,
                                 double alpha, double2* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j = blockIdx.y;
  if (i >= n) return;
  double2 s = make_double2(0.0, 0.0);
  for (int h = 0; h < nh; ++h) {
    const double2 u = U[i + h * n], v = V[j + h * n];
    s.x += u.x * v.x + u.y * v.y;
    s.y += u.y * v.x - u.x * v.y;
  }
  out[i + j * n] = make_double2(alpha * s.x, alpha * s.y);
}

// dS_W/dk and dD_W/dk of the Wu term (the S, D entries of _assemble_wu_centers_loop,
// matrix_assembly.jl:343-369, differentiated in the wavenumber): hh = k dis and
// vv = k (z_i + z_j) carry their k-derivatives dis and z_i + z_j as one dual direction
// through the same fits, and k itself is the seeded variable of the prefactors.  One
// thread per ordered pair; the Rankine part does not depend on k.
template <bool DIRECT>
__global__ void __launch_bounds__(kRows) wave_dk_kernel(AssemblyParams p, const double* __restrict__ ks,
                                                        double2* __restrict__ dS, double2* __restrict__ dD) {
  __shared__ PanelRec sp[kCols];
  const int64_t n = p.n;
  const int64_t i0 = blockIdx.x * (int64_t)kRows;
  const int64_t j0 = blockIdx.y * (int64_t)kCols;
  const int64_t i = i0 + threadIdx.x;
  const int ncol = (int)((n - j0) < kCols ? (n - j0) : kCols);
  {
    const double2* src = reinterpret_cast<const double2*>(p.P + j0);
    double2* dst = reinterpret_cast<double2*>(sp);
    for (int q = threadIdx.x; q < ncol * 16; q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  if (i >= n) return;
  const double k = ks[0];
  double ci[3], ni[3];
  for (int c = 0; c < 3; ++c) { ci[c] = p.P[i].c[c]; ni[c] = p.P[i].n[c]; }
  for (int jj = 0; jj < ncol; ++jj) {
    const int64_t j = j0 + jj;
    const PanelRec& Pj = sp[jj];
    // _wu_reduced_hh_vv (wu.jl:7-18)
    const double d2 = (ci[0] - Pj.c[0]) * (ci[0] - Pj.c[0]) + (ci[1] - Pj.c[1]) * (ci[1] - Pj.c[1]);
    const double purt = 1e-18;
    const double dis = (d2 == 0) ? sqrt(d2 + purt * purt) - purt : sqrt(d2);
    const double zz = ci[2] + Pj.c[2];
    Dn<1> H(k * dis), V(k * zz), K = Dn<1>::var(k, 0);
    H.d[0] = dis;
    V.d[0] = zz;
    CR<Dn<1>> GF, Gh, Gv;
    wu_terms_t(H, V, GF, Gh, Gv);
    const double dx1 = DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0];
    const double dx2 = DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1];
    // _wu_sd (wu.jl:112-127) on duals: s = k GF a, g = k (k^2/hh dx Gh, k^2/hh dy Gh, k Gv)
    Dn<1> dr1(0.0), dr2(0.0);
    if (fabs(H.v) > 1e-6) {
      const Dn<1> f = K * K / H;
      dr1 = f * dx1;
      dr2 = f * dx2;
    }
    const Dn<1> sr = K * GF.x, si = K * GF.y;
    const Dn<1> g0r = K * (dr1 * Gh.x), g0i = K * (dr1 * Gh.y);
    const Dn<1> g1r = K * (dr2 * Gh.x), g1i = K * (dr2 * Gh.y);
    const Dn<1> g2r = K * (K * Gv.x), g2i = K * (K * Gv.y);
    double nv[3];
    if (p.has_fixed) { nv[0] = p.fixed[0]; nv[1] = p.fixed[1]; nv[2] = p.fixed[2]; }
    else if (DIRECT) { nv[0] = Pj.n[0]; nv[1] = Pj.n[1]; nv[2] = Pj.n[2]; }
    else { nv[0] = ni[0]; nv[1] = ni[1]; nv[2] = ni[2]; }
    const double a = kMinusInv4Pi * Pj.area;
    const int64_t idx = i + j * n;
    dS[idx] = make_double2(a * sr.d[0], a * si.d[0]);
    dD[idx] = make_double2(a * (nv[0] * g0r.d[0] + nv[1] * g1r.d[0] + nv[2] * g2r.d[0]),
                           a * (nv[0] * g0i.d[0] + nv[1] * g1i.d[0] + nv[2] * g2i.d[0]));
  }
}

// RS += Re(c sum_h lS_h rS_h^T), RD += Re(-c sum_h lD_h rD_h^T)
__global__ void weights_accumulate_kernel(int64_t n, WaveWeights w, double* __restrict__ RS, double* __restrict__ RD) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j = blockIdx.y;
  if (i >= n) return;
  double2 s = make_double2(0, 0), d = s;
  for (int h = 0; h < w.nh; ++h) {
    s = zadd(s, cmulz(w.lS[i + h * n], w.rS[j + h * n]));
    d = zadd(d, cmulz(w.lD[i + h * n], w.rD[j + h * n]));
  }
  s = cmulz(w.c, s);
  d = cmulz(w.c, d);
  RS[i + j * n] += s.x;
  RD[i + j * n] -= d.x;
}

// O(N) terms of one frequency (direct): force weights w_h = i rho omega (-n . dof_h) a and
// boundary conditions b_h = -i omega (n . dof_h) depend on n and a.
//   Re(c phi_h[i] dw_h[i]) + Re(c t_h[i] db_h[i]),  t_h = S^T lam_h
// O(N) terms of one frequency (direct) for cotangents c[q, col] (influenced q; columns: the
// n_rad radiating dofs, then the n_beta headings; J = sum Re(c F), F the forces of the
// columns plus, for the headings, the Froude-Krylov forces):
//   force weights  f_q = i rho omega (-n . dof_q) a, paired with psi_q = sum_col c[q, col] phi_col;
//   radiation      b_r = -i omega (n . dof_r), paired with t_r = S^T lam_r (lam = D^-T w);
//   diffraction    b_beta = -(v . n), v = omega e^{k z} e^{i k wbar} (cos b, sin b, -i), also
//                  paired with t_beta, depends on the centre through e^{kz + ikwbar};
//   Froude-Krylov  sum p_beta (-n . dof_q) a, p_beta = rho g e^{k z} e^{i k wbar}.
// Each thread owns one panel.
__global__ void rhs_adjoint_kernel(int64_t n, const double* __restrict__ N, const double* __restrict__ A,
                                   const double* __restrict__ C, const double* __restrict__ dofs,
                                   const int32_t* __restrict__ rad, int n_rad, const int32_t* __restrict__ inf,
                                   int n_inf, int n_beta, const double* __restrict__ betas, double omega, double rho,
                                   double gacc, const double2* __restrict__ cw, const double2* __restrict__ phi,
                                   const double2* __restrict__ t, double* __restrict__ gc, double* __restrict__ gn,
                                   double* __restrict__ ga, double* __restrict__ gd) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ncol = n_rad + n_beta;
  const double n0 = N[3 * i], n1 = N[3 * i + 1], n2 = N[3 * i + 2], a = A[i];
  const double k = omega * omega / gacc;
  double g0 = 0, g1 = 0, g2 = 0, gav = 0, c0 = 0, c1 = 0, c2 = 0;
  for (int q = 0; q < n_inf; ++q) {
    const double* dof = dofs + (int64_t)inf[q] * n * 3 + 3 * i;
    const double disp = n0 * dof[0] + n1 * dof[1] + n2 * dof[2];
    double2 psi = make_double2(0.0, 0.0);
    for (int r = 0; r < ncol; ++r) psi = zadd(psi, cmulz(cw[q + (int64_t)r * n_inf], phi[i + (int64_t)r * n]));
    // Re(psi * i s) = -s Im(psi):  d/dn with s = rho omega (-dof) a, d/da with s = rho omega (-disp)
    double re = -psi.y * rho * omega;  // coefficient of the real factor (-disp a) below
    // Froude-Krylov of every heading: Re(c p) times the same real factor, and its centre terms
    for (int b = 0; b < n_beta; ++b) {
      double sb, cb;
      sincos(betas[b], &sb, &cb);
      const double wbar = C[3 * i] * cb + C[3 * i + 1] * sb;
      double sw, cw_;
      sincos(k * wbar, &sw, &cw_);
      const double pa = rho * gacc * exp(k * C[3 * i + 2]);
      const double2 cp = cmulz(cw[q + (int64_t)(n_rad + b) * n_inf], make_double2(pa * cw_, pa * sw));
      re += cp.x;
      // d p / d centre = p (i k cos b, i k sin b, k):  Re(cp (i k cos b)) = -k cos b Im(cp)
      const double f = -disp * a;
      c0 += -k * cb * cp.y * f;
      c1 += -k * sb * cp.y * f;
      c2 += k * cp.x * f;
    }
    g0 += re * (-dof[0] * a);
    g1 += re * (-dof[1] * a);
    g2 += re * (-dof[2] * a);
    gav += re * (-disp);
    double* gdi = gd + ((int64_t)inf[q] * n + i) * 3;
    gdi[0] += re * (-n0 * a);
    gdi[1] += re * (-n1 * a);
    gdi[2] += re * (-n2 * a);
  }
  for (int r = 0; r < n_rad; ++r) {
    const double* dof = dofs + (int64_t)rad[r] * n * 3 + 3 * i;
    // b = -i omega disp:  Re(t (-i omega) x) = omega Im(t) x for x = dof (d/dn) and x = n (d/d dof)
    const double ty = t[i + (int64_t)r * n].y;
    g0 += omega * ty * dof[0];
    g1 += omega * ty * dof[1];
    g2 += omega * ty * dof[2];
    double* gdi = gd + ((int64_t)rad[r] * n + i) * 3;
    gdi[0] += omega * ty * n0;
    gdi[1] += omega * ty * n1;
    gdi[2] += omega * ty * n2;
  }
  for (int b = 0; b < n_beta; ++b) {
    double sb, cb;
    sincos(betas[b], &sb, &cb);
    const double wbar = C[3 * i] * cb + C[3 * i + 1] * sb;
    double sw, cw_;
    sincos(k * wbar, &sw, &cw_);
    const double e = omega * exp(k * C[3 * i + 2]);
    const double2 amp = make_double2(e * cw_, e * sw);  // v = amp (cos b, sin b, -i)
    const double2 v0 = make_double2(amp.x * cb, amp.y * cb), v1 = make_double2(amp.x * sb, amp.y * sb);
    const double2 v2 = make_double2(amp.y, -amp.x);
    const double2 tb = t[i + (int64_t)(n_rad + b) * n];
    // b = -(v . n):  d/dn = -v;  d/dc = b (i k cos b, i k sin b, k)
    g0 += -cmulz(tb, v0).x;
    g1 += -cmulz(tb, v1).x;
    g2 += -cmulz(tb, v2).x;
    const double2 bv = make_double2(-(v0.x * n0 + v1.x * n1 + v2.x * n2), -(v0.y * n0 + v1.y * n1 + v2.y * n2));
    const double2 tbv = cmulz(tb, bv);
    c0 += -k * cb * tbv.y;
    c1 += -k * sb * tbv.y;
    c2 += k * tbv.x;
  }
  gn[3 * i] += g0;
  gn[3 * i + 1] += g1;
  gn[3 * i + 2] += g2;
  ga[i] += gav;
  gc[3 * i] += c0;
  gc[3 * i + 1] += c1;
  gc[3 * i + 2] += c2;
}

// w_r[i] = conj(sum_q c[q, r] i rho omega (-n . dof_q) a)   (conjugated for the A^H solve)
__global__ void force_weights_kernel(int64_t n, const double* __restrict__ N, const double* __restrict__ A,
                                     const double* __restrict__ dofs, const int32_t* __restrict__ inf, int n_inf,
                                     int n_rad, const double2* __restrict__ cw, double omega, double rho,
                                     double2* __restrict__ wconj) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= n || r >= n_rad) return;
  double2 w = make_double2(0.0, 0.0);
  for (int q = 0; q < n_inf; ++q) {
    const double* dof = dofs + (int64_t)inf[q] * n * 3 + 3 * i;
    const double disp = N[3 * i] * dof[0] + N[3 * i + 1] * dof[1] + N[3 * i + 2] * dof[2];
    const double s = rho * omega * -disp * A[i];  // the force weight is i s
    const double2 c = cw[q + (int64_t)r * n_inf];
    w = zadd(w, make_double2(-c.y * s, c.x * s));
  }
  wconj[i + (int64_t)r * n] = make_double2(w.x, -w.y);
}

__global__ void conj_kernel(int64_t count, double2* __restrict__ x) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < count) x[q].y = -x[q].y;
}

}  // namespace

void launch_static_adjoint(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* RS,
                           const double* RD, double* gc, double* gn, double* ga, double* gv) {
  dim3 grid((unsigned)((p.n + kRows - 1) / kRows), (unsigned)((p.n + kCols - 1) / kCols));
  if (p.direct)
    MH_LAUNCH(lc, st, "adjoint_static",
              static_adjoint_kernel<true><<<grid, kRows, 0, st>>>(p, RS, RD, GradPtrs{gc, gn, ga, gv}));
  else
    MH_LAUNCH(lc, st, "adjoint_static",
              static_adjoint_kernel<false><<<grid, kRows, 0, st>>>(p, RS, RD, GradPtrs{gc, gn, ga, gv}));
}

void launch_wave_adjoint(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double k, const double2* lS,
                         const double2* rS, const double2* lD, const double2* rD, int nh, double2 c,
                         const double2* egd_values, double* gc, double* gn, double* ga, double* RS, double* RD) {
  WaveWeights w{lS, rS, lD, rD, nh, c};
  dim3 grid((unsigned)((p.n + kRows - 1) / kRows), (unsigned)((p.n + kCols - 1) / kCols));
  const GradPtrs gp{gc, gn, ga, nullptr};
  if (p.gfs & MH_GF_WU) {
    if (p.direct)
      MH_LAUNCH(lc, st, "adjoint_wave", (wave_adjoint_kernel<true, kWaveWu><<<grid, kRows, 0, st>>>(p, k, w, nullptr, gp)));
    else
      MH_LAUNCH(lc, st, "adjoint_wave", (wave_adjoint_kernel<false, kWaveWu><<<grid, kRows, 0, st>>>(p, k, w, nullptr, gp)));
  } else if (p.gfs & MH_GF_EXACT_DELHOMMEAU) {
    if (p.direct)
      MH_LAUNCH(lc, st, "adjoint_wave",
                (wave_adjoint_kernel<true, kWaveExact><<<grid, kRows, 0, st>>>(p, k, w, egd_values, gp)));
    else
      MH_LAUNCH(lc, st, "adjoint_wave",
                (wave_adjoint_kernel<false, kWaveExact><<<grid, kRows, 0, st>>>(p, k, w, egd_values, gp)));
  }
  dim3 g2((unsigned)((p.n + 255) / 256), (unsigned)p.n);
  MH_LAUNCH(lc, st, "adjoint_weights", weights_accumulate_kernel<<<g2, 256, 0, st>>>(p.n, w, RS, RD));
}

int64_t egd_packed_pairs(int64_t n) { return n * (n + 1) / 2; }

void launch_egd_pair_values(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double k, double2* out) {
  const int64_t m = egd_packed_pairs(p.n);
  if (m <= 0) return;
  MH_LAUNCH(lc, st, "egd_pair_values",
            egd_pair_values_kernel<<<(unsigned)((m + kEgdWarps - 1) / kEgdWarps), 32 * kEgdWarps, 0, st>>>(p, k, m, out));
}

void launch_egd_dk(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double k, const double2* values,
                   double2* dS, double2* dD) {
  dim3 grid((unsigned)((p.n + kRows - 1) / kRows), (unsigned)((p.n + kCols - 1) / kCols));
  if (p.direct)
    MH_LAUNCH(lc, st, "wave_dk", egd_dk_kernel<true><<<grid, kRows, 0, st>>>(p, k, values, dS, dD));
  else
    MH_LAUNCH(lc, st, "wave_dk", egd_dk_kernel<false><<<grid, kRows, 0, st>>>(p, k, values, dS, dD));
}

void launch_outer_adj(cudaStream_t st, LaunchCounter lc, int64_t n, int nh, const double2* U, const double2* V,
                      double alpha, double2* out) {
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)n);
  MH_LAUNCH(lc, st, "outer", outer_adj_kernel<<<grid, 256, 0, st>>>(n, nh, U, V, alpha, out));
}

void launch_rhs_adjoint(cudaStream_t st, LaunchCounter lc, int64_t n, const double* N, const double* A,
                        const double* C, const double* dofs, const int32_t* rad, int n_rad, const int32_t* inf,
                        int n_inf, int n_beta, const double* betas, double omega, double rho, double gacc,
                        const double2* cw, const double2* phi, const double2* t, double* gc, double* gn, double* ga,
                        double* gd) {
  MH_LAUNCH(lc, st, "adjoint_rhs",
            rhs_adjoint_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, N, A, C, dofs, rad, n_rad, inf, n_inf,
                                                                             n_beta, betas, omega, rho, gacc, cw, phi,
                                                                             t, gc, gn, ga, gd));
}

void launch_force_weights(cudaStream_t st, LaunchCounter lc, int64_t n, const double* N, const double* A,
                          const double* dofs, const int32_t* inf, int n_inf, int n_rad, const double2* cw,
                          double omega, double rho, double2* wconj) {
  dim3 grid((unsigned)((n + 127) / 128), (unsigned)n_rad);
  MH_LAUNCH(lc, st, "adjoint_force_weights",
            force_weights_kernel<<<grid, 128, 0, st>>>(n, N, A, dofs, inf, n_inf, n_rad, cw, omega, rho, wconj));
}

void launch_wave_dk(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* k_dev, double2* dS,
                    double2* dD) {
  dim3 grid((unsigned)((p.n + kRows - 1) / kRows), (unsigned)((p.n + kCols - 1) / kCols));
  if (p.direct)
    MH_LAUNCH(lc, st, "wave_dk", wave_dk_kernel<true><<<grid, kRows, 0, st>>>(p, k_dev, dS, dD));
  else
    MH_LAUNCH(lc, st, "wave_dk", wave_dk_kernel<false><<<grid, kRows, 0, st>>>(p, k_dev, dS, dD));
}

void launch_conj(cudaStream_t st, LaunchCounter lc, int64_t count, double2* x) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "conj", conj_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, x));
}

}  // namespace mh
