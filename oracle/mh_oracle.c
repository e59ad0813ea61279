/*
 * mh_oracle.c -- CPU FP64 restatement of MarineHydro.jl's dense-BEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the oracle that the CUDA library is
 * checked against (tests/, __graft_entry__.smoke(), bench.py cpu_baseline).
 * It is never linked into or called by libmarinehydro_cuda.so.
 *
 * Each function cites the reference source it restates, as file:line within the
 * MarineHydro.jl tree.  Arithmetic follows the reference's evaluation order where
 * that order is visible in the source; the build uses -ffp-contract=off so that
 * no multiply-add is fused (Julia does not contract a*b+c without muladd).
 *
 * Third-party arithmetic the reference calls and that is not in its tree:
 *   - SpecialFunctions.jl 2.5.0 besselj0/besselj1/bessely0/bessely1 (wu.jl:1),
 *     which wrap the fdlibm-derived openlibm j0/j1/y0/y1; here the C library's
 *     j0/j1/y0/y1 (glibc, also fdlibm-derived) are called.
 *   - SpecialFunctions.jl expint(::Complex) (exact_Guevel_Delhommeau.jl:5):
 *     restated from its published definition, DLMF 6.6.2 (power series of
 *     E1) and DLMF 6.9.1 (continued fraction), see or_exp_e1.
 *   - Integrals.jl 4.6.1 + HCubature 1.8.0 (exact_Guevel_Delhommeau.jl:8-13):
 *     1-D adaptive Gauss-Kronrod (7,15) bisection with a max-error heap; the
 *     rule's nodes/weights are Kronrod's published values (QUADPACK qk15).
 *   - LinearSolve.jl LUFactorization -> LAPACK zgetrf/zgetrs
 *     (matrix_assembly.jl:411-416): restated as LU with partial pivoting on
 *     |re|+|im| (izamax), first maximum wins.
 */
#include "mh_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

#define FOURPI 12.566370614359172       /* Julia 4pi */
#define MINV4PI (-0.07957747154594767)  /* Julia -1/4pi */
static const double PI = 3.141592653589793;

/* ------------------------------------------------------------------------- */
/* small vector helpers                                                      */
/* ------------------------------------------------------------------------- */
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double norm3(const double* a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
static inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static inline void normalize3(double* a) {
    double n = norm3(a);
    a[0] /= n; a[1] /= n; a[2] /= n;
}

/* ------------------------------------------------------------------------- */
/* Birk (2021) vectorized Rankine panel: green_functions/rankine_vectorized.jl */
/* ------------------------------------------------------------------------- */
#define BIRK_ZTOL 1e-14   /* rankine_vectorized.jl:24 */
#define BIRK_DKTOL 1e-14  /* rankine_vectorized.jl:25 */

/* _abs_ad (rankine_vectorized.jl:30): keeps -0.0 as -0.0 */
static inline double abs_ad(double x) { return x < 0.0 ? -x : x; }

/* _atan_ratio (rankine_vectorized.jl:42-45) */
static inline double atan_ratio(double num, double den) {
    double flipped = den < 0.0 ? -num : num;
    return atan2(flipped, abs_ad(den));
}

/* _inplane_atan (rankine_vectorized.jl:49-54) */
static inline double inplane_atan(double z, double datan) { return fabs(z) <= BIRK_ZTOL ? 0.0 : datan; }

/* birk_panel_geometry (rankine_vectorized.jl:79-137): compute_local_system,
   compute_temporary_panel_corners, compute_area_and_centroid, compute_qgc,
   compute_local_corners.  v12 = 4 corners x 3 coords (corner-major). */
void or_birk_panel_geometry(const double* v12, double* T, double* qgc, double* lc, double* area) {
    double mid[4][3], mgc[3], s[3], ttemp[3], n[3], t[3];
    for (int i = 0; i < 4; ++i) {
        int ip = (i + 1) % 4;
        for (int c = 0; c < 3; ++c) mid[i][c] = (v12[3 * i + c] + v12[3 * ip + c]) / 2;
    }
    for (int c = 0; c < 3; ++c) {
        mgc[c] = (mid[1][c] + mid[3][c]) / 2;
        s[c] = mid[1][c] - mid[3][c];
        ttemp[c] = mid[2][c] - mid[0][c];
    }
    normalize3(s);
    cross3(s, ttemp, n);
    normalize3(n);
    cross3(n, s, t);
    normalize3(t);
    for (int c = 0; c < 3; ++c) { T[c] = s[c]; T[3 + c] = t[c]; T[6 + c] = n[c]; }
    double tc[4][2];
    for (int k = 0; k < 4; ++k) {
        double d[3] = {v12[3 * k] - mgc[0], v12[3 * k + 1] - mgc[1], v12[3 * k + 2] - mgc[2]};
        tc[k][0] = dot3(d, s);
        tc[k][1] = dot3(d, t);
    }
    double A = 0.0, Mx = 0.0, My = 0.0;
    for (int k = 0; k < 4; ++k) {
        int kn = (k + 1) % 4;
        double xk = tc[k][0], yk = tc[k][1], xk1 = tc[kn][0], yk1 = tc[kn][1];
        double A_k = (yk1 - yk) * (xk + xk1) / 2;
        double Mx_k = (xk1 - xk) * (yk * yk + yk * yk1 + yk1 * yk1) / 6;
        double My_k = (yk1 - yk) * (xk * xk + xk * xk1 + xk1 * xk1) / 6;
        if (k == 0) { A = A_k; Mx = Mx_k; My = My_k; }
        else { A += A_k; Mx += Mx_k; My += My_k; }
    }
    double clx = My / A, cly = -Mx / A;
    for (int c = 0; c < 3; ++c) qgc[c] = mgc[c] + clx * s[c] + cly * t[c];
    for (int k = 0; k < 4; ++k) { lc[2 * k] = tc[k][0] - clx; lc[2 * k + 1] = tc[k][1] - cly; }
    *area = A;
}

/* velocity_potential, eq. (46) (rankine_vectorized.jl:140-164) */
double or_birk_velocity_potential(double x, double y, double z, const double* lc) {
    double sum = 0.0;
    for (int k = 0; k < 4; ++k) {
        int kn = (k + 1) % 4;
        double xk = lc[2 * k], yk = lc[2 * k + 1], xk1 = lc[2 * kn], yk1 = lc[2 * kn + 1];
        double dx = xk1 - xk, dy = yk1 - yk;
        double dk = hypot(dx, dy);
        double c = 0.0;
        if (!(dk <= BIRK_DKTOL)) {
            double rk = sqrt((x - xk) * (x - xk) + (y - yk) * (y - yk) + z * z);
            double rk1 = sqrt((x - xk1) * (x - xk1) + (y - yk1) * (y - yk1) + z * z);
            double ek = (x - xk) * (x - xk) + z * z, ek1 = (x - xk1) * (x - xk1) + z * z;
            double hk = (x - xk) * (y - yk), hk1 = (x - xk1) * (y - yk1);
            double log_term = log((rk + rk1 - dk) / (rk + rk1 + dk));
            double log_part = ((x - xk) * dy - (y - yk) * dx) / dk * log_term;
            double datan = inplane_atan(z, atan_ratio(dy * ek - dx * hk, dx * z * rk) -
                                               atan_ratio(dy * ek1 - dx * hk1, dx * z * rk1));
            double atan_part = z * datan;
            c = -(log_part + atan_part) / FOURPI;
        }
        sum = (k == 0) ? c : sum + c;
    }
    return sum;
}

/* velocity_derivatives, eqs. (47)-(49) (rankine_vectorized.jl:168-190) */
void or_birk_velocity_derivatives(double x, double y, double z, const double* lc, double* v) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = 0; k < 4; ++k) {
        int kn = (k + 1) % 4;
        double xk = lc[2 * k], yk = lc[2 * k + 1], xk1 = lc[2 * kn], yk1 = lc[2 * kn + 1];
        double dx = xk1 - xk, dy = yk1 - yk;
        double dk = hypot(dx, dy);
        double vx = 0, vy = 0, vz = 0;
        if (!(dk <= BIRK_DKTOL)) {
            double rk = sqrt((x - xk) * (x - xk) + (y - yk) * (y - yk) + z * z);
            double rk1 = sqrt((x - xk1) * (x - xk1) + (y - yk1) * (y - yk1) + z * z);
            double ek = (x - xk) * (x - xk) + z * z, ek1 = (x - xk1) * (x - xk1) + z * z;
            double hk = (x - xk) * (y - yk), hk1 = (x - xk1) * (y - yk1);
            double log_term = log((rk + rk1 - dk) / (rk + rk1 + dk));
            vx = (dy / dk) * log_term;
            vy = (-dx / dk) * log_term;
            vz = inplane_atan(z, atan_ratio(dy * ek - dx * hk, dx * z * rk) -
                                     atan_ratio(dy * ek1 - dx * hk1, dx * z * rk1));
        }
        if (k == 0) { s0 = vx; s1 = vy; s2 = vz; }
        else { s0 += vx; s1 += vy; s2 += vz; }
    }
    v[0] = MINV4PI * s0; v[1] = MINV4PI * s1; v[2] = MINV4PI * s2;
}

/* velocity_hessian, eqs. (50)-(58) (rankine_vectorized.jl:196-235); H column-major */
void or_birk_velocity_hessian(double x, double y, double z, const double* lc, double* H) {
    double S[9] = {0};
    for (int k = 0; k < 4; ++k) {
        int kn = (k + 1) % 4;
        double xk = lc[2 * k], yk = lc[2 * k + 1], xk1 = lc[2 * kn], yk1 = lc[2 * kn + 1];
        double dx = xk1 - xk, dy = yk1 - yk;
        double dk = hypot(dx, dy);
        if (dk <= BIRK_DKTOL) continue;
        double dxk = x - xk, dyk = y - yk, dxk1 = x - xk1, dyk1 = y - yk1;
        double rk = sqrt(dxk * dxk + dyk * dyk + z * z);
        double rk1 = sqrt(dxk1 * dxk1 + dyk1 * dyk1 + z * z);
        double rsum = rk + rk1;
        double den = rsum * rsum - dk * dk;
        double rhok = rk * rk1 + dxk * dxk1 + dyk * dyk1 + z * z;
        double lamk = dxk * dyk1 - dxk1 * dyk;
        double xterm = dxk / rk + dxk1 / rk1;
        double yterm = dyk / rk + dyk1 / rk1;
        double zterm = z / rk + z / rk1;
        double rhoden = (rk * rk1) * rhok;
        double hxx = 2 * dy / den * xterm, hyx = -2 * dx / den * xterm;
        double hxy = 2 * dy / den * yterm, hyy = -2 * dx / den * yterm;
        double hxz = 2 * dy / den * zterm, hyz = -2 * dx / den * zterm;
        double hzx = z * dy * rsum / rhoden, hzy = -z * dx * rsum / rhoden;
        double hzz = lamk * rsum / rhoden;
        double h[9] = {hxx, hyx, hzx, hxy, hyy, hzy, hxz, hyz, hzz};
        for (int q = 0; q < 9; ++q) S[q] += h[q];
    }
    for (int q = 0; q < 9; ++q) H[q] = MINV4PI * S[q];
}

/* birk_phi_and_velocity, fused eq. (46)+(47)-(49) (rankine_vectorized.jl:241-267) */
void or_birk_phi_and_velocity(double x, double y, double z, const double* lc, double* phi, double* v) {
    double sx[4], sy[4], r[4], e[4], h[4];
    for (int k = 0; k < 4; ++k) {
        sx[k] = x - lc[2 * k];
        sy[k] = y - lc[2 * k + 1];
        r[k] = sqrt(sx[k] * sx[k] + sy[k] * sy[k] + z * z);
        e[k] = sx[k] * sx[k] + z * z;
        h[k] = sx[k] * sy[k];
    }
    double s[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) {
        int kn = (k + 1) % 4;
        double dx = lc[2 * kn] - lc[2 * k];
        double dy = lc[2 * kn + 1] - lc[2 * k + 1];
        double dk = hypot(dx, dy);
        double c[4] = {0, 0, 0, 0};
        if (!(dk <= BIRK_DKTOL)) {
            double rsum = r[k] + r[kn];
            double log_term = log((rsum - dk) / (rsum + dk));
            double lt_dk = log_term / dk;
            double datan = atan_ratio(dy * e[k] - dx * h[k], dx * z * r[k]) -
                           atan_ratio(dy * e[kn] - dx * h[kn], dx * z * r[kn]);
            double vzk = inplane_atan(z, datan);
            double phik = (sx[k] * dy - sy[k] * dx) * lt_dk + z * vzk;
            c[0] = phik; c[1] = dy * lt_dk; c[2] = -dx * lt_dk; c[3] = vzk;
        }
        for (int q = 0; q < 4; ++q) s[q] = (k == 0) ? c[q] : s[q] + c[q];
    }
    *phi = MINV4PI * s[0];
    v[0] = MINV4PI * s[1]; v[1] = MINV4PI * s[2]; v[2] = MINV4PI * s[3];
}

/* _vrankine_from_geom (rankine_vectorized.jl:273-287) */
void or_vrankine_from_geom(const double* point, const double* sp, double source_radius, double source_area,
                           const double* T, const double* qgc, const double* lc, double* phi, double* grad) {
    double rb[3] = {point[0] - sp[0], point[1] - sp[1], point[2] - sp[2]};
    double r = norm3(rb);
    if (r > 7 * source_radius) {
        double r3 = r * r * r;
        *phi = source_area / r;
        grad[0] = (rb[0] / r3) * source_area;
        grad[1] = (rb[1] / r3) * source_area;
        grad[2] = (rb[2] / r3) * source_area;
        return;
    }
    double d[3] = {point[0] - qgc[0], point[1] - qgc[1], point[2] - qgc[2]};
    double fl[3];
    for (int i = 0; i < 3; ++i) fl[i] = T[3 * i] * d[0] + T[3 * i + 1] * d[1] + T[3 * i + 2] * d[2];
    double phb, vl[3];
    or_birk_phi_and_velocity(fl[0], fl[1], fl[2], lc, &phb, vl);
    for (int i = 0; i < 3; ++i) {
        double vg = T[i] * vl[0] + T[3 + i] * vl[1] + T[6 + i] * vl[2];
        grad[i] = FOURPI * vg;
    }
    *phi = -FOURPI * phb;
}

/* ------------------------------------------------------------------------- */
/* Delhommeau Rankine: green_functions/rankine.jl                            */
/* ------------------------------------------------------------------------- */
/* _delhommeau_atan (rankine_vectorized.jl:58-64) */
static inline double delhommeau_atan(double ANT, double DNT, double GZ, double radius) {
    double AT = atan2(ANT, DNT);
    return fabs(GZ) >= 1e-4 * radius ? AT : 0.0;
}
static inline double sign_ad(double x) { return x < 0.0 ? -1.0 : 1.0; }

/* integral(::DelhommeauRankine) (rankine.jl:33-71) */
double or_delhommeau_rankine_integral(const double* point, const double* v12, const double* center,
                                      const double* normal, double area, double radius) {
    double rb[3] = {point[0] - center[0], point[1] - center[1], point[2] - center[2]};
    double r = norm3(rb);
    if (r > 7 * radius) return area / r;
    double integral = 0.0;
    double GZ = dot3(rb, normal);
    double RR[4];
    for (int i = 0; i < 4; ++i) {
        double d[3] = {point[0] - v12[3 * i], point[1] - v12[3 * i + 1], point[2] - v12[3 * i + 2]};
        RR[i] = norm3(d);
    }
    for (int iv = 0; iv < 4; ++iv) {
        int in = (iv + 1) % 4;
        const double* cv = v12 + 3 * iv;
        const double* nv = v12 + 3 * in;
        double ctn[3] = {nv[0] - cv[0], nv[1] - cv[1], nv[2] - cv[2]};
        double seg = norm3(ctn);
        if (seg >= 1e-3 * radius) {
            double u[3] = {ctn[0] / seg, ctn[1] / seg, ctn[2] / seg}, gyx[3];
            cross3(normal, u, gyx);
            double pv[3] = {point[0] - cv[0], point[1] - cv[1], point[2] - cv[2]};
            double GY = dot3(pv, gyx);
            double ANT = 2 * GY * seg;
            double rs = RR[in] + RR[iv];
            double DNT = rs * rs - seg * seg + 2 * abs_ad(GZ) * rs;
            double AT = delhommeau_atan(ANT, DNT, GZ, radius);
            integral -= 2 * abs_ad(GZ) * AT;
            if (fabs(GY) > 1e-5) {
                double ANL = rs + seg, DNL = rs - seg;
                integral += GY * log(ANL / DNL);
            }
        }
    }
    return integral;
}

/* both_integral_and_integral_gradient(::DelhommeauRankine) (rankine.jl:73-131) */
void or_delhommeau_rankine_both(const double* point, const double* v12, const double* center, const double* normal,
                                double area, double radius, int wrt_first, double* out_int, double* out_grad) {
    double rb[3] = {point[0] - center[0], point[1] - center[1], point[2] - center[2]};
    double r = norm3(rb);
    double integral, g[3];
    if (r > 7 * radius) {
        double r3 = r * r * r;
        integral = area / r;
        for (int c = 0; c < 3; ++c) g[c] = (1 / r3 * rb[c]) * area;
    } else {
        integral = 0.0;
        g[0] = g[1] = g[2] = 0.0;
        double GZ = dot3(rb, normal);
        double RR[4], DRX[4][3];
        for (int i = 0; i < 4; ++i) {
            double d[3] = {point[0] - v12[3 * i], point[1] - v12[3 * i + 1], point[2] - v12[3 * i + 2]};
            RR[i] = norm3(d);
            for (int c = 0; c < 3; ++c) DRX[i][c] = d[c] / RR[i];
        }
        for (int iv = 0; iv < 4; ++iv) {
            int in = (iv + 1) % 4;
            const double* cv = v12 + 3 * iv;
            const double* nv = v12 + 3 * in;
            double ctn[3] = {nv[0] - cv[0], nv[1] - cv[1], nv[2] - cv[2]};
            double seg = norm3(ctn);
            if (!(seg >= 1e-3 * radius)) continue;
            double u[3] = {ctn[0] / seg, ctn[1] / seg, ctn[2] / seg}, GYX[3];
            cross3(normal, u, GYX);
            double pv[3] = {point[0] - cv[0], point[1] - cv[1], point[2] - cv[2]};
            double GY = dot3(pv, GYX);
            double ANT = 2 * GY * seg;
            double rs = RR[in] + RR[iv];
            double DNT = rs * rs - seg * seg + 2 * abs_ad(GZ) * rs;
            double ANL = rs + seg, DNL = rs - seg;
            double ALDEN = log(ANL / DNL);
            double AT = delhommeau_atan(ANT, DNT, GZ, radius);
            double ANLX[3], ANTX[3], DNTX[3];
            for (int c = 0; c < 3; ++c) {
                ANLX[c] = DRX[in][c] + DRX[iv][c];
                ANTX[c] = 2 * seg * GYX[c];
            }
            for (int c = 0; c < 3; ++c)
                DNTX[c] = 2 * (rs + abs_ad(GZ)) * ANLX[c] + 2 * sign_ad(GZ) * rs * normal[c];
            integral -= 2 * abs_ad(GZ) * AT;
            if (fabs(GY) > 1e-5) integral += GY * ALDEN;
            double q1 = GY * (DNL - ANL);
            double q2 = 2 * abs_ad(GZ);
            double den2 = ANT * ANT + DNT * DNT;
            for (int c = 0; c < 3; ++c) {
                double term = ALDEN * GYX[c] - 2 * sign_ad(GZ) * AT * normal[c] + q1 / (ANL * DNL) * ANLX[c] -
                              q2 * (ANTX[c] * DNT - DNTX[c] * ANT) / den2;
                g[c] = g[c] - term;
            }
        }
    }
    *out_int = integral;
    double s = wrt_first ? -1.0 : 1.0;
    for (int c = 0; c < 3; ++c) out_grad[c] = s * g[c];
}

/* ------------------------------------------------------------------------- */
/* Wu (Liang-Wu-Noblesse) wave term: green_functions/wu.jl                   */
/* ------------------------------------------------------------------------- */
static double gf_dfunc_c(double tt) { /* wu.jl:131-146 */
    double v = (3168.35 + -1590.27 * tt) * tt;
    v = (-2318.58 + v) * tt;
    v = (847.8 + v) * tt;
    v = (-148.24 + v) * tt;
    return 14.19 + v;
}
static double gf_dfunc_b(double tt) { /* wu.jl:149-172 */
    double v = (-76209.82 + 19923.28 * tt) * tt;
    v = (118879.26 + v) * tt;
    v = (-97014.11 + v) * tt;
    v = (44270.15 + v) * tt;
    v = (-11336.19 + v) * tt;
    v = (1565.35 + v) * tt;
    v = (-76.765 + v) * tt;
    v = (2.894 + v) * tt;
    return 1.11 + v;
}
static double gf_dfunc_a(double tt) { /* wu.jl:174-197 */
    double v = (-46688.0 + 12622.25 * tt) * tt;
    v = (68220.87 + v) * tt;
    v = (-48811.41 + v) * tt;
    v = (16370.75 + v) * tt;
    v = (-1187.71 + v) * tt;
    v = (-754.85 + v) * tt;
    v = (249.69 + v) * tt;
    v = (-24.53 + v) * tt;
    return 2.948 + v;
}
static double gf_func_d(double tt) { /* wu.jl:235-258 */
    double v = (128170.2 + -33744.6 * tt) * tt;
    v = (-205690.43 + v) * tt;
    v = (181856.75 + v) * tt;
    v = (-96293.05 + v) * tt;
    v = (31127.39 + v) * tt;
    v = (-6072.07 + v) * tt;
    v = (667.16 + v) * tt;
    v = (-40.97 + v) * tt;
    return 0.632 + v;
}
static double gf_func_c(double tt) { /* wu.jl:260-279 */
    double v = (9136.4 + -3272.62 * tt) * tt;
    v = (-9844.35 + v) * tt;
    v = (5155.67 + v) * tt;
    v = (-1397.89 + v) * tt;
    v = (209.653 + v) * tt;
    v = (-9.747 + v) * tt;
    return 1.268 + v;
}
static double gf_func_b(double tt) { /* wu.jl:281-304 */
    double v = (-29030.24 + 7671.22 * tt) * tt;
    v = (44894.06 + v) * tt;
    v = (-36618.81 + v) * tt;
    v = (17137.74 + v) * tt;
    v = (-4780.77 + v) * tt;
    v = (796.534 + v) * tt;
    v = (-67.92 + v) * tt;
    v = (5.737 + v) * tt;
    return 0.938 + v;
}
static double gf_func_a(double tt) { /* wu.jl:306-329 */
    double v = (21859.0 + -4838.6 * tt) * tt;
    v = (-41592.9 + v) * tt;
    v = (42002.57 + v) * tt;
    v = (-24314.21 + v) * tt;
    v = (8418.94 + v) * tt;
    v = (-1763.96 + v) * tt;
    v = (215.896 + v) * tt;
    v = (-13.328 + v) * tt;
    return 1.21 + v;
}

/* StruveH0 (wu.jl:368-400) */
double or_struve_h0(double xx) {
    if (xx <= 3.0) {
        double yy = (xx / 3.0) * (xx / 3.0);
        double h = 1.909859164 + (-1.909855001 + (0.687514637 + (-0.126164557 + (0.013828813 + -0.000876918 * yy) * yy) * yy) * yy) * yy;
        return h * (xx / 3.0);
    }
    double yy = (3.0 / xx) * (3.0 / xx);
    double c1 = 2.0 * (0.99999906 + (4.77228920 + (3.85542044 + 0.32303607 * yy) * yy) * yy);
    double c2 = PI * xx * (1.0 + (4.88331068 + (4.28957333 + 0.52120508 * yy) * yy) * yy);
    return c1 / c2 + y0(xx);
}

/* StruveH1 (wu.jl:404-435) */
double or_struve_h1(double xx) {
    if (xx <= 3.0) {
        double yy = (xx / 3.0) * (xx / 3.0);
        return (1.909859286 + (-1.145914713 + (0.294656958 + (-0.042070508 + (0.003785727 + -0.000207183 * yy) * yy) * yy) * yy) * yy) * yy;
    }
    double yy = (3.0 / xx) * (3.0 / xx);
    double c1 = 2.0 * (1.00000004 + (3.92205313 + (2.64893033 + 0.27450895 * yy) * yy) * yy);
    double c2 = PI * (1.0 + (3.81095112 + (2.26216956 + 0.10885141 * yy) * yy) * yy);
    return c1 / c2 + y1(xx);
}

/* _wu_wave_term_and_derivs (wu.jl:28-37) with GF_Func_L0 (:355-366),
   GF_Func_Lp (:339-353), GF_Func_W (:333-337), GF_Func_Ls (:221-233),
   GF_Func_Lsp (:207-219), GF_Func_Wh (:201-205). */
void or_wu_wave_term_and_derivs(double hh, double vv, double* GF, double* dGF_dhh, double* dGF_dvv) {
    double dd = sqrt(hh * hh + vv * vv);
    double alpha = -vv / dd;
    double beta = hh / dd;
    double rho = dd / (1 + dd);
    double dd2 = dd * dd, dd3 = dd * dd * dd;
    double omr = 1.0 - rho;
    double omr3 = omr * omr * omr;
    double ev = exp(vv);
    /* GF_Func_Lp */
    double A = gf_func_a(rho), B = gf_func_b(rho), C = gf_func_c(rho), D = gf_func_d(rho);
    double RR = (1.0 - beta) * A;
    RR -= beta * B;
    RR -= alpha * C / (1.0 + 6.0 * alpha * rho * (1.0 - rho));
    RR += beta * (1.0 - beta) * D;
    double Lp = rho * omr3 * RR;
    /* GF_Func_L0 */
    const double gama = 0.5772156649;
    double PP = log(0.5 * (dd - vv)) + gama - 2.0 * dd2;
    PP = ev * PP;
    PP = PP + dd2 - vv;
    double L0 = 2.0 * PP / (1.0 + dd3) + 2.0 * Lp;
    /* GF_Func_W = 2 pi complex(H0, -J0) exp(vv) */
    double H0 = or_struve_h0(hh), J0 = j0(hh);
    double twopi = 2 * PI;
    double Wr = (twopi * H0) * ev, Wi = (twopi * -J0) * ev;
    GF[0] = -L0 - Wr;
    GF[1] = -0.0 - Wi;
    /* GF_Func_Lsp */
    double dA = gf_dfunc_a(rho), dB = gf_dfunc_b(rho), dC = gf_dfunc_c(rho);
    double RS = beta * dA;
    RS -= (1.0 - alpha) * dB;
    RS += beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * dC;
    double Lsp = rho * omr3 * RS;
    /* GF_Func_Ls */
    double PS = (beta + hh) / (dd - vv);
    PS = PS - 2.0 * beta + 2.0 * ev * dd - hh;
    double QS = exp(-dd) * (1.0 - beta);
    QS = QS * (1.0 + dd / (1.0 + dd3));
    double Ls = 2.0 * PS / (1.0 + dd3) - 4.0 * QS + 2.0 * Lsp;
    /* GF_Func_Wh = 2 pi (2/pi - H1 + i J1) exp(vv) */
    double H1 = or_struve_h1(hh), J1 = j1(hh);
    double Whr = (twopi * (2 / PI - H1)) * ev, Whi = (twopi * J1) * ev;
    dGF_dhh[0] = -Ls - Whr;
    dGF_dhh[1] = -0.0 - Whi;
    dGF_dvv[0] = GF[0] + 2 / dd;
    dGF_dvv[1] = GF[1];
}

/* _wu_reduced_hh_vv (wu.jl:7-18); the same reduction as with_reduced_coordinates
   (abstract_greens_function.jl:117-138) */
static inline void reduced_coords(const double* x, const double* xi, double k, double* hh, double* vv) {
    double d2 = (x[0] - xi[0]) * (x[0] - xi[0]) + (x[1] - xi[1]) * (x[1] - xi[1]);
    const double purt = 1e-18;
    double dis = (d2 == 0) ? sqrt(d2 + purt * purt) - purt : sqrt(d2);
    *hh = k * dis;
    *vv = k * (x[2] + xi[2]);
}

/* _wu_sd (wu.jl:112-127) */
void or_wu_sd(const double* x, const double* xi, const double* n, double area2, double k, double dx1, double dx2,
              double* s, double* d) {
    double hh, vv;
    reduced_coords(x, xi, k, &hh, &vv);
    double GF[2], Gh[2], Gv[2];
    or_wu_wave_term_and_derivs(hh, vv, GF, Gh, Gv);
    double dr1 = 0.0, dr2 = 0.0;
    if (fabs(hh) > 1e-6) {
        dr1 = k * k / hh * dx1;
        dr2 = k * k / hh * dx2;
    }
    /* g = k .* (dr1*dGF_dhh, dr2*dGF_dhh, k*dGF_dvv) */
    double g[3][2];
    g[0][0] = k * (dr1 * Gh[0]); g[0][1] = k * (dr1 * Gh[1]);
    g[1][0] = k * (dr2 * Gh[0]); g[1][1] = k * (dr2 * Gh[1]);
    g[2][0] = k * (k * Gv[0]);   g[2][1] = k * (k * Gv[1]);
    s[0] = (k * GF[0]) * area2;
    s[1] = (k * GF[1]) * area2;
    double nr = n[0] * g[0][0] + n[1] * g[1][0] + n[2] * g[2][0];
    double ni = n[0] * g[0][1] + n[1] * g[1][1] + n[2] * g[2][1];
    d[0] = nr * area2;
    d[1] = ni * area2;
}

/* ------------------------------------------------------------------------- */
/* Exponential integral E1 for complex argument.                             */
/* Published method restated (not SpecialFunctions' code):                   */
/*   series  E1(z) = -gamma - log z - sum_{n>=1} (-z)^n / (n n!)  (DLMF 6.6.2) */
/*   CF      e^z E1(z) = 1/(z+1- 1^2/(z+3- 2^2/(z+5- ...)))        (DLMF 6.9.1, */
/*           even contraction), evaluated with the modified Lentz method.    */
/* The series is used where its cancellation loss exp(|z| + Re z) is small;  */
/* the continued fraction elsewhere.                                         */
/* ------------------------------------------------------------------------- */
static const double EULER_GAMMA = 0.57721566490153286061;

static cplx e1_series(cplx z) {
    cplx term = 1.0, sum = 0.0;
    for (int n = 1; n < 2000; ++n) {
        term *= -z / (double)n;
        cplx add = term / (double)n;
        sum += add;
        if (cabs(add) <= 1e-17 * cabs(sum)) break;
    }
    return -EULER_GAMMA - clog(z) - sum;
}

static cplx exp_e1_cf(cplx z) {
    const double tiny = 1e-300;
    cplx b = z + 1.0;
    cplx f = b;
    if (cabs(f) < tiny) f = tiny;
    cplx C = f, D = 0.0;
    for (int i = 1; i < 5000; ++i) {
        double a = -(double)i * (double)i;
        b += 2.0;
        D = b + a * D;
        if (cabs(D) < tiny) D = tiny;
        C = b + a / C;
        if (cabs(C) < tiny) C = tiny;
        D = 1.0 / D;
        cplx delta = C * D;
        f *= delta;
        if (cabs(delta - 1.0) < 1e-16) break;
    }
    return 1.0 / f;
}

#define E1_SERIES_LOSS 4.0

void or_exp_e1(double zr, double zi, double* gr, double* gi) {
    cplx z = CMPLX(zr, zi);
    cplx g;
    if (cabs(z) + zr < E1_SERIES_LOSS) g = cexp(z) * e1_series(z);
    else g = exp_e1_cf(z);
    *gr = creal(g);
    *gi = cimag(g);
}

void or_e1(double zr, double zi, double* er, double* ei) {
    cplx z = CMPLX(zr, zi);
    cplx e;
    if (cabs(z) + zr < E1_SERIES_LOSS) e = e1_series(z);
    else e = cexp(-z) * exp_e1_cf(z);
    *er = creal(e);
    *ei = cimag(e);
}

/* ------------------------------------------------------------------------- */
/* 1-D adaptive Gauss-Kronrod (7,15) quadrature, HCubature-style bisection  */
/* of the worst segment (exact_Guevel_Delhommeau.jl:8-13).                   */
/* ------------------------------------------------------------------------- */
static const double GK_X[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                               0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                               0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                               0.207784955007898467600689403773245, 0.0};
static const double GK_WK[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
static const double GK_WG[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                                0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

typedef cplx (*integrand_fn)(double theta, double r, double z);

typedef struct { double a, b; cplx val; double err; } gk_seg;

static void gk15(integrand_fn f, double r, double z, gk_seg* s) {
    double c = 0.5 * (s->a + s->b), h = 0.5 * (s->b - s->a);
    cplx fc = f(c, r, z);
    cplx Ik = GK_WK[7] * fc, Ig = GK_WG[3] * fc;
    for (int j = 0; j < 7; ++j) {
        double dx = h * GK_X[j];
        cplx f1 = f(c - dx, r, z), f2 = f(c + dx, r, z);
        Ik += GK_WK[j] * (f1 + f2);
        if (j & 1) Ig += GK_WG[j >> 1] * (f1 + f2);
    }
    s->val = Ik * h;
    s->err = cabs((Ik - Ig) * h);
}

static double g_egd_rtol = 1e-13, g_egd_atol = 1e-15;

void or_egd_set_tolerance(double rtol, double atol) { g_egd_rtol = rtol; g_egd_atol = atol; }

#define GK_MAXSEG 4096
static cplx adaptive_gk(integrand_fn f, double r, double z, double a, double b, double rtol, double atol) {
    gk_seg segs[GK_MAXSEG];
    int ns = 1;
    segs[0].a = a; segs[0].b = b;
    gk15(f, r, z, &segs[0]);
    cplx tot_i = segs[0].val;
    double E = segs[0].err;
    while (E > fmax(atol, rtol * cabs(tot_i)) && ns < GK_MAXSEG) {
        int w = 0;
        for (int i = 1; i < ns; ++i) if (segs[i].err > segs[w].err) w = i;
        gk_seg old = segs[w];
        double m = 0.5 * (old.a + old.b);
        gk_seg s1 = {old.a, m, 0.0, 0.0}, s2 = {m, old.b, 0.0, 0.0};
        gk15(f, r, z, &s1);
        gk15(f, r, z, &s2);
        segs[w] = s1;
        segs[ns++] = s2;
        tot_i += (s1.val + s2.val) - old.val;
        E += (s1.err + s2.err) - old.err;
    }
    cplx tot = 0.0;
    for (int i = 0; i < ns; ++i) tot += segs[i].val;
    return tot;
}

/* integrand of _dimless_wave_term (exact_Guevel_Delhommeau.jl:15-26) */
static cplx egd_integrand(double theta, double r, double z) {
    double ct = cos(theta);
    cplx zeta = CMPLX(z, r * ct);
    cplx ez = cexp(zeta);
    double gr, gi;
    or_exp_e1(z, r * ct, &gr, &gi);
    /* j_zeta = exp(zeta) * (E1(zeta)/pi + i) = g/pi + i exp(zeta) */
    cplx j = CMPLX(gr, gi) / PI + I * ez;
    return CMPLX(creal(j), creal(ez));
}

/* integrand of _d_dimless_wave_term_dr (exact_Guevel_Delhommeau.jl:35-46) */
static cplx egd_dr_integrand(double theta, double r, double z) {
    double ct = cos(theta);
    cplx zeta = CMPLX(z, r * ct);
    cplx ez = cexp(zeta);
    double gr, gi;
    or_exp_e1(z, r * ct, &gr, &gi);
    cplx j = CMPLX(gr, gi) / PI + I * ez;
    cplx a = I * ct * (j - 1.0 / (PI * zeta));
    cplx b = I * ct * ez;
    return CMPLX(creal(a), creal(b));
}

void or_egd_dimless(double r, double z, double rtol, double atol, double* G) {
    cplx v = 4.0 * adaptive_gk(egd_integrand, r, z, 0.0, PI / 2, rtol, atol);
    G[0] = creal(v); G[1] = cimag(v);
}

void or_egd_dimless_dr(double r, double z, double rtol, double atol, double* dG) {
    cplx v = 4.0 * adaptive_gk(egd_dr_integrand, r, z, 0.0, PI / 2, rtol, atol);
    dG[0] = creal(v); dG[1] = cimag(v);
}

/* with_reduced_coordinates(_derivative) (abstract_greens_function.jl:117-185) with
   both_greens_and_gradient_greens(::ExactGuevelDelhommeau) (exact_Guevel_Delhommeau.jl:52-59) */
static void egd_greens_and_gradient(const double* x, const double* xi, double k, int wrt_first, int want_grad,
                                    cplx* G, cplx* grad) {
    double r, z;
    reduced_coords(x, xi, k, &r, &z);
    double g[2];
    or_egd_dimless(r, z, g_egd_rtol, g_egd_atol, g);
    cplx GF = CMPLX(g[0], g[1]);
    *G = k * GF;
    if (!want_grad) return;
    double dg[2];
    or_egd_dimless_dr(r, z, g_egd_rtol, g_egd_atol, dg);
    cplx dGdr = CMPLX(dg[0], dg[1]);
    cplx dGdz = GF + 2 / hypot(r, z);
    double d1 = 0.0, d2 = 0.0;
    if (fabs(r) > 1e-6) {
        if (wrt_first) { d1 = k * k / r * (x[0] - xi[0]); d2 = k * k / r * (x[1] - xi[1]); }
        else { d1 = k * k / r * (xi[0] - x[0]); d2 = k * k / r * (xi[1] - x[1]); }
    }
    grad[0] = k * (d1 * dGdr);
    grad[1] = k * (d2 * dGdr);
    grad[2] = k * (k * dGdz);
}

/* ------------------------------------------------------------------------- */
/* point Green functions and single-kind panel integrals                     */
/* ------------------------------------------------------------------------- */
static void refl(const double* c, double* o) { o[0] = c[0]; o[1] = c[1]; o[2] = -c[2]; }

/* greens / gradient_greens: rankine.jl:17-31, rankine_vectorized.jl:295-301,
   rankine_reflected.jl:18-30, rankine_reflected_negative.jl:10-16, wu.jl:44-77,
   exact_Guevel_Delhommeau.jl:28-59 */
void or_point_greens(unsigned kind, const double* c1, const double* c2, double k, int wrt_first, double* g,
                     double* grad) {
    cplx G = 0, gv[3] = {0, 0, 0};
    if (kind & (OR_GF_RANKINE | OR_GF_DELHOMMEAU_RANKINE | OR_GF_RANKINE_REFLECTED |
                OR_GF_DELHOMMEAU_RANKINE_REFLECTED | OR_GF_RANKINE_REFLECTED_NEGATIVE)) {
        int reflected = (kind & (OR_GF_RANKINE_REFLECTED | OR_GF_DELHOMMEAU_RANKINE_REFLECTED |
                                 OR_GF_RANKINE_REFLECTED_NEGATIVE)) != 0;
        double a[3], b[3];
        /* reflected: greens(unreflected, e1, refl(e2)) for the wrt-first gradient,
           greens(unreflected, refl(e1), e2) otherwise (rankine_reflected.jl:18-30) */
        if (reflected && wrt_first) { memcpy(a, c1, sizeof a); refl(c2, b); }
        else if (reflected) { refl(c1, a); memcpy(b, c2, sizeof b); }
        else { memcpy(a, c1, sizeof a); memcpy(b, c2, sizeof b); }
        double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
        double r = norm3(d);
        G = 1 / r;
        double r3 = r * r * r;
        for (int c = 0; c < 3; ++c) {
            double gx = 1 / r3 * (b[c] - a[c]);
            gv[c] = wrt_first ? gx : -gx;
        }
        if (kind & OR_GF_RANKINE_REFLECTED_NEGATIVE) { G = -G; for (int c = 0; c < 3; ++c) gv[c] = -gv[c]; }
    } else if (kind & OR_GF_WU) {
        double hh, vv;
        reduced_coords(c1, c2, k, &hh, &vv);
        double GF[2], Gh[2], Gv[2];
        or_wu_wave_term_and_derivs(hh, vv, GF, Gh, Gv);
        G = k * CMPLX(GF[0], GF[1]);
        double d1 = 0, d2 = 0;
        if (fabs(hh) > 1e-6) {
            if (wrt_first) { d1 = k * k / hh * (c1[0] - c2[0]); d2 = k * k / hh * (c1[1] - c2[1]); }
            else { d1 = k * k / hh * (c2[0] - c1[0]); d2 = k * k / hh * (c2[1] - c1[1]); }
        }
        cplx dh = CMPLX(Gh[0], Gh[1]), dv = CMPLX(Gv[0], Gv[1]);
        gv[0] = k * (d1 * dh); gv[1] = k * (d2 * dh); gv[2] = k * (k * dv);
    } else if (kind & OR_GF_EXACT_DELHOMMEAU) {
        egd_greens_and_gradient(c1, c2, k, wrt_first, 1, &G, gv);
    }
    g[0] = creal(G); g[1] = cimag(G);
    for (int c = 0; c < 3; ++c) { grad[2 * c] = creal(gv[c]); grad[2 * c + 1] = cimag(gv[c]); }
}

/* integral / integral_gradient for one Green function kind and one pair
   (rankine_vectorized.jl:303-316, rankine.jl:33-136, rankine_reflected.jl:33-49,
   rankine_reflected_negative.jl:18-24, wu.jl:79-85, exact_Guevel_Delhommeau.jl:61-69) */
void or_pair_integrals(unsigned kind, const double* c1, const double* v12, const double* c2, const double* n2,
                       double a2, double r2, double k, int wrt_first, double* integral, double* grad) {
    cplx Ival = 0, gv[3] = {0, 0, 0};
    int reflected = (kind & (OR_GF_RANKINE_REFLECTED | OR_GF_DELHOMMEAU_RANKINE_REFLECTED |
                             OR_GF_RANKINE_REFLECTED_NEGATIVE)) != 0;
    double p[3];
    if (reflected) refl(c1, p); else memcpy(p, c1, sizeof p);
    if (kind & (OR_GF_RANKINE | OR_GF_RANKINE_REFLECTED | OR_GF_RANKINE_REFLECTED_NEGATIVE)) {
        double T[9], qgc[3], lc[8], ar, phi, g[3];
        or_birk_panel_geometry(v12, T, qgc, lc, &ar);
        or_vrankine_from_geom(p, c2, r2, a2, T, qgc, lc, &phi, g);
        Ival = phi;
        for (int c = 0; c < 3; ++c) gv[c] = wrt_first ? -g[c] : g[c];
    } else if (kind & (OR_GF_DELHOMMEAU_RANKINE | OR_GF_DELHOMMEAU_RANKINE_REFLECTED)) {
        double in, g[3];
        /* integral() for S and both_...[2] for the gradient (matrix_assembly.jl:72-78) */
        Ival = or_delhommeau_rankine_integral(p, v12, c2, n2, a2, r2);
        or_delhommeau_rankine_both(p, v12, c2, n2, a2, r2, wrt_first, &in, g);
        for (int c = 0; c < 3; ++c) gv[c] = g[c];
    } else if (kind & OR_GF_WU) {
        double hh, vv;
        reduced_coords(p, c2, k, &hh, &vv);
        double GF[2], Gh[2], Gv[2];
        or_wu_wave_term_and_derivs(hh, vv, GF, Gh, Gv);
        Ival = (k * CMPLX(GF[0], GF[1])) * a2;
        double d1 = 0, d2 = 0;
        if (fabs(hh) > 1e-6) {
            if (wrt_first) { d1 = k * k / hh * (p[0] - c2[0]); d2 = k * k / hh * (p[1] - c2[1]); }
            else { d1 = k * k / hh * (c2[0] - p[0]); d2 = k * k / hh * (c2[1] - p[1]); }
        }
        cplx dh = CMPLX(Gh[0], Gh[1]), dv = CMPLX(Gv[0], Gv[1]);
        gv[0] = k * (d1 * dh) * a2; gv[1] = k * (d2 * dh) * a2; gv[2] = k * (k * dv) * a2;
    } else if (kind & OR_GF_EXACT_DELHOMMEAU) {
        cplx G;
        egd_greens_and_gradient(p, c2, k, wrt_first, 1, &G, gv);
        Ival = G * a2;
        for (int c = 0; c < 3; ++c) gv[c] *= a2;
    }
    if (reflected && wrt_first) gv[2] = -gv[2];
    if (kind & OR_GF_RANKINE_REFLECTED_NEGATIVE) { Ival = -Ival; for (int c = 0; c < 3; ++c) gv[c] = -gv[c]; }
    integral[0] = creal(Ival); integral[1] = cimag(Ival);
    for (int c = 0; c < 3; ++c) { grad[2 * c] = creal(gv[c]); grad[2 * c + 1] = cimag(gv[c]); }
}

/* ------------------------------------------------------------------------- */
/* Assembly (matrix_assembly.jl:164-369)                                     */
/* ------------------------------------------------------------------------- */
#define BIRK_KINDS (OR_GF_RANKINE | OR_GF_RANKINE_REFLECTED | OR_GF_RANKINE_REFLECTED_NEGATIVE)
#define DELH_KINDS (OR_GF_DELHOMMEAU_RANKINE | OR_GF_DELHOMMEAU_RANKINE_REFLECTED)
#define WAVE_KINDS (OR_GF_WU | OR_GF_EXACT_DELHOMMEAU)

static inline double nsel(const double* fixed, int direct, const double* normals, int64_t i, int64_t j, int c) {
    /* _panel_or_fixed (matrix_assembly.jl:228-230) */
    if (fixed) return fixed[c];
    return direct ? normals[3 * j + c] : normals[3 * i + c];
}

/* _add_identity! (matrix_assembly.jl:234-245) on a complex matrix */
static void add_identity(int64_t n, double* D, const double* fixed, const double* normals) {
    for (int64_t i = 0; i < n; ++i) {
        double h = 0.5;
        if (fixed) h = 0.5 * dot3(fixed, normals + 3 * i);
        D[2 * (i + i * n)] += h;
    }
}

/* assemble_birk_rankine (matrix_assembly.jl:274-331) */
static void assemble_birk(int64_t n, const double* V, const double* C, const double* N, const double* A,
                          const double* R, unsigned gfs, int direct, int include_identity, const double* fixed,
                          double* S, double* D) {
    int need_R = (gfs & OR_GF_RANKINE) != 0;
    int need_I = (gfs & OR_GF_RANKINE_REFLECTED) != 0;
    int need_N = (gfs & OR_GF_RANKINE_REFLECTED_NEGATIVE) != 0;
    int image = need_I | need_N;
    double image_sign = (need_I ? 1.0 : 0.0) + (need_N ? -1.0 : 0.0);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t j = 0; j < n; ++j) {
        double T[9], qgc[3], lc[8], ar;
        or_birk_panel_geometry(V + 12 * j, T, qgc, lc, &ar);
        const double* c2 = C + 3 * j;
        for (int64_t i = 0; i < n; ++i) {
            const double* c1 = C + 3 * i;
            double nv[3] = {nsel(fixed, direct, N, i, j, 0), nsel(fixed, direct, N, i, j, 1),
                            nsel(fixed, direct, N, i, j, 2)};
            double s = 0.0, d = 0.0, phi, g[3];
            if (need_R) {
                or_vrankine_from_geom(c1, c2, R[j], A[j], T, qgc, lc, &phi, g);
                if (!direct) { g[0] = -g[0]; g[1] = -g[1]; g[2] = -g[2]; }
                s += phi;
                d += dot3(nv, g);
            }
            if (image) {
                double c1r[3] = {c1[0], c1[1], -c1[2]};
                or_vrankine_from_geom(c1r, c2, R[j], A[j], T, qgc, lc, &phi, g);
                double gr[3];
                if (direct) { gr[0] = g[0]; gr[1] = g[1]; gr[2] = g[2]; }
                else { gr[0] = -g[0]; gr[1] = -g[1]; gr[2] = g[2]; }
                s += image_sign * phi;
                d += image_sign * dot3(nv, gr);
            }
            int64_t idx = 2 * (i + j * n);
            S[idx] = MINV4PI * s; S[idx + 1] = 0.0;
            D[idx] = MINV4PI * d; D[idx + 1] = 0.0;
        }
    }
    if (include_identity) add_identity(n, D, fixed, N);
}

/* _assemble_wu_centers_loop (matrix_assembly.jl:343-369) */
static void assemble_wu(int64_t n, const double* C, const double* N, const double* A, double k, int direct,
                        int include_identity, const double* fixed, double* S, double* D) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t j = 0; j < n; ++j) {
        const double* c2 = C + 3 * j;
        for (int64_t i = 0; i < n; ++i) {
            const double* c1 = C + 3 * i;
            double nv[3] = {nsel(fixed, direct, N, i, j, 0), nsel(fixed, direct, N, i, j, 1),
                            nsel(fixed, direct, N, i, j, 2)};
            double dx1 = direct ? c2[0] - c1[0] : c1[0] - c2[0];
            double dx2 = direct ? c2[1] - c1[1] : c1[1] - c2[1];
            double s[2], d[2];
            or_wu_sd(c1, c2, nv, A[j], k, dx1, dx2, s, d);
            int64_t idx = 2 * (i + j * n);
            S[idx] = MINV4PI * s[0]; S[idx + 1] = MINV4PI * s[1];
            D[idx] = MINV4PI * d[0]; D[idx + 1] = MINV4PI * d[1];
        }
    }
    if (include_identity) add_identity(n, D, fixed, N);
}

/* assemble_matrices_broadcasting (matrix_assembly.jl:70-88) over a GF tuple,
   canonical tuple order: Rankine, RankineReflected, RankineReflectedNegative,
   DelhommeauRankine, DelhommeauRankineReflected, GFWu, ExactGuevelDelhommeau */
static void assemble_broadcast(int64_t n, const double* V, const double* C, const double* N, const double* A,
                               const double* R, double k, unsigned gfs, int direct, int include_identity,
                               const double* fixed, double* S, double* D) {
    static const unsigned order[7] = {OR_GF_RANKINE, OR_GF_RANKINE_REFLECTED, OR_GF_RANKINE_REFLECTED_NEGATIVE,
                                      OR_GF_DELHOMMEAU_RANKINE, OR_GF_DELHOMMEAU_RANKINE_REFLECTED, OR_GF_WU,
                                      OR_GF_EXACT_DELHOMMEAU};
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t j = 0; j < n; ++j) {
        for (int64_t i = 0; i < n; ++i) {
            cplx sI = 0, sg[3] = {0, 0, 0};
            int first = 1;
            for (int q = 0; q < 7; ++q) {
                if (!(gfs & order[q])) continue;
                double I2[2], g6[6];
                or_pair_integrals(order[q], C + 3 * i, V + 12 * j, C + 3 * j, N + 3 * j, A[j], R[j], k, !direct,
                                  I2, g6);
                cplx Iq = CMPLX(I2[0], I2[1]);
                if (first) { sI = Iq; for (int c = 0; c < 3; ++c) sg[c] = CMPLX(g6[2 * c], g6[2 * c + 1]); first = 0; }
                else { sI += Iq; for (int c = 0; c < 3; ++c) sg[c] += CMPLX(g6[2 * c], g6[2 * c + 1]); }
            }
            double nv[3] = {nsel(fixed, direct, N, i, j, 0), nsel(fixed, direct, N, i, j, 1),
                            nsel(fixed, direct, N, i, j, 2)};
            cplx dn = nv[0] * sg[0] + nv[1] * sg[1] + nv[2] * sg[2];
            int64_t idx = 2 * (i + j * n);
            cplx Sv = MINV4PI * sI, Dv = MINV4PI * dn;
            S[idx] = creal(Sv); S[idx + 1] = cimag(Sv);
            D[idx] = creal(Dv); D[idx + 1] = cimag(Dv);
        }
    }
    if (include_identity) add_identity(n, D, fixed, N);
}

/* assemble_matrices on a StaticArraysMesh (matrix_assembly.jl:167-222):
   partition into static (wavenumber-independent) and wave kinds; Birk-only static
   tuples use assemble_birk_rankine, others broadcasting; a Wu-only wave tuple uses
   the fused centres loop, others broadcasting; the identity goes on the static
   part when there is one; S = S_static + S_wave, D = D_static + D_wave. */
int or_assemble(int64_t n, const double* V, const double* C, const double* N, const double* A, const double* R,
                double k, unsigned gfs, int direct, int include_identity, const double* fixed, double* S, double* D,
                int nthreads) {
#ifdef _OPENMP
    int saved = omp_get_max_threads();
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    unsigned st = gfs & (BIRK_KINDS | DELH_KINDS);
    unsigned wv = gfs & WAVE_KINDS;
    size_t bytes = (size_t)(2 * n * n) * sizeof(double);
    if (st) {
        if ((st & DELH_KINDS) == 0) assemble_birk(n, V, C, N, A, R, st, direct, include_identity, fixed, S, D);
        else assemble_broadcast(n, V, C, N, A, R, 0.0, st, direct, include_identity, fixed, S, D);
    }
    if (wv) {
        int wave_identity = (!st) && include_identity;
        double* Sw = S;
        double* Dw = D;
        if (st) {
            Sw = (double*)malloc(bytes);
            Dw = (double*)malloc(bytes);
        }
        if (wv == OR_GF_WU) assemble_wu(n, C, N, A, k, direct, wave_identity, fixed, Sw, Dw);
        else assemble_broadcast(n, V, C, N, A, R, k, wv, direct, wave_identity, fixed, Sw, Dw);
        if (st) {
            for (int64_t q = 0; q < n * n; ++q) {
                S[2 * q] += Sw[2 * q]; S[2 * q + 1] += Sw[2 * q + 1];
                D[2 * q] += Dw[2 * q]; D[2 * q + 1] += Dw[2 * q + 1];
            }
            free(Sw);
            free(Dw);
        }
    }
    if (!st && !wv) memset(S, 0, bytes), memset(D, 0, bytes);
#ifdef _OPENMP
    omp_set_num_threads(saved);
#endif
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Dense complex LU with partial pivoting (LAPACK zgetrf/zgetrs semantics)   */
/* ------------------------------------------------------------------------- */
static inline double cabs1(cplx z) { return fabs(creal(z)) + fabs(cimag(z)); }

int or_lu_solve(int64_t n, int64_t nrhs, double* Ad, double* Bd) {
    cplx* A = (cplx*)Ad;
    cplx* B = (cplx*)Bd;
    int info = 0;
    for (int64_t j = 0; j < n; ++j) {
        int64_t p = j;
        double best = cabs1(A[j + j * n]);
        for (int64_t i = j + 1; i < n; ++i) {
            double v = cabs1(A[i + j * n]);
            if (v > best) { best = v; p = i; }
        }
        if (p != j) {
            for (int64_t c = 0; c < n; ++c) { cplx t = A[j + c * n]; A[j + c * n] = A[p + c * n]; A[p + c * n] = t; }
            for (int64_t c = 0; c < nrhs; ++c) { cplx t = B[j + c * n]; B[j + c * n] = B[p + c * n]; B[p + c * n] = t; }
        }
        cplx piv = A[j + j * n];
        if (piv == 0.0) { if (!info) info = (int)(j + 1); continue; }
        for (int64_t i = j + 1; i < n; ++i) A[i + j * n] /= piv;
        for (int64_t c = j + 1; c < n; ++c) {
            cplx u = A[j + c * n];
            if (u == 0.0) continue;
            for (int64_t i = j + 1; i < n; ++i) A[i + c * n] -= A[i + j * n] * u;
        }
    }
    if (info) return info;
    for (int64_t r = 0; r < nrhs; ++r) {
        cplx* b = B + r * n;
        for (int64_t j = 0; j < n; ++j) {           /* L y = b (unit lower) */
            cplx bj = b[j];
            if (bj == 0.0) continue;
            for (int64_t i = j + 1; i < n; ++i) b[i] -= A[i + j * n] * bj;
        }
        for (int64_t j = n - 1; j >= 0; --j) {      /* U x = y */
            b[j] /= A[j + j * n];
            cplx bj = b[j];
            for (int64_t i = 0; i < j; ++i) b[i] -= A[i + j * n] * bj;
        }
    }
    return 0;
}

/* _mulvec (matrix_assembly.jl:380-390): y = S * x for an n x nrhs x */
static void mulvec(int64_t n, int64_t nrhs, const cplx* S, const cplx* x, cplx* y) {
    for (int64_t c = 0; c < nrhs; ++c)
        for (int64_t i = 0; i < n; ++i) {
            cplx s = 0;
            for (int64_t j = 0; j < n; ++j) s += S[i + j * n] * x[j + c * n];
            y[i + c * n] = s;
        }
}

/* solve(D, S, bc; direct) (matrix_assembly.jl:436-449) */
int or_solve(int64_t n, int64_t nrhs, const double* D, const double* S, const double* bc, int direct, double* phi,
             double* sources) {
    size_t nn = (size_t)(n * n), nb = (size_t)(n * nrhs);
    cplx* A = (cplx*)malloc(nn * sizeof(cplx));
    memcpy(A, D, nn * sizeof(cplx));
    int info;
    if (direct) {
        mulvec(n, nrhs, (const cplx*)S, (const cplx*)bc, (cplx*)phi);
        info = or_lu_solve(n, nrhs, (double*)A, phi);
    } else {
        memcpy(sources, bc, nb * sizeof(cplx));
        info = or_lu_solve(n, nrhs, (double*)A, sources);
        mulvec(n, nrhs, (const cplx*)S, (const cplx*)sources, (cplx*)phi);
    }
    free(A);
    return info;
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
