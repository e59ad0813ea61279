"""Generate mh_special_tables.cuh: the polynomial tables of the joint J0, J1, Y0, Y1
evaluators (mh_bessel01.cuh, FP64 and FP32) and the Chebyshev form of the Wu fits for the
FP32 Wu term (mh_wu_f32.cuh).  Run once; the output is committed, mpmath is not needed to
build.

Bessel functions (all coefficients computed here from the functions' definitions with
mpmath at 40 digits):

* 0 <= x < 8: piecewise Chebyshev interpolation (Trefethen, Approximation Theory and
  Approximation Practice, ch. 3-8) on the sixteen intervals [q/2, q/2 + 1/2) for J0 and J1,
  and on [3, 8) for Y0 and Y1 (the Wu term needs Y only above x = 3), degree 11 at the
  first-kind Chebyshev points, converted to monomials in t = x - (q/2 + 1/4), |t| <= 1/4.
  Worst absolute error measured against mpmath: 6e-17.
* x >= 8: Hankel's modulus-phase form (DLMF 10.17.3):
      J_n(x) = sqrt(2/(pi x)) (P_n(x) cos w - Q_n(x) sin w),
      Y_n(x) = sqrt(2/(pi x)) (P_n(x) sin w + Q_n(x) cos w),   w = x - n pi/2 - pi/4,
  with P_n and Q_n / s (s = 8/x) interpolated as degree-12 polynomials of u = s^2 in [0, 1]
  (Chebyshev points, monomials in u - 1/2), P_n and Q_n taken from mpmath's J_n, Y_n by
  inverting the two relations.  Worst absolute error of P, Q/s: 3e-17.
* FP32 tables: the same construction at degree 6 (half-unit intervals) and 6 (Hankel), for
  errors below FP32 rounding.
* exp and log on the integer pipe (namespace fxq): 2^(j/32) and the degree-7 series of
  2^(g/32) for exp, degree-10 Chebyshev interpolants of log on the 32 intervals of [1, 2)
  for log, all as integers c 2^62; the integer evaluation is emulated bit for bit below.
* Fixed-point tables (namespace besq) of the same FP64 polynomials for the integer-pipe
  evaluator (mh_fixpoint.cuh): 64-bit integers c 2^61 (|values| < 4).  Below x = 8 the
  variable is z = 2 t in [-1/2, 1/2) (coefficient i divided by 2^i), above it z = (u - 1/2) / 2
  in [-1/4, 1/4] (coefficient i times 2^i), so that z 2^64 is a 64-bit integer and one
  Horner step is v <- c + floor(v z) (a signed 64 x 64 -> high 64 multiply).  The coefficients
  are rounded from the 40-digit values; the integer evaluation, emulated here bit for bit,
  is checked against mpmath below.

Wu fits: the polynomials A-D and dA-dC of Liang, Wu & Noblesse (wu.jl:131-197, 235-329) in
rho in [0, 1] have monomial coefficients up to 2e5 of alternating sign, so evaluated in FP32
their rounding is amplified ~1e5-fold.  The same polynomials written exactly in the
Chebyshev basis of s = 2 rho - 1 have coefficients below 15, and Clenshaw's recurrence in
FP32 keeps the error near FP32 rounding of the values.

Usage: python gen_special_tables.py  (writes mh_special_tables.cuh beside this script)
"""
from __future__ import annotations

import os

import mpmath as mp

mp.mp.dps = 40

DEG_LOW = 11     # per half-unit interval below x = 8
DEG_HANKEL = 12  # in u = (8/x)^2
DEG_LOW_F = 6    # FP32 tables
DEG_HANKEL_F = 6

# monomial coefficients (degree 0 first) of the Wu fits, wu.jl:131-197 (dA-dC) and
# 235-329 (A-D)
WU_FITS = {
    "A": [1.21, -13.328, 215.896, -1763.96, 8418.94, -24314.21, 42002.57, -41592.9, 21859.0, -4838.6],
    "B": [0.938, 5.737, -67.92, 796.534, -4780.77, 17137.74, -36618.81, 44894.06, -29030.24, 7671.22],
    "C": [1.268, -9.747, 209.653, -1397.89, 5155.67, -9844.35, 9136.4, -3272.62],
    "D": [0.632, -40.97, 667.16, -6072.07, 31127.39, -96293.05, 181856.75, -205690.43, 128170.2, -33744.6],
    "dA": [2.948, -24.53, 249.69, -754.85, -1187.71, 16370.75, -48811.41, 68220.87, -46688.0, 12622.25],
    "dB": [1.11, 2.894, -76.765, 1565.35, -11336.19, 44270.15, -97014.11, 118879.26, -76209.82, 19923.28],
    "dC": [14.19, -148.24, 847.8, -2318.58, 3168.35, -1590.27],
}


def cheb_monomials(f, a, b, n):
    """Degree-n Chebyshev interpolant of f on [a, b] as monomial coefficients in t = x - (a+b)/2."""
    mid, h = (a + b) / 2, (b - a) / 2
    th = [mp.pi * (k + mp.mpf(1) / 2) / (n + 1) for k in range(n + 1)]
    vals = [f(mid + h * mp.cos(t)) for t in th]
    c = [2 * mp.fsum(vals[k] * mp.cos(j * th[k]) for k in range(n + 1)) / (n + 1) for j in range(n + 1)]
    c[0] /= 2
    T = [[mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]]
    for j in range(2, n + 1):
        nxt = [mp.mpf(0)] * (j + 1)
        for i, v in enumerate(T[j - 1]):
            nxt[i + 1] += 2 * v
        for i, v in enumerate(T[j - 2]):
            nxt[i] -= v
        T.append(nxt)
    mono = [mp.mpf(0)] * (n + 1)
    for j in range(n + 1):
        for i, v in enumerate(T[j]):
            mono[i] += c[j] * v
    return [mono[i] / h ** i for i in range(n + 1)]


def hankel_pq(nu, u):
    """P_nu and Q_nu / s at u = (8/x)^2 (limits 1 and (4 nu^2 - 1)/64 at u = 0)."""
    if u == 0:
        return mp.mpf(1), mp.mpf(4 * nu * nu - 1) / 64
    x = 8 / mp.sqrt(u)
    w = x - nu * mp.pi / 2 - mp.pi / 4
    J, Y = mp.besselj(nu, x), mp.bessely(nu, x)
    f = mp.sqrt(mp.pi * x / 2)
    return f * (J * mp.cos(w) + Y * mp.sin(w)), f * (Y * mp.cos(w) - J * mp.sin(w)) / (8 / x)


def horner(co, t):
    v = mp.mpf(0)
    for c in reversed(co):
        v = v * t + c
    return v


QF = 61  # fraction bits of the fixed-point Bessel coefficients and values


def q_int(x, frac=QF):
    return int(mp.nint(mp.mpf(x) * mp.mpf(2) ** frac))


def fx_horner(cq, z):
    """v <- c + floor(v z / 2^64) from the highest degree down (the device's Horner step)."""
    v = cq[-1]
    for c in reversed(cq[:-1]):
        v = c + ((v * z) >> 64)
    return v


def fx_low(rows, x):
    """The device's fixed-point evaluation below x = 8 for a double x: X = floor(x 2^60),
    interval q = X >> 59, z = (X - q 2^59 - 2^58) 2^5."""
    X = int(mp.floor(mp.mpf(x) * 2 ** 60))
    q = min(X >> 59, 15)
    z = (X - (q << 59) - (1 << 58)) << 5
    return rows, q, z


def fx_bessel_tables(tabs_exact):
    """Fixed-point rows: below 8 (variable 2 t) coefficient i / 2^i, above 8 (variable
    (u - 1/2) / 2) coefficient i * 2^i; all as integers c 2^61."""
    out = {}
    for key in ("J0", "J1", "Y0", "Y1"):
        rows = tabs_exact[key]
        n = len(rows) // (DEG_LOW + 1)
        out[key] = [q_int(rows[r * (DEG_LOW + 1) + i] / mp.mpf(2) ** i) for r in range(n) for i in range(DEG_LOW + 1)]
    for key in ("P0", "Q0", "P1", "Q1"):
        out[key] = [q_int(c * mp.mpf(2) ** i) for i, c in enumerate(tabs_exact[key])]
    for key, vals in out.items():
        assert max(abs(v) for v in vals) < 2 ** 62, key
    return out


def fx_bessel_errors(fq):
    """Worst absolute error of the integer evaluation (emulated bit for bit) against mpmath."""
    J = {"J0": lambda x: mp.besselj(0, x), "J1": lambda x: mp.besselj(1, x),
         "Y0": lambda x: mp.bessely(0, x), "Y1": lambda x: mp.bessely(1, x)}
    worst_low = mp.mpf(0)
    for key, f in J.items():
        q0 = 6 if key[0] == "Y" else 0
        for k in range(q0 * 32, 8 * 64):
            x = float(mp.mpf(k) / 64 + mp.mpf(1) / 193)
            X = int(mp.floor(mp.mpf(x) * 2 ** 60))
            q = min(X >> 59, 15)
            z = (X - (q << 59) - (1 << 58)) << 5
            assert -2 ** 63 <= z < 2 ** 63
            row = fq[key][(q - q0) * (DEG_LOW + 1):(q - q0 + 1) * (DEG_LOW + 1)]
            worst_low = max(worst_low, abs(mp.mpf(fx_horner(row, z)) / 2 ** QF - f(x)))
    worst_hk = mp.mpf(0)
    for nu in (0, 1):
        for part in (0, 1):
            key = f"{'PQ'[part]}{nu}"
            for k in range(0, 65):
                u = mp.mpf(k) / 64
                w = float(u) - 0.5
                z = int(mp.floor(mp.mpf(w) * 2 ** 63)) if w >= 0 else -int(mp.floor(-mp.mpf(w) * 2 ** 63))
                worst_hk = max(worst_hk, abs(mp.mpf(fx_horner(fq[key], z)) / 2 ** QF - hankel_pq(nu, mp.mpf(w) + mp.mpf(1) / 2)[part]))
    return worst_low, worst_hk


# ---- exp and log on the integer pipe (mh_fixpoint.cuh) ------------------------------------
EXP_DEG = 7   # 2^(g/32), g in [0, 1)
LOG_DEG = 10  # log(1 + j/32 + u/32), u in [0, 1), per interval j = 0..31


def fx_exp_tables():
    tab = [q_int(mp.mpf(2) ** (mp.mpf(j) / 32), 62) for j in range(32)]
    c = mp.log(2) / 32
    poly = [q_int(c ** k / mp.factorial(k), 62) for k in range(EXP_DEG + 1)]
    log2e = int(mp.nint(mp.log(mp.e, 2) * mp.mpf(2) ** 63))
    return tab, poly, log2e


def fx_log_tables():
    rows = []
    for j in range(32):
        a = 1 + mp.mpf(j) / 32
        f = lambda u, a=a: mp.log(a + u / 32)
        cx = cheb_monomials(f, mp.mpf(0), mp.mpf(1), LOG_DEG)  # monomials in t = u - 1/2
        # re-expand in u: sum c_i (u - 1/2)^i
        from math import comb
        cu = [mp.mpf(0)] * (LOG_DEG + 1)
        for i, ci in enumerate(cx):
            for m in range(i + 1):
                cu[m] += ci * comb(i, m) * (-mp.mpf(1) / 2) ** (i - m)
        rows += [q_int(c, 62) for c in cu]
    ln2 = int(mp.nint(mp.log(2) * mp.mpf(2) ** 64))
    return rows, ln2


def mulhi_su(v, t):
    return (v * t) >> 64


def emu_exp(x, tab, poly, log2e):
    """Bit-for-bit model of fx::exp (x <= 0, x > -745): see mh_fixpoint.cuh."""
    s = 60 if abs(x) < 8 else 53
    X = int(mp.mpf(x) * 2 ** s)  # truncation toward zero, as to_q
    prod = X * log2e             # exact 128-bit signed product
    n = prod >> (64 + s - 1)
    F = (prod >> (s - 1)) & ((1 << 64) - 1)
    j = F >> 59
    G = (F << 5) & ((1 << 64) - 1)
    v = poly[-1]
    for c in reversed(poly[:-1]):
        v = c + mulhi_su(v, G)
    R = (tab[j] * v) >> 64
    return mp.mpf(R) * mp.mpf(2) ** (n - 60)


def emu_log(w, rows, ln2):
    """Bit-for-bit model of fx::log (w > 0 normal, before the final rounding)."""
    m, e = mp.frexp(mp.mpf(w))   # w = m 2^e, m in [1/2, 1)
    n = int(e) - 1
    frac = int((m * 2 - 1) * 2 ** 52)
    j = frac >> 47
    U = (frac << 17) & ((1 << 64) - 1)
    row = rows[j * (LOG_DEG + 1):(j + 1) * (LOG_DEG + 1)]
    v = row[-1]
    for c in reversed(row[:-1]):
        v = c + mulhi_su(v, U)
    total = n * ln2 + (v << 2)
    return mp.mpf(total) / mp.mpf(2) ** 64


def fmt_int(vals):
    return ",\n    ".join(", ".join(f"{v}LL" for v in vals[i:i + 3]) for i in range(0, len(vals), 3))


def fmt(vals, single=False):
    f = (lambda v: f"{float(mp.mpf(v)):.9e}f") if single else (lambda v: f"{float(v):.17e}")
    return ",\n    ".join(", ".join(f(v) for v in vals[i:i + 4]) for i in range(0, len(vals), 4))


def bessel_tables(deg_low, deg_hankel, single):
    """Coefficient rows of the low-region tables and the Hankel polynomials, rounded to the
    target precision, and the worst absolute error of the rounded polynomials."""
    rnd = (lambda c: float(__import__("numpy").float32(float(c)))) if single else float
    J = [lambda x: mp.besselj(0, x), lambda x: mp.besselj(1, x)]
    Y = [lambda x: mp.bessely(0, x), lambda x: mp.bessely(1, x)]
    tabs, exact, worst_low, worst_hk = {}, {}, mp.mpf(0), mp.mpf(0)
    for name, fs, q0 in (("J", J, 0), ("Y", Y, 6)):
        for nu in (0, 1):
            rows, rows_x = [], []
            for q in range(q0, 16):
                a = mp.mpf(q) / 2
                cx = cheb_monomials(fs[nu], a, a + mp.mpf(1) / 2, deg_low)
                cf = [rnd(c) for c in cx]
                for k in range(33):
                    x = a + mp.mpf(k) / 64
                    worst_low = max(worst_low, abs(horner(cf, float(x - a - mp.mpf(1) / 4)) - fs[nu](x)))
                rows += cf
                rows_x += cx
            tabs[f"{name}{nu}"] = rows
            exact[f"{name}{nu}"] = rows_x
    for nu in (0, 1):
        for part in (0, 1):
            g = lambda u, nu=nu, part=part: hankel_pq(nu, u)[part]
            cx = cheb_monomials(g, mp.mpf(0), mp.mpf(1), deg_hankel)
            cf = [rnd(c) for c in cx]
            for k in range(1, 65):
                u = mp.mpf(k) / 64
                worst_hk = max(worst_hk, abs(horner(cf, float(u - mp.mpf(1) / 2)) - g(u)))
            tabs[f"{'PQ'[part]}{nu}"] = cf
            exact[f"{'PQ'[part]}{nu}"] = cx
    return tabs, exact, worst_low, worst_hk


def wu_fit_chebyshev(mono):
    """Exact Chebyshev coefficients (basis T_j(2 rho - 1)) of a monomial polynomial in rho."""
    n = len(mono) - 1
    # rho = (s + 1) / 2: expand in s, then monomials in s -> Chebyshev in s
    from math import comb
    sco = [mp.mpf(0)] * (n + 1)
    for k, c in enumerate(mono):
        for m in range(k + 1):
            sco[m] += mp.mpf(c) * comb(k, m) / mp.mpf(2) ** k
    # s^m = sum_j b_{m,j} T_j(s) (descending recursion on the Chebyshev series of s * T_j)
    cheb = [mp.mpf(0)] * (n + 1)
    for m, c in enumerate(sco):
        t = [mp.mpf(0)] * (n + 1)
        t[0] = mp.mpf(1)
        for _ in range(m):  # multiply the series by s: s T_0 = T_1, s T_j = (T_{j+1} + T_{j-1}) / 2
            u = [mp.mpf(0)] * (n + 1)
            for j, v in enumerate(t):
                if v == 0:
                    continue
                if j == 0:
                    u[1] += v
                else:
                    u[j + 1] += v / 2
                    u[j - 1] += v / 2
            t = u
        for j in range(n + 1):
            cheb[j] += c * t[j]
    return cheb


def clenshaw(c, s):
    b1 = b2 = mp.mpf(0)
    for cj in reversed(c[1:]):
        b1, b2 = 2 * s * b1 - b2 + cj, b1
    return s * b1 - b2 + c[0]


def main():
    tabs, tabx, wl, wh = bessel_tables(DEG_LOW, DEG_HANKEL, False)
    print("FP64 Bessel: worst abs error low region", mp.nstr(wl, 3), "Hankel P, Q/s", mp.nstr(wh, 3))
    tabq = fx_bessel_tables(tabx)
    wlq, whq = fx_bessel_errors(tabq)
    print("fixed-point Bessel: worst abs error low region", mp.nstr(wlq, 3), "Hankel P, Q/s", mp.nstr(whq, 3))
    assert wlq < 1e-16 and whq < 1e-16
    etab, epoly, log2e = fx_exp_tables()
    import random
    rng = random.Random(7)
    xs = [-rng.uniform(0, 1) for _ in range(400)] + [-10 ** rng.uniform(-12, 2.8) for _ in range(400)]
    xs += [0.0, -1e-300, -7.999999999, -8.0, -744.0, -0.5, -2.0 ** -40]
    worst_e = max(abs(emu_exp(x, etab, epoly, log2e) / mp.exp(x) - 1) for x in xs)
    ltab, ln2 = fx_log_tables()
    ws = [10 ** rng.uniform(-300, 300) for _ in range(300)] + [rng.uniform(0.5, 2) for _ in range(300)]
    ws += [1.0, 1 + 2.0 ** -52, 2 - 2.0 ** -52, 0.5, 3.0]
    worst_l = max(abs(emu_log(w, ltab, ln2) - mp.log(w)) for w in ws)
    print("fixed-point exp: worst relative error", mp.nstr(worst_e, 3), "; log: worst absolute error", mp.nstr(worst_l, 3))
    assert worst_e < 5e-17 and worst_l < 4e-17
    tabf, _, wlf, whf = bessel_tables(DEG_LOW_F, DEG_HANKEL_F, True)
    print("FP32 Bessel: worst abs error low region", mp.nstr(wlf, 3), "Hankel P, Q/s", mp.nstr(whf, 3))
    wu = {}
    for key, mono in WU_FITS.items():
        ch = wu_fit_chebyshev(mono)
        worst = max(abs(clenshaw(ch, 2 * mp.mpf(k) / 200 - 1) - horner([mp.mpf(c) for c in mono], mp.mpf(k) / 200))
                    for k in range(201))
        assert worst < 1e-25, (key, worst)
        wu[key] = ch
        print(f"Wu fit {key}: Chebyshev coefficients up to {float(max(abs(c) for c in ch)):.3g}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mh_special_tables.cuh")
    with open(out, "w") as fh:
        fh.write("// mh_special_tables.cuh -- generated by gen_special_tables.py (mpmath, 40 digits); do not\n")
        fh.write("// edit.  Polynomial coefficients, lowest degree first, of the J0, J1, Y0, Y1 evaluators\n")
        fh.write("// (mh_bessel01.cuh; FP64, fixed-point and FP32) and the Chebyshev form of the Wu fits\n")
        fh.write("// (mh_wu_f32.cuh).\n")
        fh.write("#pragma once\n\nnamespace mh {\n")
        for ns, tb, dl, dh, single in (("bes", tabs, DEG_LOW, DEG_HANKEL, False),
                                       ("besf", tabf, DEG_LOW_F, DEG_HANKEL_F, True)):
            ty = "float" if single else "double"
            fh.write(f"namespace {ns} {{\n\n")
            fh.write(f"constexpr int kLowTerms = {dl + 1};     // per half-unit interval, in t = x - (q/2 + 1/4)\n")
            fh.write(f"constexpr int kHankelTerms = {dh + 1};  // in u - 1/2, u = (8/x)^2\n\n")
            for key in ("J0", "J1"):
                fh.write(f"// {key} on [q/2, q/2 + 1/2), q = 0..15\n")
                fh.write(f"__device__ const {ty} k{key}[16 * kLowTerms] = {{\n    {fmt(tb[key], single)}}};\n\n")
            for key in ("Y0", "Y1"):
                fh.write(f"// {key} on [q/2, q/2 + 1/2), q = 6..15 (row q - 6)\n")
                fh.write(f"__device__ const {ty} k{key}[10 * kLowTerms] = {{\n    {fmt(tb[key], single)}}};\n\n")
            for key, what in (("P0", "P0"), ("Q0", "Q0 / s"), ("P1", "P1"), ("Q1", "Q1 / s")):
                fh.write(f"// {what} for x >= 8\n")
                fh.write(f"__constant__ {ty} k{key}[kHankelTerms] = {{\n    {fmt(tb[key], single)}}};\n\n")
            fh.write(f"}}  // namespace {ns}\n\n")
        fh.write("namespace besq {\n\n")
        fh.write(f"constexpr int kFrac = {QF};  // coefficients and values are integers v 2^-kFrac\n\n")
        for key in ("J0", "J1"):
            fh.write(f"// {key} on [q/2, q/2 + 1/2), q = 0..15, in z = 2 (x - q/2 - 1/4)\n")
            fh.write(f"__device__ const long long k{key}[16 * bes::kLowTerms] = {{\n    {fmt_int(tabq[key])}}};\n\n")
        for key in ("Y0", "Y1"):
            fh.write(f"// {key} on [q/2, q/2 + 1/2), q = 6..15 (row q - 6), in z = 2 (x - q/2 - 1/4)\n")
            fh.write(f"__device__ const long long k{key}[10 * bes::kLowTerms] = {{\n    {fmt_int(tabq[key])}}};\n\n")
        for key, what in (("P0", "P0"), ("Q0", "Q0 / s"), ("P1", "P1"), ("Q1", "Q1 / s")):
            fh.write(f"// {what} for x >= 8, in z = (u - 1/2) / 2\n")
            fh.write(f"__constant__ long long k{key}[bes::kHankelTerms] = {{\n    {fmt_int(tabq[key])}}};\n\n")
        fh.write("}  // namespace besq\n\n")
        fh.write("namespace fxq {\n\n")
        fh.write("// exp on the integer pipe: 2^(j/32) 2^62, j = 0..31; 2^(g/32) = sum_k c_k g^k, c_k 2^62,\n")
        fh.write("// g in [0, 1); log2(e) 2^63\n")
        fh.write(f"__device__ const long long kExp2Tab[32] = {{\n    {fmt_int(etab)}}};\n")
        fh.write(f"constexpr int kExpDeg = {EXP_DEG};\n")
        fh.write(f"__constant__ long long kExp2Poly[{EXP_DEG + 1}] = {{\n    {fmt_int(epoly)}}};\n")
        fh.write(f"constexpr unsigned long long kLog2eQ63 = {log2e}ULL;\n\n")
        fh.write("// log on the integer pipe: log(1 + j/32 + u/32) = sum_k c_k u^k on u in [0, 1), c_k 2^62,\n")
        fh.write("// row j = 0..31; ln 2 2^64\n")
        fh.write(f"constexpr int kLogTerms = {LOG_DEG + 1};\n")
        fh.write(f"__device__ const long long kLogTab[32 * kLogTerms] = {{\n    {fmt_int(ltab)}}};\n")
        fh.write(f"constexpr unsigned long long kLn2Q64 = {ln2}ULL;\n\n")
        fh.write("}  // namespace fxq\n\n")
        fh.write("namespace wuf {\n\n")
        fh.write("// Wu fits (wu.jl:131-197, 235-329) as sum_j c_j T_j(2 rho - 1), FP32\n")
        for key in WU_FITS:
            fh.write(f"__constant__ float kCheb{key}[{len(wu[key])}] = {{\n    {fmt(wu[key], True)}}};\n")
        fh.write("\n}  // namespace wuf\n}  // namespace mh\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
