"""Generate fte_e1_coeffs.h: polynomial pieces for the exponential integral E1.

The GPU near-field kernels evaluate E1(x), x = xi^2 r^2 > 0, as

  x <  1:  E1(x) = -gamma - ln x + x * R(x),   R(x) = Ein(x)/x
           Ein(x) = sum_{k>=1} (-1)^{k+1} x^k / (k k!)   (Abramowitz & Stegun 5.1.11)
  x >= 1:  E1(x) = exp(-x) * G(x) / x,          G(x) = x e^x E1(x)

R is entire; G is smooth on [1, inf) and tends to 1.  Each is approximated by
truncated Chebyshev series (computed here in 60-digit arithmetic with mpmath,
by Chebyshev-Gauss interpolation at degree+1 nodes), converted to monomials
in the interval-local variable t in [-1, 1] for Horner evaluation:

  R on [0, 1]:                one piece
  G on [2^k (1 + q/4), 2^k (1 + (q+1)/4)),  k = 0..9, q = 0..3   (40 pieces)

The piece for x >= 1 is selected from the binary exponent k and the top two
mantissa bits q of x.  For x >= 1024, E1(x) < 1e-447 underflows to 0.

The Stokeslet real-space weight 0.5 E1(x) - exp(-x) is evaluated for x >= 1 as
exp(-x) K(x) with K(x) = 0.5 e^x E1(x) - 1 on eighth-octave pieces (80 pieces,
degree 10).  exp(-x) itself is evaluated from 2^(-n/64) (a 64-entry table),
n = round(64 x / ln 2), times the degree-6 Taylor polynomial of exp(-r),
r = x - n ln2/64 (Cody-Waite split of ln2/64); this header holds the table and
the constants.

Run:  python fasttools2d_gb300/csrc/gen_e1_coeffs.py   (needs mpmath; the
generated header is committed so the build does not.)
"""
import os

import mpmath as mp

mp.mp.dps = 60
DEG_R = 11
DEG_G = 12
DEG_K = 10


def cheb_fit(fun, a, b, deg):
    """Chebyshev interpolation coefficients of fun on [a, b] (degree deg)."""
    n = deg + 1
    nodes = [mp.cos(mp.pi * (j + mp.mpf(1) / 2) / n) for j in range(n)]
    vals = [fun((b - a) / 2 * t + (b + a) / 2) for t in nodes]
    c = []
    for k in range(n):
        s = mp.fsum(vals[j] * mp.cos(mp.pi * k * (j + mp.mpf(1) / 2) / n) for j in range(n))
        c.append(2 * s / n)
    c[0] /= 2
    return c


def cheb_to_mono(c):
    """Convert sum c_k T_k(t) to monomial coefficients in t."""
    n = len(c)
    T = [[mp.mpf(0)] * n for _ in range(n)]
    T[0][0] = mp.mpf(1)
    if n > 1:
        T[1][1] = mp.mpf(1)
    for k in range(2, n):
        for i in range(n):
            v = -T[k - 2][i]
            if i > 0:
                v += 2 * T[k - 1][i - 1]
            T[k][i] = v
    mono = [mp.fsum(c[k] * T[k][i] for k in range(n)) for i in range(n)]
    return mono


def ein_over_x(x):
    if x == 0:
        return mp.mpf(1)
    return (mp.e1(x) + mp.euler + mp.log(x)) / x


def g_fun(x):
    return x * mp.exp(x) * mp.e1(x)


def k_fun(x):
    return mp.exp(x) * mp.e1(x) / 2 - 1


def horner(mono, t):
    acc = mp.mpf(0)
    for a in reversed(mono):
        acc = acc * t + a
    return acc


def main():
    out = []
    out.append("/* Generated by gen_e1_coeffs.py -- do not edit.  Piecewise polynomial")
    out.append(" * coefficients (monomials in the interval-local t in [-1,1], constant")
    out.append(" * term first) for the exponential integral E1; see that script. */")
    out.append("/* The includer defines FTE_E1_STORAGE_R / FTE_E1_STORAGE_G (e.g. __constant__). */")
    out.append("#pragma once")
    out.append(f"#define FTE_E1_DEG_R {DEG_R}")
    out.append(f"#define FTE_E1_DEG_G {DEG_G}")
    out.append("#define FTE_E1_NPIECE_G 40")
    cR = cheb_fit(ein_over_x, mp.mpf(0), mp.mpf(1), DEG_R)
    mR = cheb_to_mono(cR)
    err_r = max(abs(horner(mR, 2 * x - 1) - ein_over_x(x)) for x in [mp.mpf(i) / 997 for i in range(998)])
    out.append(f"/* R(x) = Ein(x)/x on [0,1], t = 2x - 1; max abs err of the truncation {float(err_r):.3e} */")
    out.append("FTE_E1_STORAGE_R double fte_e1_coef_r[FTE_E1_DEG_R + 1] = {")
    out.append("    " + ", ".join(mp.nstr(a, 20, min_fixed=-1, max_fixed=-1) for a in mR) + "};")
    out.append("/* G(x) = x e^x E1(x) on quarter-octave pieces; t = (x - mid)/half */")
    out.append("FTE_E1_STORAGE_G double fte_e1_coef_g[FTE_E1_NPIECE_G][FTE_E1_DEG_G + 1] = {")
    worst = 0.0
    for k in range(10):
        for q in range(4):
            a = mp.mpf(2) ** k * (1 + mp.mpf(q) / 4)
            b = mp.mpf(2) ** k * (1 + mp.mpf(q + 1) / 4)
            c = cheb_fit(g_fun, a, b, DEG_G)
            m = cheb_to_mono(c)
            mid, half = (a + b) / 2, (b - a) / 2
            e = max(abs(horner(m, (x - mid) / half) / g_fun(x) - 1) for x in [a + (b - a) * i / 199 for i in range(200)])
            worst = max(worst, float(e))
            out.append("    {" + ", ".join(mp.nstr(v, 20, min_fixed=-1, max_fixed=-1) for v in m) + "},")
    out.append("};")
    out.append(f"/* worst relative truncation error of the G pieces: {worst:.3e} */")

    # K(x) = 0.5 e^x E1(x) - 1 on eighth-octave pieces of [1, 1024): the
    # Stokeslet real-space weight 0.5 E1(x) - e^-x equals e^-x K(x).
    out.append(f"#define FTE_K_DEG {DEG_K}")
    out.append("#define FTE_K_NPIECE 80")
    out.append("/* K(x) = 0.5 e^x E1(x) - 1 on [2^k (1 + q/8), 2^k (1 + (q+1)/8)), k = 0..9, q = 0..7;")
    out.append(" * t = (x - mid)/half */")
    out.append("FTE_E1_STORAGE_G double fte_k_coef[FTE_K_NPIECE][FTE_K_DEG + 1] = {")
    worst_k = 0.0
    for k in range(10):
        for q in range(8):
            a = mp.mpf(2) ** k * (1 + mp.mpf(q) / 8)
            b = mp.mpf(2) ** k * (1 + mp.mpf(q + 1) / 8)
            c = cheb_fit(k_fun, a, b, DEG_K)
            m = cheb_to_mono(c)
            mid, half = (a + b) / 2, (b - a) / 2
            e = max(abs(horner(m, (x - mid) / half) / k_fun(x) - 1) for x in [a + (b - a) * i / 99 for i in range(100)])
            worst_k = max(worst_k, float(e))
            out.append("    {" + ", ".join(mp.nstr(v, 20, min_fixed=-1, max_fixed=-1) for v in m) + "},")
    out.append("};")
    out.append(f"/* worst relative truncation error of the K pieces: {worst_k:.3e} */")

    # exp(-x) = 2^(-n/64) exp(-r): table 2^(-j/64), Cody-Waite split of ln2/64
    # (the high part has 36 significant bits so n * hi is exact for n < 2^17),
    # and the Taylor coefficients (-1)^k / k! of exp(-r), |r| <= ln2/128.
    ln2_64 = mp.log(2) / 64
    hi = mp.mpf(int(mp.nint(ln2_64 * mp.mpf(2) ** 42))) / mp.mpf(2) ** 42
    lo = ln2_64 - hi
    out.append("/* exp(-x) = 2^(-n/64) exp(-r), n = round(64 x / ln 2), r = x - n ln2/64 */")
    out.append(f"#define FTE_EXP_INV_LN2_64 {mp.nstr(1 / ln2_64, 20, min_fixed=-1, max_fixed=-1)}")
    out.append(f"#define FTE_EXP_LN2_64_HI {mp.nstr(hi, 20, min_fixed=-1, max_fixed=-1)}")
    out.append(f"#define FTE_EXP_LN2_64_LO {mp.nstr(lo, 20, min_fixed=-1, max_fixed=-1)}")
    out.append("FTE_E1_STORAGE_G double fte_exp_tab[64] = {")
    out.append("    " + ", ".join(mp.nstr(mp.mpf(2) ** (-mp.mpf(j) / 64), 20, min_fixed=-1, max_fixed=-1)
                                  for j in range(64)) + "};")
    out.append("FTE_E1_STORAGE_R double fte_exp_poly[7] = {")
    out.append("    " + ", ".join(mp.nstr(mp.mpf(-1) ** k / mp.factorial(k), 20, min_fixed=-1, max_fixed=-1)
                                  for k in range(7)) + "};")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fte_e1_coeffs.h")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
    print("wrote", path, "R err", float(err_r), "G worst rel err", worst, "K worst rel err", worst_k)


if __name__ == "__main__":
    main()
