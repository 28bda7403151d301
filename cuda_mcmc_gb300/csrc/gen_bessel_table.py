"""Generate bessel_table.cuh: piecewise polynomials for
    F1(x) = J1(x) / x      and      F2(x) = J2(x) / x^2
(and, for derivatives, F3(x) = J3(x) / x^3: F1' = -x F2, F2' = -x F3)
on x in [0, XMAX) in intervals of width 1/SUB, [i/SUB, (i+1)/SUB), each a
degree-DEG polynomial in t = SUB x - (i + 0.5).  Both functions are entire and
even, with F1(0) = 1/2 and F2(0) = 1/8.  Narrow intervals and a low degree
keep the per-point evaluation short (2 table loads and 6 FMAs for F1 and F2
together) at the accuracy float32 Horner allows anyway.

Method: for every interval, interpolate the function at the DEG+1 Chebyshev
points of the interval (values from SciPy's float64 Bessel functions), convert
the Chebyshev interpolant to monomial coefficients in t (|t| <= 1/2, so the
monomial form is well conditioned), and round to float32.  The script reports
the maximum error of the float32 polynomials, evaluated with float32 Horner,
against float64 values on a dense grid.

    python cuda_mcmc_gb300/csrc/gen_bessel_table.py   # rewrites bessel_table.cuh
"""
import os

import numpy as np
from numpy.polynomial import chebyshev as Ch
from numpy.polynomial import polynomial as Po
from scipy.special import j1, jv

XMAX = 32
SUB = 8            # intervals per unit of x
DEG = 3            # odd: coefficients pack into (DEG + 1) / 2 float4
NINT = XMAX * SUB
HERE = os.path.dirname(os.path.abspath(__file__))


def f1(x):
    x = np.asarray(x, np.float64)
    out = np.empty_like(x)
    small = np.abs(x) < 1e-4
    out[small] = 0.5 - x[small] ** 2 / 16
    out[~small] = j1(x[~small]) / x[~small]
    return out


def f2(x):
    x = np.asarray(x, np.float64)
    out = np.empty_like(x)
    small = np.abs(x) < 1e-3
    out[small] = 0.125 - x[small] ** 2 / 96
    out[~small] = jv(2, x[~small]) / x[~small] ** 2
    return out


def f3(x):
    x = np.asarray(x, np.float64)
    out = np.empty_like(x)
    small = np.abs(x) < 1e-2
    out[small] = 1.0 / 48 - x[small] ** 2 / 768
    out[~small] = jv(3, x[~small]) / x[~small] ** 3
    return out


def fit(fun, i):
    c = (i + 0.5) / SUB
    # Chebyshev nodes on t in [-1/2, 1/2], x = c + t / SUB
    k = np.arange(DEG + 1)
    s = np.cos((2 * k + 1) * np.pi / (2 * (DEG + 1)))
    t = 0.5 * s
    cc = Ch.chebfit(s, fun(c + t / SUB), DEG)     # interpolant in s = 2t
    mono_s = Ch.cheb2poly(cc)                      # coefficients in s
    mono_t = mono_s * (2.0 ** np.arange(DEG + 1))  # s = 2t
    return mono_t.astype(np.float32)


def horner32(coef, d):
    d = np.float32(d)
    acc = np.float32(coef[-1])
    for a in coef[-2::-1]:
        acc = np.float32(acc * d + np.float32(a))
    return acc


def main():
    tab = np.zeros((NINT, DEG + 1, 3), np.float32)
    err = [0.0, 0.0, 0.0]
    for i in range(NINT):
        tab[i, :, 0] = fit(f1, i)
        tab[i, :, 1] = fit(f2, i)
        tab[i, :, 2] = fit(f3, i)
        xs = np.linspace(i / SUB, (i + 1) / SUB, 101)[:-1]
        for j, fun in enumerate((f1, f2, f3)):
            ref = fun(xs)
            got = np.array([horner32(tab[i, :, j],
                                     np.float32(np.float32(x) * np.float32(SUB)) - np.float32(i + 0.5))
                            for x in xs], np.float64)
            err[j] = max(err[j], float(np.max(np.abs(got - ref))))
    lines = [
        "// bessel_table.cuh -- GENERATED by gen_bessel_table.py; do not edit.",
        "//",
        "// F1(x) = J1(x)/x and F2(x) = J2(x)/x^2 on [0, %d): interval i = [i, i+1)/%d holds"
        % (XMAX, SUB),
        "// coefficients a_k (k = 0..%d) of sum_k a_k t^k, t = %d x - (i + 0.5), stored as"
        % (DEG, SUB),
        "// float4 (F1 a_2m, F2 a_2m, F1 a_2m+1, F2 a_2m+1), m = 0..%d.  Chebyshev" % ((DEG - 1) // 2),
        "// interpolants of float64 values, rounded",
        "// to float32; max |error| with float32 Horner: F1 %.2e, F2 %.2e." % tuple(err[:2]),
        "#pragma once",
        "",
        "namespace cmc {",
        "constexpr int kBesselXmax = %d;       // the tables cover x in [0, kBesselXmax)" % XMAX,
        "constexpr int kBesselSub = %d;        // intervals per unit of x" % SUB,
        "constexpr int kBesselIntervals = %d;" % NINT,
        "constexpr int kBesselDeg = %d;" % DEG,
        "static __device__ const float4 kBesselTab[%d][%d] = {" % (NINT, (DEG + 1) // 2),
    ]
    for i in range(NINT):
        row = ", ".join("{%.9ef, %.9ef, %.9ef, %.9ef}" % (tab[i, 2 * m, 0], tab[i, 2 * m, 1],
                                                           tab[i, 2 * m + 1, 0], tab[i, 2 * m + 1, 1])
                        for m in range((DEG + 1) // 2))
        lines.append("    {%s}," % row)
    lines += ["};", "",
              "// F3(x) = J3(x)/x^3, same intervals, coefficients a_0..a_%d (max |error| %.2e)."
              % (DEG, err[2]),
              "static __device__ const float kBesselTab3[%d][%d] = {" % (NINT, DEG + 1)]
    for i in range(NINT):
        lines.append("    {%s}," % ", ".join("%.9ef" % tab[i, k, 2] for k in range(DEG + 1)))
    lines += ["};", "}  // namespace cmc", ""]
    with open(os.path.join(HERE, "bessel_table.cuh"), "w") as f:
        f.write("\n".join(lines))
    print("max abs error: F1 %.3e  F2 %.3e  F3 %.3e" % tuple(err))


if __name__ == "__main__":
    main()
