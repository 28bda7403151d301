"""Generate fastmath_coef.cuh: float32 polynomial coefficients for
    atan(a)/a     = P(s),  s = a^2,  a in [0, 1]
    sin(pi r)/r   = S(s),  s = r^2,  r in [-1/2, 1/2]
    cos(pi r)     = K(s),  s = r^2,  r in [-1/2, 1/2]
Each is the Chebyshev interpolant (in s) of float64 NumPy values at DEG+1
Chebyshev points, converted to monomial form and rounded to float32.  The
script reports the max error of the float32 polynomials (float32 Horner) on
a dense grid.

    python cuda_mcmc_gb300/csrc/gen_fastmath.py   # rewrites fastmath_coef.cuh
"""
import os

import numpy as np
from numpy.polynomial import chebyshev as Ch

HERE = os.path.dirname(os.path.abspath(__file__))


def fit(fun, lo, hi, deg):
    k = np.arange(deg + 1)
    t = np.cos((2 * k + 1) * np.pi / (2 * (deg + 1)))
    s = 0.5 * (lo + hi) + 0.5 * (hi - lo) * t
    cc = Ch.chebfit(t, fun(s), deg)
    # map back from t to s: t = (2 s - (lo + hi)) / (hi - lo)
    p = Ch.cheb2poly(cc)
    a, b = 2.0 / (hi - lo), -(lo + hi) / (hi - lo)
    out = np.zeros(deg + 1)
    for j, cj in enumerate(p):           # expand cj * (a s + b)^j
        term = np.poly1d([a, b]) ** j
        coeffs = term.coeffs[::-1]
        out[:len(coeffs)] += cj * coeffs
    return out.astype(np.float32)


def horner32(c, x):
    x = np.asarray(x, np.float32)
    acc = np.full_like(x, c[-1])
    for a in c[-2::-1]:
        acc = (acc * x + np.float32(a)).astype(np.float32)
    return acc


def atan_over_a(s):
    a = np.sqrt(s)
    out = np.ones_like(s)
    nz = a > 1e-12
    out[nz] = np.arctan(a[nz]) / a[nz]
    return out


def sinpi_over_r(s):
    r = np.sqrt(s)
    out = np.full_like(s, np.pi)
    nz = r > 1e-12
    out[nz] = np.sin(np.pi * r[nz]) / r[nz]
    return out


def cospi(s):
    return np.cos(np.pi * np.sqrt(s))


def main():
    at = fit(atan_over_a, 0.0, 1.0, 7)
    sn = fit(sinpi_over_r, 0.0, 0.25, 5)
    cs = fit(cospi, 0.0, 0.25, 6)
    a = np.linspace(0, 1, 200001)
    e_at = np.max(np.abs(a.astype(np.float32) * horner32(at, (a * a).astype(np.float32)) - np.arctan(a)))
    r = np.linspace(-0.5, 0.5, 200001)
    e_sn = np.max(np.abs(r.astype(np.float32) * horner32(sn, (r * r).astype(np.float32)) - np.sin(np.pi * r)))
    e_cs = np.max(np.abs(horner32(cs, (r * r).astype(np.float32)) - np.cos(np.pi * r)))

    def arr(name, c):
        return "static __constant__ const float %s[%d] = {%s};" % (
            name, len(c), ", ".join("%.9ef" % x for x in c))

    lines = [
        "// fastmath_coef.cuh -- GENERATED by gen_fastmath.py; do not edit.",
        "// Monomial coefficients (lowest degree first) of float32 polynomial fits:",
        "//   kAtanP:  atan(a)/a in s = a^2, a in [0,1]       max |atan err| %.2e" % e_at,
        "//   kSinPiS: sin(pi r)/r in s = r^2, |r| <= 1/2    max |sin err|  %.2e" % e_sn,
        "//   kCosPiK: cos(pi r) in s = r^2, |r| <= 1/2      max |cos err|  %.2e" % e_cs,
        "#pragma once",
        "namespace cmc {",
        arr("kAtanP", at),
        arr("kSinPiS", sn),
        arr("kCosPiK", cs),
        "}  // namespace cmc",
        "",
    ]
    with open(os.path.join(HERE, "fastmath_coef.cuh"), "w") as f:
        f.write("\n".join(lines))
    print("atan %.3e  sinpi %.3e  cospi %.3e" % (e_at, e_sn, e_cs))


if __name__ == "__main__":
    main()
