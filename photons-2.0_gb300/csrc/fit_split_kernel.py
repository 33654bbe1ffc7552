"""Generate split_kernel_coeffs.h: the FP32 approximation of the short-range
factor g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2) used by the split-precision
P2P kernel.

Form (the rational shape of Abramowitz & Stegun 7.1.26, refitted here):
    erfc(u) = exp(-u^2) * erfcx(u),   erfcx(u) ~= t * sum_k a_k t^k,
    t = 1 / (1 + p u),
so  g(u) ~= exp(-u^2) * (t * P(t) + (2/sqrt(pi)) u).
The coefficients minimise the maximum relative error of g on [0, UMAX]
(Lawson's iteratively reweighted least squares); p is scanned.  Beyond UMAX
the factor exp(-u^2) < 1e-7 keeps the absolute error negligible.

Run:  python fit_split_kernel.py > split_kernel_coeffs.h
"""
import numpy as np
from scipy.special import erfc, erfcx

UMAX = 4.0
DEG = 6  # number of a_k


def g(u):
    return erfc(u) + 2.0 / np.sqrt(np.pi) * u * np.exp(-u * u)


def fit(p, x, iters=60):
    t = 1.0 / (1.0 + p * x)
    A = np.stack([t ** (k + 1) for k in range(DEG)], 1)
    h = erfcx(x)
    scale = 1.0 / (h + 2.0 / np.sqrt(np.pi) * x)  # relative error in g
    w = np.ones_like(x)
    for _ in range(iters):
        sw = np.sqrt(w) * scale
        c, *_ = np.linalg.lstsq(A * sw[:, None], h * sw, rcond=None)
        err = np.abs(A @ c - h) * scale
        w = w * err
        w /= w.sum()
    return c, err.max()


def main():
    x = np.cos(np.pi * (np.arange(6000) + 0.5) / 6000) * UMAX / 2 + UMAX / 2
    best = None
    for p in np.linspace(0.3, 1.2, 91):
        c, e = fit(p, x)
        if best is None or e < best[2]:
            best = (p, c, e)
    p, c, e = best
    u = np.linspace(0.0, UMAX, 200001)
    t = 1.0 / (1.0 + p * u)
    gp = np.exp(-u * u) * (sum(c[k] * t ** (k + 1) for k in range(DEG)) + 2.0 / np.sqrt(np.pi) * u)
    rel = np.abs(gp - g(u)) / g(u)
    print("// Generated by fit_split_kernel.py -- do not edit.")
    print("// erfcx(u) ~= sum_k SPLIT_A[k] t^(k+1), t = 1/(1 + SPLIT_P u), u in [0, %.1f]" % UMAX)
    print("// max relative error of g(u) in double precision: %.3e" % rel.max())
    print("#pragma once")
    print("#define SPLIT_NA %d" % DEG)
    print("static const double SPLIT_P = %.17g;" % p)
    print("static const double SPLIT_A[SPLIT_NA] = {%s};" % ", ".join("%.17g" % v for v in c))


if __name__ == "__main__":
    main()
