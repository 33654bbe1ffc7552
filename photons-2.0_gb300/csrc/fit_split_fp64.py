"""Piecewise polynomials for the FP64 pair factor of the P2P kernels,

    g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2),    0 <= u < NI * W,

the split-force factor of src/fmm.c:846-848 (u = r / 2rs).  On interval
i = floor(u / W), with centre m_i = (i + 1/2) W and d = u - m_i in
[-W/2, W/2), g(u) = sum_k C[k][i] d^k, evaluated by Horner's rule.  Each
interval's polynomial interpolates g at DEG + 1 Chebyshev points of the
interval (mpmath at 60 digits), then its monomial coefficients are rounded
to double.  The script checks the rounded polynomials against g at 40-digit
precision on 1500 points per interval and prints the largest absolute and
relative differences into the header: beyond u = NI W, g < 2e-27 and the
kernels fall back to erfc and exp.

Run:  python fit_split_fp64.py > split_fp64_table.h
"""
import mpmath as mp
import numpy as np

W = mp.mpf(1) / 16
NI = 128
DEG = 8


def g(u):
    return mp.erfc(u) + 2 / mp.sqrt(mp.pi) * u * mp.exp(-u * u)


def fit(i):
    """Monomial coefficients (low to high) in d of the Chebyshev
    interpolant of g(m_i + d) on [-W/2, W/2]."""
    m = (i + mp.mpf(1) / 2) * W
    h = W / 2
    n = DEG + 1
    nodes = [h * mp.cos(mp.pi * (2 * j + 1) / (2 * n)) for j in range(n)]
    vals = [g(m + x) for x in nodes]
    # solve the Vandermonde system exactly at working precision
    A = mp.matrix([[x ** k for k in range(n)] for x in nodes])
    c = mp.lu_solve(A, mp.matrix(vals))
    return [c[k] for k in range(n)]


def main():
    mp.mp.dps = 60
    coef = [fit(i) for i in range(NI)]
    C = np.array([[float(coef[i][k]) for i in range(NI)] for k in range(DEG + 1)])
    mp.mp.dps = 40
    worst_abs = worst_rel = 0.0
    for i in range(NI):
        m = (i + mp.mpf(1) / 2) * W
        for x in np.linspace(-float(W) / 2, float(W) / 2, 1500, endpoint=False):
            d = mp.mpf(float(x))
            acc = mp.mpf(0)
            for k in range(DEG, -1, -1):
                acc = acc * d + mp.mpf(C[k][i])
            exact = g(m + d)
            ae = abs(acc - exact)
            worst_abs = max(worst_abs, float(ae))
            worst_rel = max(worst_rel, float(ae / exact))
    print("// Generated by fit_split_fp64.py -- do not edit.")
    print("// g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2) on [0, %g): interval i = floor(u / %g)," % (NI * float(W), float(W)))
    print("// g = sum_k SPLIT64_C[k][i] d^k, d = u - (i + 1/2) %g; degree %d." % (float(W), DEG))
    print("// Rounded coefficients against g (40 digits, 1500 points per interval):")
    print("//   max |error| %.3e, max relative error %.3e" % (worst_abs, worst_rel))
    print("#pragma once")
    print("#define SPLIT64_W %.17g" % float(W))
    print("#define SPLIT64_INVW %.17g" % float(1 / W))
    print("#define SPLIT64_NI %d" % NI)
    print("#define SPLIT64_DEG %d" % DEG)
    print("// initialiser of a [SPLIT64_DEG + 1][SPLIT64_NI] array, coefficient of d^k in row k")
    print("#define SPLIT64_C_INIT \\")
    print("    { \\")
    for k in range(DEG + 1):
        row = ", ".join("%.17g" % v for v in C[k])
        print("        {%s}, \\" % row)
    print("    }")


if __name__ == "__main__":
    main()
