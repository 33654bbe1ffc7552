"""CPU restatement of the reference's PM long-range force.  TEST
INFRASTRUCTURE ONLY: tests/ use it to check the GPU PM (photons_pm_force).

Follows src/partmesh.c (one rank: CIC deposit :86-180, the 4-point gradient
:524-735, CIC interpolation :574-587) and the convolution of
src/conv.f90:128-247 (Green's function :171-227, with its pi: the Fortran
declares `real*8, parameter :: M_PI = 3.1415926`, a default-kind, i.e.
single-precision, literal, so pi is 3.1415926 rounded to FP32).  numpy float64 arithmetic rounds every operation on
its own, in the reference's order; the FFT is numpy's, so results differ
from the reference's 2DECOMP&FFT (and from cuFFT) in the last bits.  The
reference's PM needs 2DECOMP&FFT (Fortran), which does not build here, so
the pin is partial: src/partmesh.c itself is compiled in place
(oracle/Makefile) with the Fortran convolution replaced by a C stand-in
(oracle/pm_conv.c), and this restatement matches it to 3e-15 of the largest
force (tests/golden/pm/, made by tests/golden/make_golden.py).  The
convolution's Green's function is a restatement on both sides.
"""
from __future__ import annotations

import numpy as np

PM_PI = float(np.float32(3.1415926))  # 3.141592502593994


def _axis(x, norm, delta, N):
    """nearest cell, the neighbour on the particle's side, their weights."""
    c = (x * norm).astype(np.int64)  # C's (int) cast truncates toward zero
    w = (x - (c + 0.5) * delta) * norm
    cn = np.where(w > 0, c + 1, c - 1)
    w = np.where(w > 0, w, -w)
    wn = 1.0 - w
    return c % N, cn % N, w, wn


def _cic(pos, N, L):
    norm = N / L
    delta = 1.0 / norm
    i, ii, wi, win = _axis(pos[:, 0], norm, delta, N)
    j, jj, wj, wjn = _axis(pos[:, 1], norm, delta, N)
    k, kk, wk, wkn = _axis(pos[:, 2], norm, delta, N)
    # the eight corners in the reference's order with their weight triples
    return [((i, j, k), (win, wjn, wkn)), ((ii, j, k), (wi, wjn, wkn)), ((i, jj, k), (win, wj, wkn)),
            ((ii, jj, k), (wi, wj, wkn)), ((i, j, kk), (win, wjn, wk)), ((ii, j, kk), (wi, wjn, wk)),
            ((i, jj, kk), (win, wj, wk)), ((ii, jj, kk), (wi, wj, wk))]


def green(N, L, rs):
    """G on the half spectrum [N, N, N//2+1] (src/conv.f90:171-227)."""
    nhalf = N // 2
    ismth2 = 2 * PM_PI * rs / L
    ismth2 = ismth2 * ismth2
    pref = L * L / (PM_PI * N * N * N)
    a = np.arange(N)
    a = np.where(a > nhalf, a - N, a)
    c = np.arange(N // 2 + 1)

    def sinc(q):
        f = PM_PI * q.astype(np.float64) / N
        with np.errstate(invalid="ignore", divide="ignore"):
            s = np.sin(f) / f
        return np.where(q == 0, 1.0, s)

    fx = sinc(a)[:, None, None]
    fy = sinc(a)[None, :, None]
    fz = sinc(c)[None, None, :]
    k2 = (a[:, None, None] ** 2 + a[None, :, None] ** 2 + c[None, None, :] ** 2).astype(np.float64)
    ff = 1.0 / (fx * fy * fz)
    with np.errstate(invalid="ignore", divide="ignore"):
        gf = pref * np.exp(-k2 * ismth2) * ff * ff * ff * ff / k2
    gf[0, 0, 0] = pref
    return gf


def pm_force(pos, boxsize, nside, rs, mass):
    """acc_pm (n, 3) of the reference's PM at one rank (G-free)."""
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    N, L = int(nside), float(boxsize)
    corners = _cic(pos, N, L)
    rho = np.zeros((N, N, N))
    for (ci, cj, ck), (a, b, c) in corners:
        np.add.at(rho, (ci, cj, ck), mass * a * b * c)
    renormal = N / L
    renormal = renormal * renormal * renormal
    rho *= renormal
    rk = np.fft.rfftn(rho) * green(N, L, rs)
    psi = np.fft.irfftn(rk, s=(N, N, N), axes=(0, 1, 2)) * (N * N * N)  # the unnormalised inverse
    invx = 0.5 * N / L
    c1, c2 = (4.0 / 3.0) * invx, (1.0 / 6.0) * invx
    grads = []
    for ax in range(3):
        g = c1 * (np.roll(psi, -1, ax) - np.roll(psi, 1, ax))
        grads.append(g - c2 * (np.roll(psi, -2, ax) - np.roll(psi, 2, ax)))
    out = np.empty_like(pos)
    for d in range(3):
        acc = None
        for (ci, cj, ck), (a, b, c) in corners:
            t = a * b * c * grads[d][ci, cj, ck]
            acc = t if acc is None else acc + t
        out[:, d] = acc
    return out
