"""Seeded synthetic particle sets for the five force-pass workloads, and the
reference's rules for the derived force parameters.

The reference reads Gadget-2 files or draws uniform randoms
(src/initial.c:558-620); the workloads used here are defined by their
shapes, sizes and distributions instead, and are generated from fixed seeds:

* ``grid32``     32^3 particles, L=100: regular grid + N(0, 0.3*spacing)
                 offsets, seed 1, wrapped periodic.  Mesh 32, leaf <= 16.
* ``nfw128``     128^3, L=200: 50 % uniform + 50 % in 64 NFW halos
                 (c ~ U[5,15], halo masses log-uniform over two decades),
                 seed 2.  Mesh 128.
* ``zeldovich256`` 256^3, L=500: Zel'dovich displacement of a Gaussian field
                 with P(k) ~ k^-2, rms displacement 0.5 spacing, seed 3.
                 Mesh 256.
* ``boxes256``   256 independent periodic boxes, N_b log-uniform in
                 [16^3, 64^3], L_b ~ U[20,100], 70 % Plummer (a=0.05 L_b)
                 + 30 % uniform, seed 4.
* ``zeldovich512`` 512^3, L=1000, P(k) ~ k^-1.5, seed 5.

Force parameters follow src/initial.c:316-345: rs = 1.25 L / mesh,
rcut = 4.5 rs, softening = 0.03 L / N^(1/3) (computed with the reference's
pow(N, 0.3333333)), and the particle mass of src/initial.c:596
(Omega_m * 3 * 0.01 / (8 pi G) * L^3 / N with the demo's G).
"""
from __future__ import annotations

import math

import numpy as np

GRAV_CONST = 43007.105732  # demo/lcdm_g2.run:25
OMEGA_M = 0.3


def force_params(n_total, boxsize, mesh, theta=0.5, maxleaf=16):
    """Derived force-pass parameters by the reference's rules."""
    rs = 1.25 * boxsize / float(mesh)
    return {
        "boxsize": float(boxsize),
        "maxleaf": int(maxleaf),
        "theta": float(theta),
        "rs": rs,
        "rcut": 4.5 * rs,
        "eps": 0.03 * boxsize / math.pow(float(n_total), 0.3333333),
        "mass": (OMEGA_M * 3 * 0.01) / (8.0 * math.pi * GRAV_CONST) * boxsize ** 3 / float(n_total),
    }


def _wrap(pos, boxsize):
    pos = np.mod(pos, boxsize)
    # np.mod can return exactly boxsize for tiny negative inputs
    pos[pos >= boxsize] -= boxsize
    return pos


def grid_gaussian(nside, boxsize, sigma_frac=0.3, seed=1):
    rng = np.random.default_rng(seed)
    dx = boxsize / nside
    i = (np.arange(nside) + 0.5) * dx
    g = np.stack(np.meshgrid(i, i, i, indexing="ij"), -1).reshape(-1, 3)
    pos = g + rng.normal(0.0, sigma_frac * dx, size=g.shape)
    return _wrap(pos, boxsize)


def _nfw_radii(rng, n, c):
    """Radii in units of r_vir from the NFW profile truncated at r_vir."""
    mu = lambda x: np.log1p(x) - x / (1.0 + x)
    u = rng.random(n) * mu(c)
    lo = np.zeros(n)
    hi = np.full(n, float(c))
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        big = mu(mid) > u
        hi = np.where(big, mid, hi)
        lo = np.where(big, lo, mid)
    return 0.5 * (lo + hi) / c


def _iso(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def uniform_plus_nfw(nside, boxsize, nhalo=64, seed=2):
    rng = np.random.default_rng(seed)
    n = nside ** 3
    n_bg = n // 2
    n_halo = n - n_bg
    bg = rng.random((n_bg, 3)) * boxsize
    w = 10.0 ** rng.uniform(0.0, 2.0, nhalo)
    counts = np.floor(w / w.sum() * n_halo).astype(np.int64)
    counts[np.argsort(-w)[: n_halo - counts.sum()]] += 1
    conc = rng.uniform(5.0, 15.0, nhalo)
    centres = rng.random((nhalo, 3)) * boxsize
    rho = n / boxsize ** 3
    parts = [bg]
    for h in range(nhalo):
        m = counts[h]
        rvir = (3.0 * m / (4.0 * math.pi * 200.0 * rho)) ** (1.0 / 3.0)
        r = _nfw_radii(rng, m, conc[h]) * rvir
        parts.append(centres[h] + r[:, None] * _iso(rng, m))
    pos = np.concatenate(parts)
    return _wrap(pos, boxsize)


def zeldovich(nside, boxsize, index, seed, rms_frac=0.5, dtype=np.float64):
    """Grid + Zel'dovich displacement of a Gaussian field with P(k) ~ k^index."""
    import scipy.fft as sfft

    rng = np.random.default_rng(seed)
    dx = boxsize / nside
    white = rng.standard_normal((nside, nside, nside), dtype=np.float32 if dtype == np.float32 else np.float64)
    dk = sfft.rfftn(white, workers=-1)
    del white
    k1 = 2.0 * np.pi * np.fft.fftfreq(nside, d=dx)
    kz = 2.0 * np.pi * np.fft.rfftfreq(nside, d=dx)
    kx = k1[:, None, None]
    ky = k1[None, :, None]
    kzz = kz[None, None, :]
    k2 = kx * kx + ky * ky + kzz * kzz
    k2[0, 0, 0] = 1.0
    dk *= np.sqrt(k2 ** (0.5 * index))
    dk[0, 0, 0] = 0.0
    psi = []
    for kc in (kx, ky, kzz):
        comp = sfft.irfftn(1j * kc * dk / k2, s=(nside,) * 3, workers=-1)
        psi.append(comp.reshape(-1))
    del dk
    psi = np.stack(psi, -1)
    psi *= rms_frac * dx / np.sqrt(np.mean(np.sum(psi * psi, axis=1)))
    i = (np.arange(nside) + 0.5) * dx
    g = np.stack(np.meshgrid(i, i, i, indexing="ij"), -1).reshape(-1, 3)
    return _wrap(g + psi, boxsize)


def plummer_boxes(nbox=256, seed=4, nmin=16 ** 3, nmax=64 ** 3):
    """List of (pos, params) for independent periodic boxes."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nbox):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        L = rng.uniform(20.0, 100.0)
        n_pl = int(round(0.7 * n))
        a = 0.05 * L
        r = np.empty(0)
        while r.size < n_pl:
            u = rng.random(2 * n_pl)
            rr = a / np.sqrt(np.maximum(u, 1e-300) ** (-2.0 / 3.0) - 1.0)
            r = np.concatenate([r, rr[rr < 0.5 * L]])
        r = r[:n_pl]
        pl = 0.5 * L + r[:, None] * _iso(rng, n_pl)
        bg = rng.random((n - n_pl, 3)) * L
        pos = _wrap(np.concatenate([pl, bg]), L)
        mesh = max(1, int(round(n ** (1.0 / 3.0))))
        out.append((pos, force_params(n, L, mesh)))
    return out


WORKLOADS = {
    "grid32": dict(nside=32, boxsize=100.0, mesh=32, maxleaf=16),
    "nfw128": dict(nside=128, boxsize=200.0, mesh=128, maxleaf=16),
    "zeldovich256": dict(nside=256, boxsize=500.0, mesh=256, maxleaf=16),
    "zeldovich512": dict(nside=512, boxsize=1000.0, mesh=512, maxleaf=16),
}


def make(name, nside=None, maxleaf=None, theta=0.5):
    """(pos[N,3] float64, params) for a named workload; ``nside`` rescales
    the particle count at fixed density and clustering (box scaled with it)."""
    w = WORKLOADS[name]
    ns = nside or w["nside"]
    L = w["boxsize"] * ns / w["nside"]
    mesh = ns
    if name == "grid32":
        pos = grid_gaussian(ns, L, 0.3, seed=1)
    elif name == "nfw128":
        pos = uniform_plus_nfw(ns, L, nhalo=max(1, int(round(64 * (ns / 128) ** 3))), seed=2)
    elif name == "zeldovich256":
        pos = zeldovich(ns, L, -2.0, seed=3)
    elif name == "zeldovich512":
        pos = zeldovich(ns, L, -1.5, seed=5)
    else:
        raise KeyError(name)
    p = force_params(pos.shape[0], L, mesh, theta=theta, maxleaf=maxleaf or w["maxleaf"])
    return pos, p
