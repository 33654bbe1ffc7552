"""The split-force factor g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2) of
src/fmm.c:846-848 as the FP64 kernels evaluate it: piecewise polynomials
whose coefficients csrc/fit_split_fp64.py generates into
csrc/split_fp64_table.h.  On the CPU: the committed table is the script's
output, and its polynomials (Horner in double) stay within a few 1e-17 of
g.  On the GPU: the kernels' evaluation against erfc and exp there."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "photons-2.0_gb300", "csrc")
HEADER = os.path.join(CSRC, "split_fp64_table.h")


def g_ref(u):
    from scipy.special import erfc
    return erfc(u) + 2.0 / np.sqrt(np.pi) * u * np.exp(-u * u)


def load_table():
    text = open(HEADER).read()
    w = float(re.search(r"#define SPLIT64_W (\S+)", text).group(1))
    ni = int(re.search(r"#define SPLIT64_NI (\d+)", text).group(1))
    deg = int(re.search(r"#define SPLIT64_DEG (\d+)", text).group(1))
    rows = re.findall(r"\{([^{}]+)\}", text.split("#define SPLIT64_C_INIT", 1)[1])
    c = np.array([[float(v) for v in r.split(",") if v.strip()] for r in rows])
    assert c.shape == (deg + 1, ni)
    return w, ni, deg, c


def horner(u, w, ni, deg, c):
    i = np.floor(u / w).astype(int)
    d = u - (i + 0.5) * w
    acc = c[deg][i]
    for k in range(deg - 1, -1, -1):
        acc = acc * d + c[k][i]
    return acc


def test_table_is_the_fit_scripts_output():
    pytest.importorskip("mpmath")
    out = subprocess.run([sys.executable, os.path.join(CSRC, "fit_split_fp64.py")], capture_output=True, text=True,
                         check=True).stdout
    assert out == open(HEADER).read()


def test_table_polynomials_match_erfc_and_exp():
    """Horner in double against g at 30 digits: within 1.5e-16 (half an ulp
    of g near 1), relative 1e-14 where pairs carry force (u < 4); and
    against the double erfc and exp formula, which carries its own
    rounding, within 5e-16 on a dense grid."""
    mp = pytest.importorskip("mpmath")
    pytest.importorskip("scipy")
    w, ni, deg, c = load_table()
    mp.mp.dps = 30
    u = np.concatenate([np.random.default_rng(1).uniform(0.0, ni * w, 6000), np.arange(ni) * w])  # + interval edges
    exact = np.array([float(mp.erfc(x) + 2 / mp.sqrt(mp.pi) * x * mp.exp(-x * x)) for x in u])
    err = np.abs(horner(u, w, ni, deg, c) - exact)
    assert err.max() <= 1.5e-16, err.max()
    near = u < 4.0
    assert (err[near] / exact[near]).max() <= 1e-14
    grid = np.linspace(0.0, ni * w, 200001, endpoint=False)
    assert np.abs(horner(grid, w, ni, deg, c) - g_ref(grid)).max() <= 5e-16


@pytest.mark.gpu
def test_device_split_factor_matches_erfc_and_exp(ph):
    u = np.concatenate([np.linspace(0.0, 10.0, 400001), np.random.default_rng(5).uniform(0.0, 8.0, 100000)])
    tab = ph.split_factor_fp64(u)
    exact = ph.split_factor_fp64(u, exact=True)
    err = np.abs(tab - exact)
    assert err.max() <= 5e-16, err.max()
    assert np.array_equal(tab[u >= 8.0], exact[u >= 8.0])  # beyond the table: erfc and exp
