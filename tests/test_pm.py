"""PM long-range force (src/partmesh.c at one rank, src/conv.f90:128-247).

The oracle (oracle/pm_oracle.py) restates the reference's deposit, Green's
function, gradient and interpolation in numpy.  It is pinned to the
reference's own PM code: src/partmesh.c compiled in place, with only the
Fortran convolution (which needs 2DECOMP&FFT) replaced by a stand-in
(oracle/pm_conv.c), through the golden fixtures in tests/golden/pm/ and,
where the reference tree is present, live.  It is also checked against the
analytic long-range part of the force split, and the GPU PM
(photons_pm_force) is checked against it."""
import glob
import os

import numpy as np
import pytest
from scipy.special import erfc

from conftest import GOLDEN

PM_GOLDEN = sorted(glob.glob(os.path.join(GOLDEN, "pm", "*.npz")))


@pytest.fixture(scope="module")
def pm_oracle():
    import pm_oracle as m
    return m


def _g(u):
    return erfc(u) + 2 / np.sqrt(np.pi) * u * np.exp(-u * u)


def test_oracle_matches_long_range_kernel(pm_oracle):
    """Two equal masses: the PM force along their separation equals
    m/r^2 (1 - g(r/2rs)), the complement of the short-range split factor,
    to the mesh's accuracy (a few per cent at 3-8 cells)."""
    N, L, rs, m = 64, 64.0, 1.25, 1.0
    rng = np.random.default_rng(0)
    for r in (3.0, 4.0, 6.0, 8.0):
        ratios = []
        for _ in range(6):
            c = rng.random(3) * L
            d = rng.standard_normal(3)
            d /= np.linalg.norm(d)
            pos = np.stack([c, (c + r * d) % L])
            a = pm_oracle.pm_force(pos, L, N, rs, m)
            ratios.append(a[0] @ d / (m / r ** 2 * (1 - _g(r / (2 * rs)))))
            # equal and opposite
            assert np.allclose(a[0], -a[1], rtol=0, atol=1e-6 * np.abs(a[0]).max())
        assert abs(np.mean(ratios) - 1) < 0.02, (r, ratios)
        assert max(abs(x - 1) for x in ratios) < 0.06, (r, ratios)


@pytest.mark.parametrize("path", PM_GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_pm_golden(pm_oracle, path):
    """The numpy restatement against the reference's partmesh.c outputs:
    the same deposit, halo exchange, gradient stencil and interpolation, so
    only the transforms' rounding (numpy FFT against a direct DFT) differs."""
    z = np.load(path)
    L, N, rs, m = z["params"]
    got = pm_oracle.pm_force(z["pos"], L, int(N), rs, m)
    want = z["acc_pm"]
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_oracle_matches_reference_pm_live(pm_oracle):
    """The same against the reference library itself, on a fresh input."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference tree is not on this machine")
    ref = oracle.RefOracle()
    rng = np.random.default_rng(11)
    L, N = 30.0, 20
    pos = rng.random((800, 3)) * L
    pos[:300] = (np.array([2.0, 29.0, 15.0]) + rng.normal(scale=0.8, size=(300, 3))) % L  # across the faces
    want = ref.pm_force(pos, L, N, 1.25 * L / N, 0.3)
    got = pm_oracle.pm_force(pos, L, N, 1.25 * L / N, 0.3)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
@pytest.mark.parametrize("nside", [32, 48])
def test_gpu_pm_matches_oracle(ph, ics, pm_oracle, nside):
    """FP64 throughout; the FFTs (cuFFT vs numpy) and the atomic deposit
    order differ only in the last bits."""
    fp = ph.ForcePass(0)
    for pos, p in (ics.make("grid32", nside=24), ics.make("nfw128", nside=24)):
        want = pm_oracle.pm_force(pos, p["boxsize"], nside, p["rs"], p["mass"])
        got = fp.pm_force(pos, p, nside)
        scale = np.abs(want).max()
        assert np.abs(got - want).max() <= 1e-10 * scale
        rel = np.linalg.norm(got - want, axis=1) / np.maximum(np.linalg.norm(want, axis=1), 1e-3 * scale)
        assert np.median(rel) <= 1e-12


@pytest.mark.gpu
def test_gpu_pm_device_io(ph, ics):
    torch = pytest.importorskip("torch")
    pos, p = ics.make("nfw128", nside=16)
    fp = ph.ForcePass(0)
    host = fp.pm_force(pos, p, 32)
    dpos = torch.from_numpy(pos).cuda()
    dacc = torch.empty_like(dpos)
    prm = ph.make_params(p, ph.FP64, 0, ph.F_DEVICE_IO)
    import ctypes as C
    rc = fp.lib.photons_pm_force(fp.h, C.byref(prm), 32, pos.shape[0], C.c_void_p(dpos.data_ptr()),
                                 C.c_void_p(dacc.data_ptr()))
    assert rc == 0
    got = dacc.cpu().numpy()
    assert np.abs(got - host).max() <= 1e-12 * np.abs(host).max()


@pytest.mark.gpu
@pytest.mark.parametrize("path", PM_GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_pm_matches_reference_golden(ph, path):
    """The GPU PM against the reference's partmesh.c outputs (cuFFT against
    a direct DFT, atomic against sequential deposit: last bits only)."""
    z = np.load(path)
    L, N, rs, m = z["params"]
    p = dict(boxsize=L, theta=0.5, rs=rs, rcut=4.5 * rs, eps=0.0, mass=m, maxleaf=16)
    got = ph.ForcePass(0).pm_force(z["pos"], p, int(N))
    want = z["acc_pm"]
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()
