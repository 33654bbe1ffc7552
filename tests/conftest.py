import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def ph():
    """The package (photons-2.0_gb300), with its CUDA library built."""
    mod = __graft_entry__.load_package()
    if not os.path.exists(mod.library_path()):
        sys.path.insert(0, __graft_entry__.PKG_DIR)
        import build as pkg_build
        sys.path.pop(0)
        pkg_build.build()
    return mod


@pytest.fixture(scope="session")
def ics(ph):
    from photons_gb300 import ics as m
    return m


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_port()
    return oracle


@pytest.fixture(scope="session")
def port(oracle_mod):
    return oracle_mod.PortOracle()


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    for k in ("pos_in", "pos_tree"):  # stored as FP32 where the input itself is FP32 (exact)
        d[k] = d[k].astype(np.float64)
    pr = d["params"]
    d["p"] = dict(boxsize=pr[0], theta=pr[1], rs=pr[2], rcut=pr[3], eps=pr[4], mass=pr[5], maxleaf=int(pr[6]))
    return d
