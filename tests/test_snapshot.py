"""Gadget-2 snapshots (the reference's SnapFormat 2, src/snapshot.c): the
library's reader against the reference's own readers on the reference's
demo initial conditions, and a write/read round trip.  Host code only."""
import os

import numpy as np
import pytest


def _demo(oracle_mod, name):
    path = os.path.join(oracle_mod.REFROOT, "demo", name)
    if not os.path.exists(path):
        pytest.skip("reference demo snapshots not present")
    try:
        ref = oracle_mod.RefOracle()
    except FileNotFoundError:
        pytest.skip("reference build not present")
    return path, ref


@pytest.mark.parametrize("name", ["ic_lcdm.gdt2", "ic_merger.gdt2"])
def test_reader_matches_reference(ph, oracle_mod, name):
    path, ref = _demo(oracle_mod, name)
    hr, pr, vr = ref.gadget(path)
    h, p, v = ph.gadget_read(path)
    assert np.array_equal(p, pr)
    assert np.array_equal(v, vr)
    assert h["boxsize"] == hr["boxsize"] and h["mass"][1] == hr["mass"]
    assert h["omega0"] == hr["omega0"] and h["omega_lambda"] == hr["omega_lambda"]
    assert h["hubble"] == hr["hubble"] and h["redshift"] == hr["redshift"]
    assert sum(h["npart_total"]) == hr["npart_total"]


def test_partial_read(ph, oracle_mod):
    path, _ = _demo(oracle_mod, "ic_merger.gdt2")
    _, p, v = ph.gadget_read(path)
    _, p2, v2 = ph.gadget_read(path, first=39990, count=20)  # across the species boundary
    assert np.array_equal(p2, p[39990:40010]) and np.array_equal(v2, v[39990:40010])


def test_write_read_round_trip(ph, tmp_path):
    rng = np.random.default_rng(1)
    n = 1000
    pos = rng.random((n, 3)) * 100.0
    vel = rng.standard_normal((n, 3)) * 50.0
    z = 49.0
    h = dict(npart=[0, n, 0, 0, 0, 0], mass=[0.0, 2.5, 0, 0, 0, 0], time=1 / (1 + z), redshift=z,
             npart_total=[0, n, 0, 0, 0, 0], num_files=1, boxsize=100.0, omega0=0.3, omega_lambda=0.7, hubble=0.7)
    path = str(tmp_path / "snap.gdt2")
    ph.gadget_write(path, h, pos, vel)
    assert os.path.getsize(path) == 4 + 256 + 4 + 2 * (4 + 12 * n + 4)
    hr, p, v = ph.gadget_read(path)
    g = (1.0 / (1.0 + z)) ** 1.5
    assert np.array_equal(p, pos.astype(np.float32).astype(np.float64))
    assert np.array_equal(v, (vel.astype(np.float32).astype(np.float64) / g).astype(np.float32).astype(np.float64) * g)
    assert hr["npart"] == [0, n, 0, 0, 0, 0] and hr["boxsize"] == 100.0 and hr["redshift"] == z


def test_errors(ph, tmp_path):
    with pytest.raises(ph.PhotonsError, match="cannot open"):
        ph.gadget_read(str(tmp_path / "missing.gdt2"))
    path = str(tmp_path / "short.gdt2")
    ph.gadget_write(path, dict(npart=[0, 10, 0, 0, 0, 0], boxsize=1.0), np.zeros((10, 3)), np.zeros((10, 3)))
    with pytest.raises(ph.PhotonsError, match="holds 10 particles"):
        ph.gadget_read(path, first=5, count=10)
    with open(path, "r+b") as f:
        f.truncate(200)
    with pytest.raises(ph.PhotonsError, match="truncated"):
        ph.gadget_read(path)
