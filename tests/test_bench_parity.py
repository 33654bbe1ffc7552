"""bench.py's parity leg and reference arm on CPU.

The parity leg compares a GPU pass (tree, lists, counters, FP64 forces on a
subset) with the oracle on the same input; here a stand-in for the GPU
context serves the oracle's own full pass, so the leg must report every
item equal, and a planted difference (in the oracle's output) must show.
The reference arm runs the oracle on the GPU arm's workload and prints the
same config."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class FullPassStandIn:
    """The accessors bench.parity_leg reads from a GPU context, served from
    the oracle's own full pass."""

    def __init__(self, r):
        self.r = r

    def counters(self):
        c = dict(self.r["counters"])
        t, s, _ = self.r["lists"]["p2p"]
        tr = self.r["tree"]
        first = c["first_leaf"]
        nt = tr["leaf_npart"][t - first].astype(np.int64)
        ns = tr["leaf_npart"][s - first].astype(np.int64)
        c["pairs_local"] = int(np.where(t == s, nt * (nt - 1), nt * ns).sum())
        c["pairs_image"] = c["p2p_count_remote"]
        return c

    def perm(self):
        return self.r["perm"]

    def lists(self):
        return self.r["lists"]


def test_parity_leg_reports_equal_and_catches_a_difference(port, ics):
    pos, p = ics.make("nfw128", nside=20, maxleaf=8)
    full = port.run(pos, p, capture=True, tree=True, nthreads=4)
    acc = np.empty_like(full["acc"])
    acc[full["perm"]] = full["acc"]
    tg = np.random.default_rng(1).choice(pos.shape[0], 200, replace=False).astype(np.int32)
    out = bench.parity_leg(FullPassStandIn(full), pos, p, tg, acc[tg], acc[tg], 4)
    assert out["counts_equal"] and out["perm_equal"] and all(out["lists_equal"].values())
    assert out["fp64_ok"] and out["fp64_max_rel"] == 0.0
    # a planted mistake: one list entry of the stand-in's pass moved to another source
    t, s, im = (x.copy() for x in full["lists"]["p2p"])
    s[5] = s[6]
    bad = dict(full, lists=dict(full["lists"], p2p=(t, s, im)))
    out = bench.parity_leg(FullPassStandIn(bad), pos, p, tg, acc[tg] * (1 + 1e-9), acc[tg], 4)
    assert not out["lists_equal"]["p2p"] and not out["fp64_ok"]


def test_reference_arm_same_config_and_counters(tmp_path, port, ics):
    """The reference arm runs the GPU arm's workload (here at 24^3) and
    prints the GPU arm's config, its pair counts and a positive rate."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--nside", "24",
                        "--maxleaf", "64", "--steps", "2", "--warmup", "1"], capture_output=True, text=True,
                       timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    pos, p = bench.workload(24, 64)

    class A:
        workload, nside = "zeldovich256", 24

    assert line["config"] == json.loads(json.dumps(bench.workload_config(A, p, pos.shape[0])))
    full = port.run(pos, p, capture=False, tree=False, nthreads=4)
    for k in ("idxP2P", "idxM2L", "p2p_count_remote", "nleaf", "nnode", "n_p2p_ext", "n_m2l_ext"):
        assert line["counters"][k] == full["counters"][k], k
    assert line["e2e"]["value"] == line["value"]
