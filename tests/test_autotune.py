"""The leaf-size autotuner's choice rule, on the host with a stand-in pass.

autotune_leaf times each candidate MAXLEAF (both FP32 P2P kernels, mutual
and one-way, at leaf sizes 48-64), measures each one's median relative
error against the FP64 direct sum on a sample, and returns the fastest
candidate within the error bound, else the most accurate one, together
with the flag that selects its kernel.  The stand-in pass returns forces
with a chosen relative error and reports chosen device times, so the rule
is checked without a GPU."""
import numpy as np
import pytest


class StandInPass:
    """ForcePass look-alike: forces = truth x (1 + err[key]), device time ms[key]."""

    def __init__(self, truth, ms, err):
        self.truth, self.ms, self.err = truth, ms, err
        self.runs = []
        self.key = None

    def run(self, pos, q, precision, flags=0):
        self.key = (q["maxleaf"], flags)
        self.runs.append((self.key, precision))
        return self.truth * (1.0 + self.err[self.key])

    def timings(self):
        # the autotuner scores total - upload - download (the device part)
        return dict(total=self.ms[self.key] + 0.75, upload=0.5, download=0.25, tree=0.0, walk=0.0, p2p=0.0,
                    farfield=0.0)

    def counters(self):
        return dict(pairs_local=7000, pairs_image=400)


@pytest.fixture()
def setup(ph, monkeypatch):
    rng = np.random.default_rng(5)
    n = 500
    pos = rng.random((n, 3)) * 10.0
    truth = rng.normal(size=(n, 3))
    monkeypatch.setattr(ph, "direct_sum", lambda pos_, p_, tgt: truth[tgt])
    p = dict(boxsize=10.0, theta=0.5, rs=0.5, rcut=2.25, eps=0.01, mass=1.0, maxleaf=16)
    return pos, truth, p


def test_fastest_within_bound_and_both_kernels_timed(ph, setup):
    pos, truth, p = setup
    ow = ph.F_ONE_WAY
    ms = {(16, 0): 9.0, (32, 0): 7.0, (48, 0): 6.0, (48, ow): 6.5, (64, 0): 5.0, (64, ow): 5.5}
    err = {(16, 0): 5e-4, (32, 0): 9e-5, (48, 0): 6e-5, (48, ow): 6e-5, (64, 0): 2e-5, (64, ow): 2e-5}
    fp = StandInPass(truth, ms, err)
    best, table, flags = ph.autotune_leaf(fp, pos, p, candidates=(16, 32, 48, 64), sample=200, repeats=2,
                                          shapes=False)
    assert (best, flags) == (64, 0)
    # every candidate ran `repeats` times; leaf 48 and 64 once per kernel
    keys = [k for k, _ in fp.runs]
    assert keys.count((16, 0)) == 2 and keys.count((32, 0)) == 2
    for leaf in (48, 64):
        assert keys.count((leaf, 0)) == 2 and keys.count((leaf, ow)) == 2
    assert all(prec == ph.FP32_SPLIT for _, prec in fp.runs)
    rows = {(r["maxleaf"], r["flags"]): r for r in table}
    assert set(rows) == set(ms)
    for k, r in rows.items():
        assert r["ms"] == pytest.approx(ms[k])
        assert r["median"] == pytest.approx(err[k], rel=1e-6)
        assert r["pairs_per_particle"] == pytest.approx(7400 / pos.shape[0])
    assert rows[(48, 0)]["kernel"] == "mutual" and rows[(48, ow)]["kernel"] == "one-way"
    assert rows[(16, 0)]["kernel"] == "one-way"


def test_one_way_kernel_chosen_where_faster(ph, setup):
    pos, truth, p = setup
    ow = ph.F_ONE_WAY
    ms = {(32, 0): 7.0, (48, 0): 6.0, (48, ow): 4.0}
    err = {(32, 0): 3e-5, (48, 0): 2e-5, (48, ow): 2e-5}
    best, table, flags = ph.autotune_leaf(StandInPass(truth, ms, err), pos, p, candidates=(32, 48), sample=100,
                                          repeats=1, shapes=False)
    assert (best, flags) == (48, ow)


def test_slow_accurate_candidate_loses_to_a_fast_one_within_bound(ph, setup):
    pos, truth, p = setup
    ms = {(16, 0): 3.0, (24, 0): 8.0}
    err = {(16, 0): 9e-5, (24, 0): 1e-6}
    best, _, flags = ph.autotune_leaf(StandInPass(truth, ms, err), pos, p, candidates=(16, 24), sample=100,
                                      repeats=1, shapes=False)
    assert (best, flags) == (16, 0)


def test_most_accurate_when_none_within_bound(ph, setup):
    pos, truth, p = setup
    ms = {(16, 0): 1.0, (24, 0): 2.0, (32, 0): 3.0}
    err = {(16, 0): 9e-3, (24, 0): 4e-4, (32, 0): 6e-4}
    best, table, flags = ph.autotune_leaf(StandInPass(truth, ms, err), pos, p, candidates=(16, 24, 32),
                                          error_bound=1e-4, sample=100, repeats=1, shapes=False)
    assert (best, flags) == (24, 0)
    assert len(table) == 3


def test_fp64_times_one_kernel_per_leaf(ph, setup):
    pos, truth, p = setup
    ms = {(48, 0): 2.0, (64, 0): 1.0}
    err = {(48, 0): 1e-6, (64, 0): 1e-6}
    fp = StandInPass(truth, ms, err)
    best, table, flags = ph.autotune_leaf(fp, pos, p, candidates=(48, 64), sample=100, repeats=1,
                                          precision=ph.FP64)
    assert (best, flags) == (64, 0)
    assert [k for k, _ in fp.runs] == [(48, 0), (64, 0)]
    assert all(prec == ph.FP64 for _, prec in fp.runs)
    assert all(r["kernel"] == "one-way" for r in table)


def test_kernel_builds_timed_at_the_chosen_leaf(ph, setup):
    """With shapes on, a mutual-kernel choice is re-timed in every build of
    that kernel, with either source staging (cp.async or TMA bulk copies),
    and the fastest within the bound wins; a one-way choice is not
    re-timed."""
    pos, truth, p = setup
    ow = ph.F_ONE_WAY
    ms = {(32, 0): 9.0, (64, 0): 5.0, (64, ow): 7.0}
    err = {(32, 0): 9e-5, (64, 0): 2e-5, (64, ow): 2e-5}
    for sh in range(1, ph.P2P_SHAPES):
        for bulk in (0, ph.F_P2P_BULK):
            ms[(64, ph.F_P2P_SHAPE(sh) | bulk)] = 5.0 + 0.1 * sh + (0.05 if bulk else 0.0)
            err[(64, ph.F_P2P_SHAPE(sh) | bulk)] = 2e-5
    ms[(64, ph.F_P2P_SHAPE(3))] = 4.2
    fp = StandInPass(truth, ms, err)
    best, table, flags = ph.autotune_leaf(fp, pos, p, candidates=(32, 64), sample=100, repeats=1)
    assert (best, flags) == (64, ph.F_P2P_SHAPE(3))
    assert {k for k, _ in fp.runs} == set(ms)
    ms[(64, ph.F_P2P_SHAPE(4) | ph.F_P2P_BULK)] = 4.1
    fp = StandInPass(truth, ms, err)
    best, table, flags = ph.autotune_leaf(fp, pos, p, candidates=(32, 64), sample=100, repeats=1)
    assert (best, flags) == (64, ph.F_P2P_SHAPE(4) | ph.F_P2P_BULK)
    ms2 = {(32, 0): 3.0}
    fp = StandInPass(truth, ms2, {(32, 0): 9e-5})
    best, _, flags = ph.autotune_leaf(fp, pos, p, candidates=(32,), sample=100, repeats=1)
    assert (best, flags) == (32, 0) and [k for k, _ in fp.runs] == [(32, 0)]
