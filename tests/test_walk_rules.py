"""The rule behind one of the walk's FP32 shortcuts, checked on the CPU
against the reference's MAC (src/fmm.c:267-326): the C restatement always,
and the reference's own compiled function where it is built.

The walk decides node pairs near the MAC's touching window (gap sum 1e-4)
in FP32, where a large box's FP32 error can exceed the window, and returns
"open" without the exact FP64 test.  That relies on the MAC answering
"open" (0) on either side of the window: with gap sum S < 0.1 w (w the
largest half-width sum) and S < rcut, the gaps are too small for the
cutoff drop and the boxes too close for the accept at theta <= 1."""
import numpy as np
import pytest


def near_touching_pairs(n, seed):
    """Box pairs whose gaps sum to at most a tenth of the largest half-width
    sum: the touching window and far beyond it."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        wi = rng.uniform(0.01, 60.0, 3)
        wj = rng.uniform(0.01, 60.0, 3)
        w = 0.5 * (wi + wj)
        S = w.max() * 0.1 * rng.choice([rng.uniform(0, 1e-6), rng.uniform(0, 1e-3), rng.uniform(0, 1.0)])
        axes = rng.random(3) < 0.6
        if not axes.any():
            axes[rng.integers(3)] = True
        share = rng.random(3) * axes
        gaps = S * share / share.sum()
        # axes without a gap overlap (|d| <= w); with one, |d| = w + gap
        d = np.where(axes, w + gaps, rng.uniform(0, 1, 3) * w) * rng.choice([-1.0, 1.0], 3)
        theta = rng.uniform(0.05, 1.0)
        rcut = max(S, 1e-3) * rng.uniform(1.01, 1e4)
        out.append((wi, wj, d, theta, rcut))
    return out


def test_mac_opens_near_the_touching_window_port(port):
    for wi, wj, d, theta, rcut in near_touching_pairs(20000, 5):
        assert port.acceptance(wi, wj, d, theta, rcut) == 0, (wi, wj, d, theta, rcut)


def test_mac_opens_near_the_touching_window_reference(oracle_mod):
    if not oracle_mod.ref_available():
        pytest.skip("the reference oracle is not built here")
    ref = oracle_mod.RefOracle()
    for wi, wj, d, theta, rcut in near_touching_pairs(5000, 6):
        assert ref.acceptance(wi, wj, d, theta, rcut) == 0, (wi, wj, d, theta, rcut)


def test_the_rule_needs_its_conditions(port):
    """Outside the conditions the MAC does accept or drop: an opening angle
    above 2/sqrt(3) accepts boxes whose gaps sum to 0.1 w, and a cutoff
    below the gap drops them (the walk then takes the exact test)."""
    wi = wj = np.array([1.0, 1.0, 1.0])
    d = np.array([1.1, 1.0, 1.0])  # one gap of 0.1 = 0.1 w (w = 1)
    assert port.acceptance(wi, wj, d, 1.9, 10.0) == 1
    assert port.acceptance(wi, wj, d, 0.5, 0.05) == -1
    assert port.acceptance(wi, wj, d, 0.5, 10.0) == 0
