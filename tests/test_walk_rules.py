"""The walk's FP32 decisions, checked on the CPU: the rule behind its
touching shortcut against the reference's MAC (src/fmm.c:267-326; the C
restatement always, the reference's own compiled function where it is
built), and an FP32 emulation of its MAC and image-pruning filters against
the exact FP64 rules on inputs drawn next to every threshold.

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


# ---------------------------------------------------------------------------
# The FP32 filters' margins: an emulation of the walk's FP32 arithmetic in
# numpy float32 (each operation rounded to FP32; products also fused, as the
# compiler may contract a*b+c) must never decide against the exact FP64 rule
# when it decides at all.  Inputs are drawn next to the rules' thresholds.

F = np.float32


def _hilo(c):
    hi = F(c)
    return hi, F(c - np.float64(hi))


def _centre_diff32(hb, lb, ha, la, o, Lhi, Llo):
    if o < 0:
        hb, lb = F(hb - Lhi), F(lb - Llo)
    elif o > 0:
        ha, la = F(ha - Lhi), F(la - Llo)
    return F(F(hb - ha) + F(lb - la))


def _sumsq(g, fused):
    if not fused:
        return F(F(F(g[0] * g[0]) + F(g[1] * g[1])) + F(g[2] * g[2]))
    acc = F(g[0] * g[0])
    for k in (1, 2):
        acc = F(np.float64(g[k]) * np.float64(g[k]) + np.float64(acc))
    return acc


def _pruned_fp32(d, rw, bw, rc2, k2, fused):
    """The walk's image_pruned_fp32 step by step in FP32."""
    h = [F(F(rw[i] + bw[i]) * F(0.5)) for i in range(3)]
    a = [F(abs(d[i])) for i in range(3)]
    u = [F(a[i] + h[i]) for i in range(3)]
    g = [max(F(a[i] - h[i]), F(0)) for i in range(3)]
    dm2 = _sumsq(g, fused)
    gu = F(F(F(g[0] * u[0]) + F(g[1] * u[1])) + F(g[2] * u[2]))
    edm = F(F(F(4e-6) * gu) + F(F(1e-6) * F(dm2 + rc2)))
    if dm2 >= F(rc2 + edm):
        return 1
    if dm2 > F(rc2 - edm):
        return -2
    wmax = max(bw)
    lhs, rhs = F(wmax * wmax), F(k2 * dm2)
    ew = F(F(F(2e-6) * F(lhs + rhs)) + F(k2 * edm))
    if lhs < F(rhs - ew):
        return 1
    if lhs > F(rhs + ew):
        return 0
    return -2


def _pruned_fp64(cr, cb, s, rw, bw, rcut, theta):
    """The sender-side pruning rule (src/remotes.c:97-158) in FP64."""
    dr = 0.0
    for i in range(3):
        gap = abs((cr[i] - cb[i]) - s[i]) - (rw[i] + bw[i]) * 0.5
        if gap > 0.0:
            dr += gap * gap
    dr = np.sqrt(dr)
    return dr >= rcut or max(bw) < 0.95 * theta * dr


def _pruning_cases(n, seed):
    rng = np.random.default_rng(seed)
    L = 500.0
    Lhi, Llo = _hilo(L)
    for _ in range(n):
        rw = rng.uniform(1.0, 80.0, 3)
        bw = rng.uniform(0.5, 40.0, 3)
        theta = rng.uniform(0.3, 1.0)
        rcut = rng.uniform(5.0, 30.0)
        h = 0.5 * (rw + bw)
        # gaps on some axes, scaled so that dr sits next to rcut or next to
        # max(bw) / (0.95 theta)
        axes = rng.random(3) < 0.7
        if not axes.any():
            axes[rng.integers(3)] = True
        dirn = rng.random(3) * axes
        dirn /= np.linalg.norm(dirn)
        target = rcut if rng.random() < 0.5 else max(bw) / (0.95 * theta)
        dr = target * (1.0 + rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-9, -3))
        gaps = dr * dirn
        d = np.where(axes, h + gaps, rng.uniform(0, 1, 3) * h) * rng.choice([-1.0, 1.0], 3)
        cr = rng.uniform(0, L, 3)
        m = np.zeros(3, int)
        cb = cr + d
        for i in range(3):  # node centre inside the box, the image shift makes up the rest
            if cb[i] >= L:
                cb[i] -= L
                m[i] = 1
            elif cb[i] < 0:
                cb[i] += L
                m[i] = -1
        yield cr, cb, m, rw, bw, rcut, theta, L, Lhi, Llo


def test_fp32_pruning_filter_never_contradicts_fp64():
    decided = 0
    for cr, cb, m, rw, bw, rcut, theta, L, Lhi, Llo in _pruning_cases(4000, 11):
        rh = [_hilo(x) for x in cr]
        bh = [_hilo(x) for x in cb]
        d = [_centre_diff32(bh[i][0], bh[i][1], rh[i][0], rh[i][1], m[i], Lhi, Llo) for i in range(3)]
        exact = _pruned_fp64(cr, cb, m * L, rw, bw, rcut, theta)
        for fused in (False, True):
            r = _pruned_fp32(d, [F(x) for x in rw], [F(x) for x in bw], F(rcut * rcut),
                             F((0.95 * theta) ** 2), fused)
            if r != -2:
                decided += 1
                assert bool(r) == exact, (cr, cb, m, rw, bw, rcut, theta, fused)
    assert decided > 2000  # most cases are decided in FP32 even this close to the thresholds


def _mac_fp32(wi, wj, d, theta2, c2, fused):
    """The walk's acceptance_fp32 step by step in FP32."""
    w = [F(F(wi[i] + wj[i]) * F(0.5)) for i in range(3)]
    a = [F(abs(d[i])) for i in range(3)]
    u = [F(a[i] + w[i]) for i in range(3)]
    g = [max(F(a[i] - w[i]), F(0)) for i in range(3)]
    S = F(F(g[0] + g[1]) + g[2])
    eS = F(F(2e-6) * F(F(u[0] + u[1]) + u[2]))
    if S < F(F(1e-4) - eS):
        return 0
    if S < F(F(1e-4) + eS):
        smax = F(F(1e-4) + F(F(2) * eS))
        hw = max(w)
        return 0 if (theta2 <= F(1) and smax < F(F(0.1) * hw) and F(smax * smax) < c2) else -2
    dm2 = _sumsq(g, fused)
    gu = F(F(F(g[0] * u[0]) + F(g[1] * u[1])) + F(g[2] * u[2]))
    edm = F(F(F(4e-6) * gu) + F(F(1e-6) * F(dm2 + c2)))
    if dm2 >= F(c2 + edm):
        return -1
    if dm2 > F(c2 - edm):
        return -2
    dd2 = _sumsq(d, fused)
    edd = F(F(2e-6) * F(dd2 + c2))
    if dd2 > F(c2 + edd):
        return 0
    if dd2 >= F(c2 - edd):
        return -2
    wmax = F(max(w) * F(2))
    lhs, rhs = F(wmax * wmax), F(theta2 * dd2)
    ew = F(F(2e-6) * F(lhs + rhs))
    if lhs < F(rhs - ew):
        return 1
    if lhs > F(rhs + ew):
        return 0
    return -2


def _mac_cases(n, seed):
    """Node pairs next to each of the MAC's thresholds: the touching window,
    the cutoff on the gaps, the cutoff on the centres, the opening angle."""
    rng = np.random.default_rng(seed)
    L = 500.0
    Lhi, Llo = _hilo(L)
    for k in range(n):
        kind = k % 4
        theta = rng.uniform(0.3, 1.0)
        rcut = rng.uniform(5.0, 30.0)
        # opening-angle cases need boxes small against rcut (2 wmax / theta < rcut)
        wmax_hi = 0.45 * theta * rcut if kind == 3 else 60.0
        wi = rng.uniform(0.05, wmax_hi, 3)
        wj = rng.uniform(0.05, wmax_hi, 3)
        w = 0.5 * (wi + wj)
        near = 1.0 + rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-9, -3)
        axes = rng.random(3) < 0.7
        if not axes.any():
            axes[rng.integers(3)] = True
        dirn = rng.random(3) * axes
        if kind == 0:  # gap sum next to 1e-4
            gaps = 1e-4 * near * dirn / dirn.sum()
        elif kind == 1:  # gaps' norm next to rcut
            gaps = rcut * near * dirn / np.linalg.norm(dirn)
        else:
            gaps = rng.uniform(0, rcut, 3) * dirn
        d = np.where(axes, w + gaps, rng.uniform(0, 1, 3) * w) * rng.choice([-1.0, 1.0], 3)
        if kind == 2:  # centre distance next to rcut
            d *= rcut * near / np.linalg.norm(d)
        elif kind == 3:  # opening angle: 2 wmax = theta dd
            d *= 2.0 * w.max() / theta * near / np.linalg.norm(d)
        ca = rng.uniform(0, L, 3)
        cb = ca - d  # d = c_a - c_b', c_b' = c_b + m L
        m = np.zeros(3, int)
        for i in range(3):
            if cb[i] >= L:
                cb[i] -= L
                m[i] = 1
            elif cb[i] < 0:
                cb[i] += L
                m[i] = -1
        yield ca, cb, m, wi, wj, theta, rcut, L, Lhi, Llo


def test_fp32_mac_filter_never_contradicts_fp64(port):
    decided = 0
    for ca, cb, m, wi, wj, theta, rcut, L, Lhi, Llo in _mac_cases(4000, 13):
        dist = ca - (cb + m * L)
        exact = port.acceptance(wi, wj, dist, theta, rcut)
        ah = [_hilo(x) for x in ca]
        bh = [_hilo(x) for x in cb]
        e = [_centre_diff32(bh[i][0], bh[i][1], ah[i][0], ah[i][1], m[i], Lhi, Llo) for i in range(3)]
        for fused in (False, True):
            r = _mac_fp32([F(x) for x in wi], [F(x) for x in wj], e, F(theta * theta), F(rcut * rcut), fused)
            if r != -2:
                decided += 1
                assert r == exact, (ca, cb, m, wi, wj, theta, rcut, fused, r, exact)
    assert decided > 2000
