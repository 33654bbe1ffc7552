"""Kick-drift-kick integration (src/photoNs.c:141-196, 257-268;
src/initial.c:639-683): the time integrals on the host, the kick and drift
kernels and one device-resident step.

CPU tests pin the oracle's restatement of kick_loga / drift_loga, and the
library's host copy, to the reference (compiled in place when present, else
the committed golden values).  GPU tests compare the kernels and the step
with the oracle's kick / drift loops and a host-composed step, bit for bit.
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _golden_rows():
    return np.load(os.path.join(GOLDEN, "time", "loga_integrals.npz"))["rows"]


def test_loga_integrals_golden(port, ph):
    for om, ox, la, lb, kick, drift in _golden_rows():
        assert port.kick_loga(om, ox, la, lb) == kick
        assert port.drift_loga(om, ox, la, lb) == drift
        assert ph.kick_loga(om, ox, la, lb) == kick
        assert ph.drift_loga(om, ox, la, lb) == drift


def test_loga_integrals_match_reference(port, oracle_mod):
    try:
        ref = oracle_mod.RefOracle()
    except FileNotFoundError:
        pytest.skip("reference build not present")
    rng = np.random.default_rng(5)
    for _ in range(20):
        om = float(rng.uniform(0.1, 1.0))
        a0 = float(np.exp(rng.uniform(math.log(0.005), math.log(1.0))))
        la, lb = math.log(a0), math.log(a0) + float(rng.uniform(1e-4, 0.3))
        assert port.kick_loga(om, 1 - om, la, lb) == ref.kick_loga(om, 1 - om, la, lb)
        assert port.drift_loga(om, 1 - om, la, lb) == ref.drift_loga(om, 1 - om, la, lb)


def test_loga_integrals_match_quadrature(port):
    """Independent check of the integrands: the Simpson sums over 128
    intervals agree to 1e-9 with adaptive quadrature of the integrals over
    log a of z/h (kick) and z^2/h (drift), h = 0.1 sqrt(Om z^3 + OL)."""
    scipy_integrate = pytest.importorskip("scipy.integrate")
    om, ox = 0.3, 0.7
    la, lb = math.log(0.5), math.log(0.6)

    def h(l):
        z = math.exp(-l)
        return 0.1 * math.sqrt(om * z ** 3 + ox)

    kick = scipy_integrate.quad(lambda l: math.exp(-l) / h(l), la, lb, epsabs=0, epsrel=1e-13)[0]
    drift = scipy_integrate.quad(lambda l: math.exp(-2 * l) / h(l), la, lb, epsabs=0, epsrel=1e-13)[0]
    assert abs(port.kick_loga(om, ox, la, lb) / kick - 1) < 1e-9
    assert abs(port.drift_loga(om, ox, la, lb) / drift - 1) < 1e-9


def test_oracle_drift_wraps_like_the_reference(port):
    L = 10.0
    pos = np.array([0.1, 9.9, 5.0, 0.0, 9.999999999999998, 3.0])
    vel = np.array([-1.0, 1.0, 26.0, -1e-300, 0.0, -33.0])
    port.drift(pos, vel, 0.5, L)
    assert np.all((pos >= 0) & (pos < L))
    assert pos[0] == -0.4 + L and pos[2] == (5.0 + 13.0) - L


@pytest.mark.gpu
def test_kick_drift_kernels_match_oracle(ph, port):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    n = 100003  # odd coordinate count exercises the tail
    L = 37.5
    pos = rng.random((n, 3)) * L
    pos[:100] = rng.choice([0.0, L * (1 - 1e-16), 1e-12, L - 1e-12], size=(100, 3))
    vel = rng.standard_normal((n, 3)) * 3.0
    vel[:50] *= 40.0  # several box lengths per step
    acc = rng.standard_normal((n, 3))
    dkh, dd = 0.0173, 0.91
    dpos, dvel, dacc = (torch.from_numpy(a.copy()).cuda() for a in (pos, vel, acc))
    ph.kick(n, dvel.data_ptr(), dacc.data_ptr(), dkh)
    ph.drift(n, dpos.data_ptr(), dvel.data_ptr(), dd, L)
    torch.cuda.synchronize()
    port.kick(vel, acc, dkh)
    port.drift(pos, vel, dd, L)
    assert np.array_equal(dvel.cpu().numpy(), vel)
    assert np.array_equal(dpos.cpu().numpy(), pos)
    assert pos.min() >= 0 and pos.max() < L


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["FP64", "FP32_SPLIT"])
def test_kdk_step_matches_host_composition(ph, port, ics, precision):
    """photons_kdk_step == kick (oracle) + drift (oracle) + force pass + kick."""
    torch = pytest.importorskip("torch")
    pos, p = ics.make("zeldovich512", nside=24, maxleaf=16)
    rng = np.random.default_rng(3)
    vel = rng.standard_normal(pos.shape) * 0.5
    prec = getattr(ph, precision)
    om, ox = 0.3, 0.7
    la, lb = math.log(0.5), math.log(0.505)
    G = 43007.105732
    dkh = 0.5 * ph.kick_loga(om, ox, la, lb) * G
    dd = ph.drift_loga(om, ox, la, lb)
    fp = ph.ForcePass(0)
    acc0 = fp.run(pos, p, precision=prec)
    dpos, dvel, dacc = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (pos, vel, acc0))
    torch.cuda.synchronize()
    fp.kdk_step_device(dpos.data_ptr(), dvel.data_ptr(), dacc.data_ptr(), pos.shape[0], p, dkh, dd, precision=prec)
    hp, hv = pos.copy(), vel.copy()
    port.kick(hv, acc0, dkh)
    port.drift(hp, hv, dd, p["boxsize"])
    acc1 = fp.run(hp, p, precision=prec)
    port.kick(hv, acc1, dkh)
    assert np.array_equal(dpos.cpu().numpy(), hp)
    assert np.array_equal(dacc.cpu().numpy(), acc1)
    assert np.array_equal(dvel.cpu().numpy(), hv)


@pytest.mark.gpu
def test_kdk_step_with_pm_matches_host_composition(ph, port, ics):
    """The full step with both halves of the force, against the oracle's
    kicks and drift around separately computed short-range and PM forces."""
    torch = pytest.importorskip("torch")
    pos, p = ics.make("zeldovich512", nside=24, maxleaf=16)
    rng = np.random.default_rng(5)
    vel = rng.standard_normal(pos.shape) * 0.5
    nside = 24
    la, lb = math.log(0.5), math.log(0.505)
    dkh = 0.5 * ph.kick_loga(0.3, 0.7, la, lb) * 43007.105732
    dd = ph.drift_loga(0.3, 0.7, la, lb)
    fp = ph.ForcePass(0)
    acc0 = fp.run(pos, p, precision=ph.FP64)
    pm0 = fp.pm_force(pos, p, nside)
    dpos, dvel, dacc, dpm = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (pos, vel, acc0, pm0))
    torch.cuda.synchronize()
    fp.kdk_step_pm_device(dpos.data_ptr(), dvel.data_ptr(), dacc.data_ptr(), dpm.data_ptr(), pos.shape[0], p, nside,
                          dkh, dd, precision=ph.FP64)
    hp, hv = pos.copy(), vel.copy()
    port.kick(hv, pm0, dkh)
    port.kick(hv, acc0, dkh)
    port.drift(hp, hv, dd, p["boxsize"])
    acc1 = fp.run(hp, p, precision=ph.FP64)
    pm1 = fp.pm_force(hp, p, nside)
    assert np.array_equal(dpos.cpu().numpy(), hp)
    assert np.array_equal(dacc.cpu().numpy(), acc1)
    # the PM deposit adds with atomics: its last bits vary between runs
    gpm = dpm.cpu().numpy()
    assert np.abs(gpm - pm1).max() <= 1e-12 * np.abs(pm1).max()
    port.kick(hv, acc1, dkh)
    port.kick(hv, gpm, dkh)
    assert np.array_equal(dvel.cpu().numpy(), hv)


def _kdk_factors(ph):
    la, lb = math.log(0.5), math.log(0.505)
    return 0.5 * ph.kick_loga(0.3, 0.7, la, lb) * 43007.105732, ph.drift_loga(0.3, 0.7, la, lb)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["FP64", "FP32_SPLIT"])
def test_kdk_steps_as_one_graph_match_the_steps_one_by_one(ph, ics, precision):
    """From the second step on, photons_kdk_step runs the kick, the drift,
    the force pass and the second kick as one captured graph (the pass's own
    graph has run with the same key), with new factors every step: over
    several steps positions, velocities and accelerations equal the same
    steps launched one by one in another context, bit for bit."""
    torch = pytest.importorskip("torch")
    pos, p = ics.make("zeldovich512", nside=24, maxleaf=16)
    n = pos.shape[0]
    vel = np.random.default_rng(5).standard_normal(pos.shape) * 0.5
    dkh, dd = _kdk_factors(ph)
    prec = getattr(ph, precision)
    fa, fb = ph.ForcePass(0), ph.ForcePass(0)
    acc0 = fa.run(pos, p, precision=prec)
    a = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (pos, vel, acc0)]
    b = [t.clone() for t in a]
    stream = torch.cuda.current_stream()
    fb.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    for step in range(4):
        k, d = dkh * (1 + 0.1 * step), dd * (1 - 0.05 * step)
        fa.kdk_step_device(*(t.data_ptr() for t in a), n, p, k, d, precision=prec)
        ph.kick(n, b[1].data_ptr(), b[2].data_ptr(), k, stream.cuda_stream)
        ph.drift(n, b[0].data_ptr(), b[1].data_ptr(), d, p["boxsize"], stream.cuda_stream)
        fb.run_device(b[0].data_ptr(), b[2].data_ptr(), n, p, precision=prec)
        ph.kick(n, b[1].data_ptr(), b[2].data_ptr(), k, stream.cuda_stream)
        torch.cuda.synchronize()
        for x, y in zip(a, b):
            assert torch.equal(x, y), step


@pytest.mark.gpu
@pytest.mark.parametrize("precision,maxleaf", [("FP32_SPLIT", 48), ("FP64", 16)])
def test_kdk_graph_step_whose_pass_outgrows_the_last_one(ph, ics, precision, maxleaf):
    """The captured step's pass does not fit what the previous pass needed:
    velocities toward the box centre gather the particles (each drift
    shrinks their distances to the centre by a quarter), so the list
    entries per leaf double from step to step and outgrow the mutual
    kernel's reaction buffer (its first guess, or what the last pass needed
    with 1/16 to spare).  The graph's second kick then stops itself and the
    call repeats the pass with a larger buffer (more launches than a step
    that fits, the last one here, which does not drift); positions,
    velocities and accelerations still equal the steps launched one by one,
    bit for bit.  Three drifts are as far as this input goes: on the fourth
    the mean-split tree needs more than 2N/MAXLEAF nodes, the reference's
    capacity."""
    torch = pytest.importorskip("torch")
    n = 32 ** 3
    L = 64.0
    p = ics.force_params(n, L, 128, theta=0.5, maxleaf=maxleaf)  # rcut 2.8
    prec = getattr(ph, precision)
    rng = np.random.default_rng(11)
    pos = rng.uniform(0.25 * L, 0.75 * L, (n, 3))
    dd = 0.01
    vel = -(pos - 0.5 * L) / (4.0 * dd)
    dkh = 1e-9  # the kicks stay tiny, so the motion is the drift's
    fa, fb = ph.ForcePass(0), ph.ForcePass(0)
    acc0 = fa.run(pos, p, precision=prec)
    a = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (pos, vel, acc0)]
    b = [t.clone() for t in a]
    stream = torch.cuda.current_stream()
    fb.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    count = ph.load_library().photons_launch_count
    pairs, launches = [], []
    for step, d in enumerate((dd, dd, dd, 0.0)):
        l0 = count()
        fa.kdk_step_device(*(t.data_ptr() for t in a), n, p, dkh, d, precision=prec)
        launches.append(count() - l0)
        c = fa.counters()
        pairs.append(c["pairs_local"] + c["pairs_image"])
        ph.kick(n, b[1].data_ptr(), b[2].data_ptr(), dkh, stream.cuda_stream)
        ph.drift(n, b[0].data_ptr(), b[1].data_ptr(), d, L, stream.cuda_stream)
        fb.run_device(b[0].data_ptr(), b[2].data_ptr(), n, p, precision=prec)
        ph.kick(n, b[1].data_ptr(), b[2].data_ptr(), dkh, stream.cuda_stream)
        torch.cuda.synchronize()
        for x, y in zip(a, b):
            assert torch.equal(x, y), step
    assert pairs[1] > 1.5 * pairs[0] and pairs[2] > 1.5 * pairs[1] and pairs[3] == pairs[2]
    assert launches[2] > launches[3]  # the repeated pass


@pytest.mark.gpu
@pytest.mark.parametrize("maxleaf", [16, 64])
def test_ordered_kdk_step_is_the_step_in_tree_order(ph, ics, maxleaf):
    """photons_kdk_step_ordered leaves pos, vel, acc and ids in the pass's
    tree order: after one step from the same state they are the plain
    step's arrays permuted by ids, bit for bit; over further steps (each
    build starting from the previous tree order) the trajectories agree to
    the FP32 rounding of the force."""
    torch = pytest.importorskip("torch")
    pos, p = ics.make("zeldovich512", nside=24, maxleaf=maxleaf)
    n = pos.shape[0]
    vel = np.random.default_rng(7).standard_normal(pos.shape) * 0.5
    dkh, dd = _kdk_factors(ph)
    fa, fb = ph.ForcePass(0), ph.ForcePass(0)
    acc0 = fa.run(pos, p, precision=ph.FP32_SPLIT)
    plain = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (pos, vel, acc0)]
    ordered = [t.clone() for t in plain]
    ids = torch.arange(n, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    for step in range(3):
        fa.kdk_step_device(*(t.data_ptr() for t in plain), n, p, dkh, dd, precision=ph.FP32_SPLIT)
        fb.kdk_step_ordered_device(*(t.data_ptr() for t in ordered), ids.data_ptr(), n, p, dkh, dd,
                                   precision=ph.FP32_SPLIT)
        torch.cuda.synchronize()
        idx = ids.cpu().numpy()
        assert np.array_equal(np.sort(idx), np.arange(n))
        got = [t.cpu().numpy() for t in ordered]
        want = [t.cpu().numpy()[idx] for t in plain]
        if step == 0:
            for g, w in zip(got, want):
                assert np.array_equal(g, w)
        else:
            L = p["boxsize"]
            dpos = np.abs(got[0] - want[0])
            dpos = np.minimum(dpos, L - dpos)  # periodic
            assert dpos.max() <= 1e-9 * L
            e = np.linalg.norm(got[2] - want[2], axis=1) / np.linalg.norm(want[2], axis=1)
            assert np.median(e) <= 1e-5


@pytest.mark.gpu
def test_ordered_kdk_step_with_pm(ph, ics):
    torch = pytest.importorskip("torch")
    pos, p = ics.make("zeldovich512", nside=24, maxleaf=64)
    n, nside = pos.shape[0], 24
    vel = np.random.default_rng(9).standard_normal(pos.shape) * 0.5
    dkh, dd = _kdk_factors(ph)
    fa, fb = ph.ForcePass(0), ph.ForcePass(0)
    acc0 = fa.run(pos, p, precision=ph.FP32_SPLIT)
    pm0 = fa.pm_force(pos, p, nside)
    plain = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (pos, vel, acc0, pm0)]
    ordered = [t.clone() for t in plain]
    ids = torch.arange(n, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    fa.kdk_step_pm_device(*(t.data_ptr() for t in plain), n, p, nside, dkh, dd, precision=ph.FP32_SPLIT)
    fb.kdk_step_ordered_device(ordered[0].data_ptr(), ordered[1].data_ptr(), ordered[2].data_ptr(), ids.data_ptr(),
                               n, p, dkh, dd, precision=ph.FP32_SPLIT, nside=nside,
                               acc_pm_ptr=ordered[3].data_ptr())
    torch.cuda.synchronize()
    idx = ids.cpu().numpy()
    got = [t.cpu().numpy() for t in ordered]
    want = [t.cpu().numpy()[idx] for t in plain]
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[2], want[2])
    # the PM deposit adds with atomics: its last bits vary between runs
    assert np.abs(got[3] - want[3]).max() <= 1e-12 * np.abs(want[3]).max()
    assert np.abs(got[1] - want[1]).max() <= 1e-12 * np.abs(want[1]).max()
