"""The reference-named entry points (fmm_construct ... fmm_ext) driven
through the reference's globals, as src/photoNs.c:97-116 drives them, and
the batched operators and the FP64 direct sum against the oracle."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def rel_err(a, b, p):
    """Per-particle relative error |a-b|/|b|.  Where the net force cancels
    below 1e-4 of one nearest-neighbour pair force m/D^2 (D = L/N^(1/3);
    exact lattices cancel to ~1e-5 of it), the error is taken relative to
    that floor instead of the cancelled value."""
    nb = np.linalg.norm(b, axis=1)
    spacing = p["boxsize"] / np.cbrt(b.shape[0])
    floor = 1e-4 * p["mass"] / spacing ** 2
    return np.linalg.norm(a - b, axis=1) / np.maximum(nb, floor)


@pytest.mark.parametrize("name", ["grid16_leaf16", "nfw16_leaf8"])
def test_driver_sequence_matches_reference(ph, name):
    g = load_golden(name)
    ref = ph.Reference()
    ref.setup(g["pos_in"], g["p"])
    acc_task = ref.force_pass()
    part = ref.part()
    # part[] permuted into tree order, like the reference
    assert np.array_equal(part["pos"], g["pos_tree"])
    assert rel_err(acc_task, g["acc_task"], g["p"]).max() <= 1e-10
    assert rel_err(part["acc"], g["acc"], g["p"]).max() <= 1e-10
    c = ref.counters()
    assert c["idxP2P"] == g["counters"][0]
    assert c["idxM2L"] == g["counters"][1]
    assert c["walk_m2l_count"] == g["counters"][2]
    assert c["p2p_count_remote"] == g["counters"][3]
    ref.deconstruct()


def _pm_golden():
    import glob
    import os
    from conftest import GOLDEN
    return sorted(glob.glob(os.path.join(GOLDEN, "pm", "*.npz")))


@pytest.mark.parametrize("path", _pm_golden(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_partmesh_matches_reference_pm(ph, path):
    """partmesh_thread() on the reference's globals against the reference's
    own partmesh.c outputs (cuFFT against a direct DFT: last bits)."""
    z = np.load(path)
    L, N, rs, m = z["params"]
    ref = ph.Reference()
    ref.setup(z["pos"], dict(boxsize=L, theta=0.5, rs=rs, rcut=4.5 * rs, eps=0.0, mass=m, maxleaf=16))
    got = ref.pm(int(N))
    want = z["acc_pm"]
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()


def test_driver_sequence_with_pm_thread(ph):
    """The driver's step with the PM on its own thread beside fmm_task: the
    FMM result is unchanged and acc_pm is the PM of the tree-ordered part[]."""
    import pm_oracle
    g = load_golden("grid16_leaf16")
    ref = ph.Reference()
    ref.setup(g["pos_in"], g["p"])
    nside = 16
    ref.force_pass(pm_nside=nside)
    part = ref.part()
    assert rel_err(part["acc"], g["acc"], g["p"]).max() <= 1e-10
    p = g["p"]
    want = pm_oracle.pm_force(part["pos"], p["boxsize"], nside, p["rs"], p["mass"])
    assert np.abs(part["acc_pm"] - want).max() <= 1e-10 * np.abs(want).max()
    ref.deconstruct()


def test_operators_match_oracle(ph, port):
    rng = np.random.default_rng(2)
    n = 64
    d = rng.normal(size=(n, 3)) * 4
    M = rng.normal(size=(n, 20))
    L0 = rng.normal(size=(n, 20))
    rs = 1.7
    got = ph.op_batch("m2l", d, M, L0, rs)
    want = np.array([L0[i] + port.m2l(d[i], M[i], rs) for i in range(n)])
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    got = ph.op_batch("m2m", d, M, L0)
    want = np.array([L0[i] + port.m2m(d[i], M[i]) for i in range(n)])
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    got = ph.op_batch("l2l", d, M, L0)
    want = np.array([L0[i] + port.l2l(d[i], M[i]) for i in range(n)])
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_direct_sum_matches_oracle(ph, port, ics):
    pos, p = ics.make("nfw128", nside=24)
    targets = np.random.default_rng(4).choice(pos.shape[0], 500, replace=False).astype(np.int32)
    got = ph.direct_sum(pos, p, targets)
    want = port.direct_sum(pos, p, targets, nthreads=8)
    assert rel_err(got, want, p).max() <= 1e-10


def test_fp32_fma_probe_runs(ph):
    v = ph.fp32_fma_peak(2048)
    assert 1.0 < v < 1000.0


IMAGE_SHIFTS = [(mi, mj, mk) for mi in (-1, 0, 1) for mj in (-1, 0, 1) for mk in (-1, 0, 1) if (mi, mj, mk) != (0, 0, 0)]


@pytest.mark.parametrize("name", ["grid16_leaf16", "nfw16_leaf8"])
def test_fmm_remote_per_image_then_host_downward(ph, name):
    """fmm_ext's own sequence spelled out through the exported entry points
    (src/fmm.c:1028-1070): after fmm_task, fmm_remote(0, shift) for the 26
    image shifts, then the host walk_l2l from the root and l2p of every
    leaf.  The accelerations and counters equal the reference's pass (the
    nfw16 fixture has local and image M2L, so the host downward pass carries
    the GPU's local expansions)."""
    import ctypes as C
    g = load_golden(name)
    p = g["p"]
    ref = ph.Reference()
    ref.setup(g["pos_in"], p)
    lib = ref.lib
    lib.walk_l2l.argtypes = [C.c_int]
    lib.l2p.argtypes = [C.c_int]
    lib.fmm_construct()
    lib.fmm_prepare()
    lib.fmm_task()
    part = ref.part()
    assert rel_err(part["acc"].copy(), g["acc_task"], p).max() <= 1e-10
    for s in IMAGE_SHIFTS:
        shift = (C.c_double * 3)(*(float(v) * p["boxsize"] for v in s))
        lib.fmm_remote(0, shift)
    first_node = C.c_int.in_dll(lib, "first_node").value
    first_leaf, last_leaf = C.c_int.in_dll(lib, "first_leaf").value, C.c_int.in_dll(lib, "last_leaf").value
    lib.walk_l2l(first_node)
    for n in range(first_leaf, last_leaf):
        lib.l2p(n)
    assert rel_err(part["acc"], g["acc"], p).max() <= 1e-10
    c = ref.counters()
    assert [c[k] for k in ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote")] == list(g["counters"][:4])
    ref.deconstruct()


@pytest.mark.parametrize("entry", ["p2p_kernel", "p2p_kernel_rinvsqrt"])
def test_kernels_h_leaf_pairs_sum_to_the_local_task_phase(ph, entry):
    """The inc/kernels.h entry points, one call per task of the reference's
    own local P2P list (in its order; a leaf with itself through
    p2p_kernel_inleaf), after fmm_prepare: part[].acc equals the
    reference's accelerations after fmm_task (no M2L in this fixture)."""
    g = load_golden("grid16_leaf16")
    p = g["p"]
    ref = ph.Reference()
    ref.setup(g["pos_in"], p)
    lib = ref.lib
    for name in ("p2p_kernel", "p2p_kernel_rinvsqrt", "p2p_kernel_inleaf"):
        getattr(lib, name).argtypes = [C_int(), C_int()]
        getattr(lib, name).restype = None
    lib.fmm_construct()
    lib.fmm_prepare()
    part = ref.part()
    part["acc"] = 0.0
    fn = getattr(lib, entry)
    t, s, _ = g["list_p2p"]
    for a, b in zip(t.tolist(), s.tolist()):
        if a == b and entry == "p2p_kernel":
            lib.p2p_kernel_inleaf(a, b)
        else:
            fn(a, b)
    assert ph.load_library().photons_gpu_status() == 0
    assert rel_err(part["acc"], g["acc_task"], p).max() <= 1e-10
    ref.deconstruct()


def C_int():
    import ctypes
    return ctypes.c_int
