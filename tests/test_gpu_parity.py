"""GPU force pass against the reference: golden fixtures (reference
outputs) and the CPU oracle on the same seeded inputs, through the C ABI.

Tolerances: the FP64 GPU variant must match per-particle accelerations to
1e-10 relative (the reference's FP64 arithmetic in a different summation
order); interaction-list counts and lists must match exactly.  The FP32
split variant is checked against the FP64 GPU variant on the same lists:
median relative error <= 2e-6 and 99th percentile <= 2e-5 here (the north
star's budget is a median of 1e-4)."""
import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

COUNTERS = ["idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "NLEAF", "NNODE", "nleaf", "nnode",
            "first_leaf", "first_node", "direct_local_start", "n_p2p", "n_m2l", "n_p2p_ext", "n_m2l_ext",
            "n_images"]
FP64_TOL = 1e-10


def digest(t, s, im):
    key = (t.astype(np.int64) << 34) | (s.astype(np.int64) << 5) | im.astype(np.int64)
    key.sort()
    return hashlib.sha256(key.tobytes()).hexdigest()


def rel_err(a, b, p):
    """Per-particle relative error |a-b|/|b|.  Where the net force cancels
    below 1e-4 of one nearest-neighbour pair force m/D^2 (D = L/N^(1/3);
    exact lattices cancel to ~1e-5 of it), the error is taken relative to
    that floor instead of the cancelled value."""
    nb = np.linalg.norm(b, axis=1)
    spacing = p["boxsize"] / np.cbrt(b.shape[0])
    floor = 1e-4 * p["mass"] / spacing ** 2
    return np.linalg.norm(a - b, axis=1) / np.maximum(nb, floor)


@pytest.fixture(scope="module")
def fp(ph):
    f = ph.ForcePass(0)
    yield f
    f.close()


@pytest.mark.parametrize("name", golden_names())
def test_fp64_matches_reference_golden(ph, fp, name):
    g = load_golden(name)
    acc = fp.run(g["pos_in"], g["p"], precision=ph.FP64, flags=ph.F_TREE_ORDER | ph.F_KEEP_LISTS | ph.F_MULTIPOLES)
    c = fp.counters()
    assert [c[k] for k in COUNTERS] == list(g["counters"])
    # the reference's permutation of part[]
    assert np.array_equal(fp.positions(), g["pos_tree"])
    # every interaction list, as a multiset
    for kind, (t, s, im) in fp.lists().items():
        assert digest(t, s, im) == str(g["digest_" + kind]), kind
    # tree: integer structure exact, geometry to the last bits of the mean
    tr = fp.tree()
    for k in ("leaf_ipart", "leaf_npart", "node_npart", "node_son"):
        assert np.array_equal(tr[k], g["tree_" + k]), k
    for k in ("leaf_center", "leaf_width", "node_center", "node_width", "node_split"):
        assert np.allclose(tr[k], g["tree_" + k], rtol=1e-13, atol=1e-13 * g["p"]["boxsize"]), k
    if "tree_node_M" in g:
        for k in ("leaf_M", "node_M"):
            ref = g["tree_" + k]
            assert np.abs(tr[k] - ref).max() <= 1e-11 * (np.abs(ref).max() + 1e-300), k
    assert rel_err(acc, g["acc"], g["p"]).max() <= FP64_TOL
    # local task phase alone (src/fmm.c:909-984): local P2P, no far field
    if "acc_task" in g:
        acc_task = fp.run(g["pos_in"], g["p"], precision=ph.FP64, image_mask=1,
                          flags=ph.F_TREE_ORDER | ph.F_NO_FARFIELD)
        assert rel_err(acc_task, g["acc_task"], g["p"]).max() <= FP64_TOL


@pytest.mark.parametrize("name", golden_names())
def test_fp32_split_precision_golden(ph, fp, name):
    g = load_golden(name)
    a64 = fp.run(g["pos_in"], g["p"], precision=ph.FP64)
    a32 = fp.run(g["pos_in"], g["p"], precision=ph.FP32_SPLIT)
    if name.startswith("lattice"):
        # net forces are ~1e-5 residuals of cancelling pair forces: bound the
        # error against one nearest-neighbour pair force instead
        pair = g["p"]["mass"] / (g["p"]["boxsize"] / np.cbrt(a64.shape[0])) ** 2
        assert np.abs(a32 - a64).max() <= 1e-5 * pair
        return
    e = rel_err(a32, a64, g["p"])
    if name.startswith("demo"):
        # z = 49 initial conditions: displacements are a small fraction of the
        # spacing, so net forces are residuals of much larger pair forces and
        # FP32 rounding is amplified relative to them (still far inside 1e-4)
        assert np.median(e) <= 1e-5, np.median(e)
        assert np.percentile(e, 99) <= 1e-4, np.percentile(e, 99)
        return
    assert np.median(e) <= 2e-6, np.median(e)
    assert np.percentile(e, 99) <= 2e-5, np.percentile(e, 99)


@pytest.mark.parametrize("workload,nside,maxleaf", [("grid32", 32, 16), ("nfw128", 32, 8), ("grid32", 24, 32),
                                                    ("nfw128", 28, 64)])
def test_fp64_matches_oracle(ph, fp, ics, port, workload, nside, maxleaf):
    pos, p = ics.make(workload, nside=nside, maxleaf=maxleaf)
    r = port.run(pos, p, capture=False, tree=False, nthreads=8)
    acc = fp.run(pos, p, precision=ph.FP64)
    c = fp.counters()
    for k in COUNTERS[:10] + ["n_p2p_ext", "n_m2l_ext"]:
        assert c[k] == r["counters"][k], k
    acc_ref = np.empty_like(r["acc"])
    acc_ref[r["perm"]] = r["acc"]
    assert rel_err(acc, acc_ref, p).max() <= FP64_TOL


def test_pass_is_deterministic(ph, fp, ics):
    pos, p = ics.make("nfw128", nside=24, maxleaf=8)
    for prec in (ph.FP32_SPLIT, ph.FP64):
        a = fp.run(pos, p, precision=prec)
        b = fp.run(pos, p, precision=prec)
        assert np.array_equal(a, b)


def test_device_io_matches_host_io(ph, fp, ics):
    torch = pytest.importorskip("torch")
    pos, p = ics.make("grid32", nside=16)
    host = fp.run(pos, p, precision=ph.FP32_SPLIT)
    dpos = torch.from_numpy(pos).cuda()
    dacc = torch.empty_like(dpos)
    torch.cuda.synchronize()
    fp.run_device(dpos.data_ptr(), dacc.data_ptr(), pos.shape[0], p, precision=ph.FP32_SPLIT)
    assert np.array_equal(dacc.cpu().numpy(), host)


@pytest.mark.parametrize("precision", ["FP64", "FP32_SPLIT"])
def test_graph_pass_matches_stage_pass(ph, ics, monkeypatch, precision):
    """The captured-graph pass (default) and the stage-by-stage pass give
    identical accelerations; so does a graph whose first capture launches
    too few tree levels and is grown and re-captured."""
    pos, p = ics.make("nfw128", nside=32, maxleaf=8)
    prec = getattr(ph, precision)
    graph = ph.ForcePass(0).run(pos, p, precision=prec)
    monkeypatch.setenv("PHOTONS_GRAPH", "0")
    stages = ph.ForcePass(0).run(pos, p, precision=prec)
    monkeypatch.delenv("PHOTONS_GRAPH")
    monkeypatch.setenv("PHOTONS_TREE_LEVELS", "2")
    fp = ph.ForcePass(0)
    grown = fp.run(pos, p, precision=prec)
    again = fp.run(pos, p, precision=prec)
    assert np.array_equal(graph, stages)
    assert np.array_equal(graph, grown)
    assert np.array_equal(graph, again)
    assert fp.counters()["depth"] > 2


@pytest.mark.parametrize("workload,nside,maxleaf", [("grid32", 32, 48), ("nfw128", 32, 64), ("zeldovich256", 32, 64),
                                                    ("nfw128", 40, 48), ("zeldovich256", 32, 60),
                                                    ("zeldovich256", 24, 56)])
def test_mutual_pairs_match_one_way(ph, ics, monkeypatch, workload, nside, maxleaf):
    """The FP32 kernel that evaluates each symmetric leaf pair (local or
    periodic image) once, reactions through a buffer, against the one-way
    kernel and the FP64 pass: the same forces to FP32 rounding,
    deterministic from pass to pass.  Covers the default build at leaf
    48-64, the 48-slot tile (halo leaves of 33-48 particles) and lists too
    long to pair (every build: the next test)."""
    pos, p = ics.make(workload, nside=nside, maxleaf=maxleaf)
    fp = ph.ForcePass(0)
    a64 = fp.run(pos, p, precision=ph.FP64)
    mutual = fp.run(pos, p, precision=ph.FP32_SPLIT)
    again = fp.run(pos, p, precision=ph.FP32_SPLIT)
    monkeypatch.setenv("PHOTONS_P2P_KERNEL", "packed")
    one_way = ph.ForcePass(0).run(pos, p, precision=ph.FP32_SPLIT)
    assert np.array_equal(mutual, again)
    e_mu, e_ow = rel_err(mutual, a64, p), rel_err(one_way, a64, p)
    assert np.median(e_mu) <= 1.5 * np.median(e_ow) + 1e-7, (np.median(e_mu), np.median(e_ow))
    assert np.percentile(e_mu, 99) <= 2e-5
    assert np.median(rel_err(mutual, one_way, p)) <= 5e-6


@pytest.mark.parametrize("workload,nside,maxleaf", [("zeldovich256", 32, 64), ("nfw128", 40, 48)])
def test_every_p2p_build_gives_the_same_forces(ph, ics, workload, nside, maxleaf):
    """The mutual kernel's builds that the autotuner chooses between
    (resident blocks per SM, interleaved dependency chains, the 6-target
    path): each is deterministic, within the split-precision bar of the FP64
    pass, and agrees with the others to FP32 rounding; an unknown build is
    an error."""
    pos, p = ics.make(workload, nside=nside, maxleaf=maxleaf)
    fp = ph.ForcePass(0)
    a64 = fp.run(pos, p, precision=ph.FP64)
    base = None
    for shape in range(ph.P2P_SHAPES):
        flags = ph.F_P2P_SHAPE(shape)
        a = fp.run(pos, p, precision=ph.FP32_SPLIT, flags=flags)
        assert np.array_equal(a, fp.run(pos, p, precision=ph.FP32_SPLIT, flags=flags))
        e = rel_err(a, a64, p)
        assert np.median(e) <= 2e-6 and np.percentile(e, 99) <= 2e-5, (shape, np.median(e))
        base = a if base is None else base
        assert np.median(rel_err(a, base, p)) <= 1e-6, shape
    with pytest.raises(ph.PhotonsError, match="shape"):
        fp.run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_P2P_SHAPE(ph.P2P_SHAPES))
    fp.close()


@pytest.mark.parametrize("workload,nside,maxleaf", [("zeldovich256", 32, 64), ("nfw128", 32, 48)])
def test_bulk_staged_sources_give_the_same_forces(ph, ics, workload, nside, maxleaf):
    """Source leaves staged by TMA bulk copies (one copy per entry,
    completing on the stage's mbarrier) or by per-lane cp.async: the same
    bytes reach shared memory, so every build gives bit-identical forces."""
    pos, p = ics.make(workload, nside=nside, maxleaf=maxleaf)
    fp = ph.ForcePass(0)
    for shape in range(ph.P2P_SHAPES):
        a = fp.run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_P2P_SHAPE(shape))
        b = fp.run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_P2P_SHAPE(shape) | ph.F_P2P_BULK)
        assert np.array_equal(a, b), shape
    fp.close()


def test_bulk_staging_wait_has_a_time_limit(ph, ics, monkeypatch):
    """A bulk copy whose mbarrier never completes (the test hook arms it for
    16 bytes more than the copy brings): every staging wait gives up after
    its two-second limit, the pass fails with an error instead of hanging,
    and the context then runs the same pass correctly."""
    import time

    pos, p = ics.make("zeldovich256", nside=16, maxleaf=64)
    fp = ph.ForcePass(0)
    good = fp.run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_P2P_BULK)
    monkeypatch.setenv("PHOTONS_TEST_STAGE_SHORTFALL", "1")
    t0 = time.time()
    with pytest.raises(ph.PhotonsError, match="bulk copy did not complete"):
        fp.run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_P2P_BULK)
    assert time.time() - t0 < 60
    monkeypatch.delenv("PHOTONS_TEST_STAGE_SHORTFALL")
    assert np.array_equal(fp.run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_P2P_BULK), good)
    fp.close()


def test_mutual_pairs_graph_and_stage_paths_agree(ph, ics, monkeypatch):
    """The mutual kernel inside the captured graph and launched stage by
    stage (where the reaction buffer is sized between the stages) agree
    bit for bit."""
    pos, p = ics.make("zeldovich256", nside=40, maxleaf=56)
    graph = ph.ForcePass(0).run(pos, p, precision=ph.FP32_SPLIT)
    monkeypatch.setenv("PHOTONS_GRAPH", "0")
    stages = ph.ForcePass(0).run(pos, p, precision=ph.FP32_SPLIT)
    assert np.array_equal(graph, stages)


def test_one_way_flag_selects_the_one_way_kernel(ph, ics, monkeypatch):
    """PHOTONS_F_ONE_WAY at leaf 64 runs the one-way kernel: the same
    accelerations, bit for bit, as forcing it through the environment."""
    pos, p = ics.make("zeldovich256", nside=32, maxleaf=64)
    flagged = ph.ForcePass(0).run(pos, p, precision=ph.FP32_SPLIT, flags=ph.F_ONE_WAY)
    mutual = ph.ForcePass(0).run(pos, p, precision=ph.FP32_SPLIT)
    monkeypatch.setenv("PHOTONS_P2P_KERNEL", "packed")
    packed = ph.ForcePass(0).run(pos, p, precision=ph.FP32_SPLIT)
    assert np.array_equal(flagged, packed)
    assert not np.array_equal(flagged, mutual)  # the default at leaf 64 is the mutual kernel
    assert np.median(rel_err(flagged, mutual, p)) <= 5e-6


def test_autotuner_times_both_kernels_from_leaf_48(ph, ics):
    pos, p = ics.make("nfw128", nside=32, maxleaf=16)
    fp = ph.ForcePass(0)
    best, table, flags = ph.autotune_leaf(fp, pos, p, candidates=(32, 48), sample=500, repeats=1)
    assert sorted((r["maxleaf"], r["kernel"]) for r in table) == [(32, "one-way"), (48, "mutual"), (48, "one-way")]
    chosen = [r for r in table if r["maxleaf"] == best and r["flags"] == flags]
    assert len(chosen) == 1
    ok = [r for r in table if r["median"] <= 1e-4]
    if ok:
        assert chosen[0]["ms"] == min(r["ms"] for r in ok)


def test_context_release_returns_device_memory(ph, ics):
    """Contexts that ran passes of both precisions (tree, lists, reaction
    slots, captured graphs) give their device memory back on release."""
    torch = pytest.importorskip("torch")
    pos, p = ics.make("zeldovich256", nside=32, maxleaf=64)
    torch.cuda.synchronize()
    f = ph.ForcePass(0)  # a first context pays the library's one-time setup
    f.run(pos, p, precision=ph.FP32_SPLIT)
    f.close()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        f = ph.ForcePass(0)
        f.run(pos, p, precision=ph.FP32_SPLIT)
        f.run(pos, p, precision=ph.FP64)
        f.close()
    torch.cuda.synchronize()
    assert free0 - torch.cuda.mem_get_info()[0] < (64 << 20)


def test_capacity_overflow_is_an_error(ph, fp):
    pos = np.full((100, 3), 3.0)
    p = dict(boxsize=10.0, theta=0.5, rs=1.0, rcut=4.5, eps=0.01, mass=1.0, maxleaf=8)
    with pytest.raises(ph.PhotonsError, match="error 4"):
        fp.run(pos, p, precision=ph.FP64)
    # the context stays usable
    pos2 = np.random.default_rng(0).random((500, 3)) * 10.0
    fp.run(pos2, p, precision=ph.FP64)


def test_too_few_particles_is_an_error(ph, fp):
    pos = np.random.default_rng(1).random((8, 3))
    p = dict(boxsize=1.0, theta=0.5, rs=0.1, rcut=0.45, eps=0.01, mass=1.0, maxleaf=8)
    with pytest.raises(ph.PhotonsError, match="error 5"):
        fp.run(pos, p)


@pytest.mark.parametrize("nside,maxleaf", [(32, 8), (40, 16)])
def test_fp32_split_precision_clustered(ph, fp, ics, nside, maxleaf):
    """Clustered input with many M2L tasks: the split far field (FP32 M2L
    and L2P) stays within the precision budget of the FP64 pass."""
    pos, p = ics.make("nfw128", nside=nside, maxleaf=maxleaf)
    a64 = fp.run(pos, p, precision=ph.FP64)
    assert fp.counters()["walk_m2l_count"] > 1000
    a32 = fp.run(pos, p, precision=ph.FP32_SPLIT)
    e = rel_err(a32, a64, p)
    assert np.median(e) <= 2e-6, np.median(e)
    assert np.percentile(e, 99) <= 2e-5, np.percentile(e, 99)


@pytest.mark.parametrize("workload,nside,maxleaf", [("zeldovich256", 32, 64), ("nfw128", 32, 16),
                                                    ("nfw128", 24, 100), ("grid32", 16, 8)])
def test_fp64_mutual_matches_one_way(ph, ics, workload, nside, maxleaf):
    """FP64 passes evaluate each symmetric leaf pair (local or periodic
    image) once, reactions through the slot buffer: the same forces as the
    one-way FP64 kernel to FP64 rounding, deterministic from pass to pass.
    Leaf 100 runs targets in two chunks of up to 64."""
    pos, p = ics.make(workload, nside=nside, maxleaf=maxleaf)
    fp = ph.ForcePass(0)
    mutual = fp.run(pos, p, precision=ph.FP64)
    again = fp.run(pos, p, precision=ph.FP64)
    one_way = ph.ForcePass(0).run(pos, p, precision=ph.FP64, flags=ph.F_ONE_WAY)
    assert np.array_equal(mutual, again)
    assert rel_err(mutual, one_way, p).max() <= 1e-12


def test_pass_with_library_pinned_buffers(ph, ics):
    """Host buffers from photons_host_alloc (ph.host_array), which the
    pass's kernels read and write over the host link, give the same forces
    as pageable host arrays (copied by cudaMemcpyAsync), also through views
    that start 8 bytes off a 16-byte boundary (the copy kernel's 8-byte
    path), and are released with the array."""
    pos, p = ics.make("zeldovich256", nside=24, maxleaf=64)
    fp = ph.ForcePass(0)
    plain = fp.run(pos, p, precision=ph.FP32_SPLIT)
    hp = ph.host_array(pos.shape)
    hp[:] = pos
    ha = ph.host_array(pos.shape)
    fp.run(hp, p, precision=ph.FP32_SPLIT, out=ha)
    assert np.array_equal(ha, plain)
    n = pos.shape[0]
    hp2 = ph.host_array((3 * n + 1,))
    ha2 = ph.host_array((3 * n + 1,))
    vp, va = hp2[1:].reshape(n, 3), ha2[1:].reshape(n, 3)  # 8 bytes into the pinned blocks
    assert vp.ctypes.data % 16 == 8 and va.ctypes.data % 16 == 8
    vp[:] = pos
    fp.run(vp, p, precision=ph.FP32_SPLIT, out=va)
    assert np.array_equal(va, plain)
    del hp, ha, vp, va, hp2, ha2


def _full_size_parity(ph, fp, port, pos, p, precision, tol, nsub=10000):
    """The GPU pass against the oracle at a workload's full size: counters,
    the tree-order permutation, every list as a multiset, and the forces on
    a random subset of particles (the oracle forms only those)."""
    import os
    n = pos.shape[0]
    tg = np.random.default_rng(17).choice(n, nsub, replace=False).astype(np.int32)
    r = port.run_sample(pos, p, tg, nthreads=os.cpu_count() or 4, lists=True, perm=True)
    acc = fp.run(pos, p, precision=precision, flags=ph.F_KEEP_LISTS)
    c = fp.counters()
    for k in ("nleaf", "nnode", "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "n_p2p_ext", "n_m2l_ext",
              "pairs_local", "pairs_image"):
        assert c[k] == r["counters"][k], k
    assert np.array_equal(fp.perm(), r["perm"])
    gl = fp.lists()
    for kind, (t, s, im) in r["lists"].items():
        assert digest(*gl[kind]) == digest(t, s, im), kind
    e = rel_err(acc[tg], r["acc"], p)
    assert e.max() <= tol, e.max()
    return e


@pytest.mark.parametrize("maxleaf", [16, 24])
def test_c1_nfw128_full_size_matches_oracle(ph, fp, ics, port, maxleaf):
    """128^3 particles, 50 % in 64 NFW halos (local and image M2L occur): the
    reference's leaf 16 and the autotuned leaf 24, FP64 within 1e-10."""
    pos, p = ics.make("nfw128", maxleaf=maxleaf)
    _full_size_parity(ph, fp, port, pos, p, ph.FP64, FP64_TOL)


def test_c2_zeldovich256_full_size_lists_match_oracle(ph, fp, ics, port):
    """The headline input, 256^3 at leaf 64: tree, permutation, counters and
    lists identical to the oracle's; the FP32 split forces on 10^4 particles
    within the split-precision bar of the oracle's FP64 ones."""
    pos, p = ics.make("zeldovich256", maxleaf=64)
    e = _full_size_parity(ph, fp, port, pos, p, ph.FP32_SPLIT, 1e-3)
    assert np.median(e) <= 2e-6, np.median(e)
