"""The CPU oracle (oracle/photons_oracle.c) against the reference: the
committed golden fixtures (made by the reference's own sources), and the
reference library itself where its tree is present."""
import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden

COUNTERS = ["idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "NLEAF", "NNODE", "nleaf", "nnode",
            "first_leaf", "first_node", "direct_local_start", "n_p2p", "n_m2l", "n_p2p_ext", "n_m2l_ext",
            "n_images"]


def digest(t, s, im):
    key = (t.astype(np.int64) << 34) | (s.astype(np.int64) << 5) | im.astype(np.int64)
    key.sort()
    return hashlib.sha256(key.tobytes()).hexdigest()


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_golden(port, name):
    g = load_golden(name)
    r = port.run(g["pos_in"], g["p"], capture=True, tree=True, nthreads=4)
    assert [r["counters"][k] for k in COUNTERS] == list(g["counters"])
    # the same in-place permutation of the particles
    assert np.array_equal(r["pos"], g["pos_tree"])
    assert np.array_equal(g["pos_in"][r["perm"]], r["pos"])
    for kind, (t, s, im) in r["lists"].items():
        assert digest(t, s, im) == str(g["digest_" + kind]), kind
        if "list_" + kind in g:
            # full lists, in the reference's order
            assert np.array_equal(np.stack([t, s, im]), g["list_" + kind]), kind
    # without M2L the sums run in the reference's order: identical bits
    if "acc_task" in g:
        assert np.array_equal(r["acc_task"], g["acc_task"])
    if g["counters"][2] == 0:
        assert np.array_equal(r["acc"], g["acc"])
    else:
        assert rel_err(r["acc"], g["acc"]).max() < 1e-12
    for k in ("leaf_ipart", "leaf_npart", "node_npart", "node_son", "leaf_center", "leaf_width", "node_center",
              "node_width", "node_split"):
        assert np.array_equal(r["tree"][k], g["tree_" + k]), k
    for k in ("leaf_M", "node_M", "leaf_L", "node_L"):
        if "tree_" + k in g:
            ref = g["tree_" + k]
            scale = np.abs(ref).max() + 1e-300
            assert np.abs(r["tree"][k] - ref).max() <= 1e-12 * scale, k


def test_port_threads_bit_identical(port, ics):
    pos, p = ics.make("grid32", nside=16)
    a = port.run(pos, p, capture=False, tree=False, nthreads=1)["acc"]
    b = port.run(pos, p, capture=False, tree=False, nthreads=7)["acc"]
    assert np.array_equal(a, b)


def test_operators_match_reference(oracle_mod, port):
    if not oracle_mod.ref_available():
        pytest.skip("reference oracle not built here")
    ref = oracle_mod.RefOracle()
    rng = np.random.default_rng(5)
    for _ in range(50):
        d = rng.normal(size=3) * 5
        M = rng.normal(size=20)
        rs = rng.uniform(0.5, 4.0)
        a, b = ref.m2l(d, M, rs), port.m2l(d, M, rs)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()
        a, b = ref.m2m(d, M), port.m2m(d, M)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()
        a, b = ref.l2l(d, M), port.l2l(d, M)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()


def test_acceptance_matches_reference(oracle_mod, port):
    if not oracle_mod.ref_available():
        pytest.skip("reference oracle not built here")
    ref = oracle_mod.RefOracle()
    rng = np.random.default_rng(9)
    cases = []
    for _ in range(3000):
        wi = rng.uniform(0.1, 4.0, 3)
        wj = rng.uniform(0.1, 4.0, 3)
        dist = rng.normal(size=3) * 8
        cases.append((wi, wj, dist))
    # touching boxes, exactly adjacent faces
    for _ in range(200):
        wi = rng.uniform(0.5, 2.0, 3)
        wj = rng.uniform(0.5, 2.0, 3)
        dist = (wi + wj) * 0.5 * rng.choice([-1.0, 0.0, 1.0], 3)
        cases.append((wi, wj, dist))
    for theta in (0.3, 0.5, 0.8):
        for wi, wj, dist in cases:
            assert ref.acceptance(wi, wj, dist, theta, 10.0) == port.acceptance(wi, wj, dist, theta, 10.0)


def test_port_matches_reference_full_c0(oracle_mod, port, ics):
    """The 32^3 workload against the reference library run here."""
    if not oracle_mod.ref_available():
        pytest.skip("reference oracle not built here")
    pos, p = ics.make("grid32")
    r = oracle_mod.RefOracle().run(pos, p, capture=False, tree=False)
    q = port.run(pos, p, capture=False, tree=False, nthreads=8)
    assert {k: r["counters"][k] for k in COUNTERS[:10]} == {k: q["counters"][k] for k in COUNTERS[:10]}
    assert np.array_equal(r["acc"], q["acc"])


def test_capacity_overflow_is_an_error(port):
    """Coincident particles defeat the mean split; the reference would write
    past its 2N/MAXLEAF leaf array (src/fmm.c:203-209)."""
    pos = np.full((100, 3), 3.0)
    p = dict(boxsize=10.0, theta=0.5, rs=1.0, rcut=4.5, eps=0.01, mass=1.0, maxleaf=8)
    with pytest.raises(RuntimeError, match="code [34]"):
        port.run(pos, p, capture=False, tree=False)


def test_too_few_particles_is_an_error(port):
    pos = np.random.default_rng(1).random((8, 3))
    p = dict(boxsize=1.0, theta=0.5, rs=0.1, rcut=0.45, eps=0.01, mass=1.0, maxleaf=8)
    with pytest.raises(RuntimeError, match="code 5"):
        port.run(pos, p, capture=False, tree=False)


def test_direct_sum_small(port):
    rng = np.random.default_rng(3)
    L = 10.0
    pos = rng.random((300, 3)) * L
    p = dict(boxsize=L, theta=0.5, rs=0.5, rcut=2.25, eps=0.05, mass=2.0, maxleaf=8)
    targets = np.arange(0, 300, 7, dtype=np.int32)
    got = port.direct_sum(pos, p, targets, rmax=4.0)
    from scipy.special import erfc
    for k, i in enumerate(targets):
        d = pos - pos[i]
        d -= L * np.round(d / L)
        r = np.linalg.norm(d, axis=1)
        m = (r < 4.0) & (np.arange(300) != i)
        rr = r[m]
        u = 0.5 * rr / p["rs"]
        f = p["mass"] * (erfc(u) + 2 / np.sqrt(np.pi) * u * np.exp(-u * u)) / np.maximum(rr, p["eps"]) ** 3
        want = (d[m] * f[:, None]).sum(0)
        assert np.allclose(got[k], want, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("name,nside,maxleaf", [("grid32", 16, 16), ("nfw128", 24, 8)])
def test_port_walks_on_threads_keep_the_sequential_lists(port, ics, name, nside, maxleaf):
    """The walks run as sub-walks on several threads and are concatenated in
    traversal order: the lists equal the one-thread walk's, in order."""
    pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
    a = port.run(pos, p, capture=True, tree=False, nthreads=1)
    b = port.run(pos, p, capture=True, tree=False, nthreads=6)
    assert a["counters"] == b["counters"]
    for kind in a["lists"]:
        assert all(np.array_equal(x, y) for x, y in zip(a["lists"][kind], b["lists"][kind])), kind
    assert np.array_equal(a["acc"], b["acc"])


@pytest.mark.parametrize("name,nside,maxleaf", [("zeldovich256", 20, 64), ("nfw128", 24, 8)])
def test_port_sampled_pass_equals_full_pass(port, ics, name, nside, maxleaf):
    """Forces for a target subset only (the parity leg at full size): the
    subset's accelerations, counters and permutation are the full pass's,
    bit for bit, also when the tree is reused for another subset; the pair
    counts are the reference's pair set."""
    pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
    n = pos.shape[0]
    full = port.run(pos, p, capture=True, tree=True, nthreads=4)
    acc = np.empty_like(full["acc"])
    acc[full["perm"]] = full["acc"]
    rng = np.random.default_rng(3)
    tg = rng.choice(n, 300, replace=False).astype(np.int32)
    r = port.run_sample(pos, p, tg, nthreads=4, lists=True, perm=True)
    assert np.array_equal(r["acc"], acc[tg])
    assert np.array_equal(r["perm"], full["perm"])
    for k, v in full["counters"].items():
        assert r["counters"][k] == v, k
    for kind in full["lists"]:
        assert all(np.array_equal(x, y) for x, y in zip(full["lists"][kind], r["lists"][kind])), kind
    # the reference's pair set: n_t n_s per task less a leaf's self pairs, plus image pairs
    tr = full["tree"]
    first = full["counters"]["first_leaf"]
    t, s, _ = full["lists"]["p2p"]
    nt, ns = tr["leaf_npart"][t - first].astype(np.int64), tr["leaf_npart"][s - first].astype(np.int64)
    assert r["counters"]["pairs_local"] == int(np.where(t == s, nt * (nt - 1), nt * ns).sum())
    assert r["counters"]["pairs_image"] == full["counters"]["p2p_count_remote"]
    tg2 = rng.choice(n, 200, replace=False).astype(np.int32)
    a2, secs = port.forces_sample(tg2)
    assert np.array_equal(a2, acc[tg2]) and secs >= 0
    a3, _ = port.forces_sample(tg)
    assert np.array_equal(a3, acc[tg])


def test_port_domain_split_follows_the_reference_rules(port):
    """src/domains.c:400-425 with equal times and src/toptree.c:157-182:
    two ranks split x at the middle, three put two domains left of 2/3 L
    (split again in y), four split x then y; every domain's first axis is
    the next after its parent's."""
    box, axis, split = port.domains(2, 100.0)
    assert np.allclose(box[0], [[0, 0, 0], [50, 100, 100]]) and np.allclose(box[1], [[50, 0, 0], [100, 100, 100]])
    assert list(axis) == [1, 1] and np.allclose(split, [50])
    box, axis, split = port.domains(3, 90.0)
    assert np.allclose(split, [60, 45])
    assert sorted(map(tuple, box[:, 1].round(9).tolist())) == [(60, 45, 90), (60, 90, 90), (90, 90, 90)]
    box, axis, split = port.domains(4, 100.0)
    assert list(axis) == [2, 2, 2, 2] and np.allclose(split, [50, 50, 50])


@pytest.mark.parametrize("name,nside,maxleaf", [("grid32", 20, 16), ("nfw128", 24, 8)])
def test_port_received_trees_reproduce_the_image_walk(port, ics, name, nside, maxleaf):
    """The restatement of the exported tree (src/remotes.c:60-169) and of
    the walk against a received tree (:213-552): at one rank, sending the
    26 periodic images through export + received walk gives the pinned
    single-rank pass bit for bit; at several ranks both routes for a rank's
    own images give the same counters and forces to rounding."""
    pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
    full = port.run(pos, p, capture=False, tree=False, nthreads=4)
    plain = np.empty_like(full["acc"])
    plain[full["perm"]] = full["acc"]
    acc, cnt, rank = port.run_domains(pos, p, 1, nthreads=4, explicit_self=True)
    assert np.array_equal(acc, plain) and (rank == 0).all()
    for k in COUNTERS[:4] + ["n_p2p_ext", "n_m2l_ext", "nleaf", "nnode"]:
        assert cnt[0][k] == full["counters"][k], k
    for P in (2, 3):
        a, c, r = port.run_domains(pos, p, P, nthreads=4)
        b, d, _ = port.run_domains(pos, p, P, nthreads=4, explicit_self=True)
        assert np.bincount(r).size == P and c == d
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_port_plain_pass_after_a_domain_prepare(port, ics):
    """A state that prepared one rank's domain runs the next plain pass over
    the whole box again."""
    pos, p = ics.make("grid32", nside=16)
    want = port.run(pos, p, capture=False, tree=False, nthreads=2)["counters"]
    port.prepare_domain(pos[pos[:, 0] < 0.5 * p["boxsize"]], p, [0, 0, 0], [0.5 * p["boxsize"], p["boxsize"],
                                                                           p["boxsize"]], 1)
    got = port.run(pos, p, capture=False, tree=False, nthreads=2)["counters"]
    assert got == want
