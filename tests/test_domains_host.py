"""The host side of the multi-rank pass against the reference's own
compiled src/domains.c and src/toptree.c (called through the same
globals, CPU only): the first decomposition's split planes and each rank's
first axis, the rank every particle goes to, and the load-balancing move
of the planes.  Skipped where the reference is not built here."""
import ctypes as C
import os

import numpy as np
import pytest

DOMAIN_NODE = np.dtype([("son", "i4", 2), ("time_node", "f8"), ("time_left", "f8"), ("time_right", "f8"),
                        ("split", "f8"), ("split_previous", "f8")], align=True)
BODY = np.dtype([("pos", "f8", 3), ("acc", "f8", 3), ("vel", "f8", 3), ("acc_pm", "f8", 3)])
SAVED = [(C.c_int, "PROC_SIZE"), (C.c_int, "PROC_RANK"), (C.c_int, "first_domain"), (C.c_int, "last_domain"),
         (C.c_int, "mostleft"), (C.c_int, "this_domain"), (C.c_double, "BOXSIZE"), (C.c_void_p, "domtree")]


@pytest.fixture(scope="module")
def ref(oracle_mod):
    if not oracle_mod.ref_available():
        pytest.skip("reference oracle not built here")
    lib = oracle_mod.RefOracle().lib
    saved = [(t, n, t.in_dll(lib, n).value) for t, n in SAVED]
    yield lib
    for t, n, v in saved:
        t.in_dll(lib, n).value = v


def _setup(lib, P, L):
    """src/initial.c:197-222 for rank 0 of P, and the box."""
    ml = 1
    while ml < 2 * P - 1:
        ml *= 2
    ml = 0 if P == 1 else ml // 2 - 1
    for name, v in (("PROC_SIZE", P), ("PROC_RANK", 0), ("first_domain", P - 1), ("last_domain", 2 * P - 2),
                    ("mostleft", ml), ("this_domain", ml if ml <= 2 * P - 2 else ml - P)):
        C.c_int.in_dll(lib, name).value = v
    C.c_double.in_dll(lib, "BOXSIZE").value = L
    return ml


def _domtree(lib, P):
    addr = C.c_void_p.in_dll(lib, "domtree").value
    buf = (C.c_char * (DOMAIN_NODE.itemsize * (2 * P - 1))).from_address(addr)
    return np.frombuffer(buf, DOMAIN_NODE)


@pytest.mark.parametrize("P", [1, 2, 3, 4, 5, 6, 8])
def test_split_planes_and_axes_match_reference(ph, ref, P):
    L = 150.0
    _setup(ref, P, L)
    ref.domain_initialize()
    tree = _domtree(ref, P)
    doms, split = ph.domain_split(P, L)
    assert np.array_equal(split, tree["split"][:P - 1])
    # each rank's box: the planes around its domain node; its first axis
    # is the depth of that node mod 3 (src/toptree.c:157-182)
    ml = C.c_int.in_dll(ref, "mostleft").value
    for r, d in enumerate(doms):
        dom = r + ml if r + ml <= 2 * P - 2 else r + ml - P
        depth = int(np.floor(np.log2(dom + 1)))
        assert d.axis == depth % 3
        lo, hi = np.zeros(3), np.full(3, L)
        node, path = dom, []
        while node > 0:
            parent = (node - 1) // 2
            path.append((parent, node == 2 * parent + 2))
            node = parent
        for k, (parent, upper) in enumerate(reversed(path)):
            ax = k % 3
            if upper:
                lo[ax] = split[parent]
            else:
                hi[ax] = split[parent]
        assert np.array_equal(list(d.lo), lo) and np.array_equal(list(d.hi), hi)


@pytest.mark.parametrize("P", [2, 3, 5])
def test_particle_ranks_match_reference(ph, ref, P):
    L = 100.0
    _setup(ref, P, L)
    ref.domain_initialize()
    rng = np.random.default_rng(P)
    pos = rng.random((4000, 3)) * L
    pos[:50, 0] = 0.5 * L  # on a plane: the lower side, as the reference's "> split" test
    _, split = ph.domain_split(P, L)
    ranks = ph.domain_assign(P, split, pos)
    body = np.zeros(pos.shape[0], BODY)
    body["pos"] = pos
    send = np.zeros(P, np.int32)
    ref.prepare_body_inOrderOf_domain.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    ref.prepare_body_inOrderOf_domain(0, body.ctypes.data, pos.shape[0], 0, send.ctypes.data)
    assert np.array_equal(np.bincount(ranks, minlength=P), send)
    # the reference orders the particles by its domain tree's traversal
    # (lower side first); each block is one rank's
    ml = C.c_int.in_dll(ref, "mostleft").value

    def leaves(i):
        return [i] if i >= P - 1 else leaves(2 * i + 1) + leaves(2 * i + 2)

    first = 0
    for dom in leaves(0):
        r = (dom - ml + P) % P
        blk = body["pos"][first:first + send[r]]
        assert (ph.domain_assign(P, split, blk) == r).all()
        first += send[r]


@pytest.mark.parametrize("P", [2, 3, 4, 6])
def test_rebalance_matches_reference(ph, ref, P):
    L = 80.0
    ml = _setup(ref, P, L)
    ref.domain_initialize()
    tree = _domtree(ref, P)
    rng = np.random.default_rng(10 + P)
    times = rng.uniform(0.5, 2.0, P)
    for r in range(P):
        dom = r + ml if r + ml <= 2 * P - 2 else r + ml - P
        tree["time_node"][dom] = times[r]
    ref.fill_time_domtree.argtypes = [C.c_int]
    ref.fill_time_domtree.restype = C.c_double
    ref.fill_time_domtree(0)
    _, split0 = ph.domain_split(P, L)
    bl = (C.c_double * 3)(0.0, 0.0, 0.0)
    br = (C.c_double * 3)(L, L, L)
    ref.determine_split_node.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
    ref.determine_split_node(0, P, 0, C.c_void_p.in_dll(ref, "domtree").value, bl, br)
    doms, split = ph.domain_rebalance(P, L, split0, times)
    assert np.allclose(split, tree["split"][:P - 1], rtol=1e-15, atol=0)
    assert not np.array_equal(split, split0)
