"""The library's host entry points of operator.h and photoNs.h:325 (p2m,
m2m, m2l, l2l, l2p, walk_m2m, walk_l2l, acceptance) against the
reference's own compiled src/operator.c and src/fmm.c, called side by side
through the same globals on the same data.  The reference's top-tree code
(src/toptree.c:185-244) calls these on host data, so they must agree with
it: acceptance exactly, the operators to 1e-13 of the largest component
(the library sums the same Cartesian expansions in multi-index order).
CPU only: no GPU call is made; skipped where the reference is not built."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden

NODE = np.dtype([("updated", "i4"), ("npart", "i4"), ("son", "i4", 2), ("split", "f8"), ("width", "f8", 3),
                 ("center", "f8", 3), ("M", "f8", 20), ("L", "f8", 20)], align=True)
PACK = np.dtype([("npart", "i4"), ("ipart", "i4"), ("width", "f8", 3), ("center", "f8", 3), ("M", "f8", 20),
                 ("L", "f8", 20)], align=True)
BODY = np.dtype([("pos", "f8", 3), ("acc", "f8", 3), ("vel", "f8", 3), ("acc_pm", "f8", 3)])
TOL = 1e-13
_dp = C.POINTER(C.c_double)


SAVED = [(C.c_void_p, "part"), (C.c_void_p, "btree"), (C.c_void_p, "leaf"), (C.c_int, "first_leaf"),
         (C.c_int, "first_node"), (C.c_int, "last_leaf"), (C.c_int, "last_node"), (C.c_double, "MASSPART"),
         (C.c_double, "splitRadius"), (C.c_double, "cutoffRadius"), (C.c_double, "open_angle")]


@pytest.fixture(scope="module")
def libs(ph, oracle_mod):
    """Both libraries, with the globals these tests point at their own
    arrays restored afterwards (the reference frees its tree through them)."""
    if not oracle_mod.ref_available():
        pytest.skip("reference oracle not built here")
    assert NODE.itemsize == 392 and PACK.itemsize == 376 and BODY.itemsize == 96
    ours = C.CDLL(ph.library_path(), mode=os.RTLD_LOCAL)
    ref = oracle_mod.RefOracle().lib
    saved = [[(t, n, t.in_dll(lib, n).value) for t, n in SAVED] for lib in (ours, ref)]
    for lib in (ours, ref):
        for name in ("m2m", "m2l", "l2l"):
            getattr(lib, name).argtypes = [C.c_double] * 3 + [_dp, _dp]
            getattr(lib, name).restype = None
        lib.p2m.argtypes = [C.c_int, C.c_int, _dp, _dp]
        lib.l2p.argtypes = [C.c_int]
        lib.walk_m2m.argtypes = [C.c_int]
        lib.walk_l2l.argtypes = [C.c_int]
        lib.acceptance.argtypes = [_dp, _dp, _dp]
        lib.acceptance.restype = C.c_int
    yield ours, ref
    for lib, vals in zip((ours, ref), saved):
        for t, n, v in vals:
            t.in_dll(lib, n).value = v


def _set(lib, ctype, name, v):
    ctype.in_dll(lib, name).value = v


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _close(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= TOL * scale


def test_multipole_operators_match_reference(libs):
    rng = np.random.default_rng(21)
    for rs in (0.7, 2.44):
        for lib in libs:
            _set(lib, C.c_double, "splitRadius", rs)
        for _ in range(60):
            d = rng.normal(size=3) * rng.uniform(0.5, 8.0)
            src = rng.normal(size=20)
            base = rng.normal(size=20)
            for name in ("m2m", "m2l", "l2l"):
                outs = []
                for lib in libs:
                    out = base.copy()
                    getattr(lib, name)(d[0], d[1], d[2], _ptr(src), _ptr(out))
                    outs.append(out)
                assert _close(outs[0], outs[1]), name


def test_acceptance_matches_reference_exactly(libs):
    rng = np.random.default_rng(8)
    for theta, rcut in ((0.5, 10.0), (0.3, 4.0), (0.8, 17.5)):
        for lib in libs:
            _set(lib, C.c_double, "open_angle", theta)
            _set(lib, C.c_double, "cutoffRadius", rcut)
        for k in range(4000):
            wi, wj = rng.uniform(0.1, 6.0, 3), rng.uniform(0.1, 6.0, 3)
            if k % 5 == 0:  # touching and aligned boxes
                dist = (wi + wj) * 0.5 * rng.choice([-1.0, 0.0, 1.0], 3)
            else:
                dist = rng.normal(size=3) * rcut
            got = [lib.acceptance(_ptr(wi), _ptr(wj), _ptr(dist)) for lib in libs]
            assert got[0] == got[1], (wi, wj, dist, got)


def _install_tree(lib, g, body, nodes, leaves):
    """The golden tree into lib's globals, indexed by reference ids as
    src/fmm.c:259-260 sets them up (btree -= first_node, leaf -= first_leaf)."""
    c = dict(zip(["idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "NLEAF", "NNODE", "nleaf", "nnode",
                  "first_leaf", "first_node"], g["counters"][:10]))
    fl, fn = int(c["first_leaf"]), int(c["first_node"])
    _set(lib, C.c_int, "first_leaf", fl)
    _set(lib, C.c_int, "first_node", fn)
    _set(lib, C.c_int, "last_leaf", fl + int(c["nleaf"]))
    _set(lib, C.c_int, "last_node", fn + int(c["nnode"]) - 1)
    _set(lib, C.c_double, "MASSPART", float(g["p"]["mass"]))
    C.c_void_p.in_dll(lib, "part").value = body.ctypes.data
    C.c_void_p.in_dll(lib, "btree").value = nodes.ctypes.data - fn * NODE.itemsize
    C.c_void_p.in_dll(lib, "leaf").value = leaves.ctypes.data - fl * PACK.itemsize
    return fl, fn


def _golden_tree(g):
    nl, nn = len(g["tree_leaf_ipart"]), len(g["tree_node_npart"])
    leaves = np.zeros(nl, PACK)
    leaves["npart"], leaves["ipart"] = g["tree_leaf_npart"], g["tree_leaf_ipart"]
    leaves["center"], leaves["width"] = g["tree_leaf_center"], g["tree_leaf_width"]
    nodes = np.zeros(nn, NODE)
    nodes["npart"], nodes["son"] = g["tree_node_npart"], g["tree_node_son"]
    nodes["split"], nodes["center"], nodes["width"] = g["tree_node_split"], g["tree_node_center"], g["tree_node_width"]
    body = np.zeros(len(g["pos_tree"]), BODY)
    body["pos"] = g["pos_tree"]
    return body, nodes, leaves


@pytest.mark.parametrize("name", ["nfw16_leaf8", "grid12_leaf4", "grid16_leaf16"])
def test_tree_operators_match_reference_on_golden_trees(libs, name):
    """p2m of every leaf, walk_m2m from the root, walk_l2l from the root
    with random local expansions, and l2p of every leaf, on the
    reference's own tree for the golden input."""
    g = load_golden(name)
    rng = np.random.default_rng(4)
    results = []
    L_root = rng.normal(size=20)
    L_leaf = rng.normal(size=(len(g["tree_leaf_ipart"]), 20)) * 1e-3
    for lib in libs:
        body, nodes, leaves = _golden_tree(g)
        fl, fn = _install_tree(lib, g, body, nodes, leaves)
        for i in range(len(leaves)):
            M = np.zeros(20)
            lib.p2m(int(leaves["ipart"][i]), int(leaves["npart"][i]), _ptr(np.ascontiguousarray(leaves["center"][i])),
                    _ptr(M))
            leaves["M"][i] = M
        lib.walk_m2m(fn)
        nodes["L"][0] = L_root
        leaves["L"] = L_leaf
        lib.walk_l2l(fn)
        for i in range(len(leaves)):
            lib.l2p(fl + i)
        results.append((leaves["M"].copy(), nodes["M"].copy(), leaves["L"].copy(), nodes["L"].copy(),
                        body["acc"].copy()))
    for k, what in enumerate(("leaf M (p2m)", "node M (walk_m2m)", "leaf L (walk_l2l)", "node L (walk_l2l)",
                              "acc (l2p)")):
        assert _close(results[0][k], results[1][k]), what
    # and the multipoles are the reference pass's own where the fixture keeps them
    if "tree_leaf_M" in g:
        assert _close(results[0][0], g["tree_leaf_M"]) and _close(results[0][1], g["tree_node_M"])
