"""Generate the golden fixtures in tests/golden/ by running the reference's
own FMM sources (compiled in place into oracle/_ref/libphotons_ref.so by
oracle/Makefile, with the one-rank MPI stand-in) on small seeded inputs.

    make -C oracle ref && python tests/golden/make_golden.py [names]

Each fixture holds the input positions and force parameters, and the
reference's outputs: the tree-ordered positions (its in-place permutation),
the accelerations after fmm_task and after fmm_ext, the counters, the tree
and a digest of every interaction list (full lists for the small cases).
time/ holds the reference's kick and drift factors; pm/ the reference's PM
accelerations (src/partmesh.c, with the Fortran convolution of
src/conv.f90 replaced by oracle/pm_conv.c, which needs no 2DECOMP&FFT).
"""
from __future__ import annotations

import hashlib
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

spec = importlib.util.spec_from_file_location("ics", os.path.join(ROOT, "photons-2.0_gb300", "ics.py"))
ics = importlib.util.module_from_spec(spec)
spec.loader.exec_module(ics)


def list_digest(t, s, im):
    key = (t.astype(np.int64) << 34) | (s.astype(np.int64) << 5) | im.astype(np.int64)
    key.sort()
    return hashlib.sha256(key.tobytes()).hexdigest()


def cases():
    out = []
    pos, p = ics.make("grid32", nside=16)
    out.append(("grid16_leaf16", pos, p, True))
    pos, p = ics.make("nfw128", nside=16)
    p["maxleaf"] = 8
    out.append(("nfw16_leaf8", pos, p, False))
    pos, p = ics.make("grid32", nside=12)
    p["maxleaf"] = 4
    out.append(("grid12_leaf4", pos, p, False))
    # Exact lattice: many coordinates equal a node's mean.  The cutoff is
    # kept small against the box because the reference sizes its image
    # export buffer as 1.1*NNODE entries (src/fmm.c:1004-1011) while the
    # export holds nodes and leaves; a box mostly within rcut of its faces
    # overflows that buffer in the reference itself.
    n = 12
    L = 12.0
    g = (np.arange(n) + 0.5) * (L / n)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    p = ics.force_params(pos.shape[0], L, 24, theta=0.5, maxleaf=6)
    out.append(("lattice12_leaf6", pos, p, True))
    # one particle per leaf: pair splits at the midpoint
    rng = np.random.default_rng(11)
    pos = rng.random((300, 3)) * 20.0
    p = ics.force_params(300, 20.0, 40, theta=0.5, maxleaf=1)
    out.append(("random300_leaf1", pos, p, True))
    # the reference's demo initial conditions (z = 49 LCDM, 32^3 particles)
    # read by its own Gadget-2 reader, with its demo run's parameters
    # (demo/lcdm_g2.run: OPENANGLE 0.4, MaxPackage 8, NumMeshSide 32) and its
    # derived force parameters (src/initial.c:316-337)
    demo = os.path.join(oracle.REFROOT, "demo", "ic_lcdm.gdt2")
    if os.path.exists(demo):
        hd, pos, _ = oracle.RefOracle().gadget(demo)
        L = hd["boxsize"]
        rs = 1.25 * L / 32
        p = dict(boxsize=L, theta=0.4, rs=rs, rcut=4.5 * rs, eps=0.03 * L / pow(float(pos.shape[0]), 0.3333333),
                 mass=hd["mass"], maxleaf=8)
        out.append(("demo_lcdm_leaf8", pos, p, False))
    return out


def main(only=None):
    ref = oracle.RefOracle()
    for name, pos, p, full in cases():
        if only and name not in only:
            continue
        r = ref.run(pos, p, capture=True, tree=True)
        d = {
            "pos_in": pos, "pos_tree": r["pos"], "acc_task": r["acc_task"], "acc": r["acc"],
            "params": np.array([p["boxsize"], p["theta"], p["rs"], p["rcut"], p["eps"], p["mass"], p["maxleaf"]]),
            "counters": np.array([r["counters"][k] for k in oracle.COUNTER_NAMES], np.int64),
        }
        for k, v in r["tree"].items():
            if k.endswith("_M") or k.endswith("_L"):
                if full:
                    d["tree_" + k] = v
            else:
                d["tree_" + k] = v
        for kind, (t, s, im) in r["lists"].items():
            d["digest_" + kind] = np.array(list_digest(t, s, im))
            d["ntarget_" + kind] = np.bincount(t - t.min(), minlength=1).astype(np.int32) if t.size else np.zeros(0, np.int32)
            if full:
                d["list_" + kind] = np.stack([t, s, im]).astype(np.int32)
        if name.startswith("demo"):
            # positions are FP32 in the snapshot, so FP32 storage is exact;
            # the fmm_task-only accelerations are left out to keep it small
            d["pos_in"] = d["pos_in"].astype(np.float32)
            d["pos_tree"] = d["pos_tree"].astype(np.float32)
            assert np.array_equal(d["pos_in"].astype(np.float64), pos)
            del d["acc_task"]
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **d)
        c = r["counters"]
        print("%-18s N=%6d p2p=%8d m2l=%6d p2p_ext=%7d m2l_ext=%5d  %6.1f KB" % (
            name, pos.shape[0], c["idxP2P"], c["idxM2L"], c["n_p2p_ext"], c["n_m2l_ext"], os.path.getsize(path) / 1024))


def time_integrals():
    """The reference's kick_loga / drift_loga (src/initial.c:639-683) over a
    spread of steps and cosmologies -> time/loga_integrals.npz."""
    ref = oracle.RefOracle()
    rng = np.random.default_rng(21)
    rows = []
    for om in (0.3, 0.25, 1.0):
        ox = 1.0 - om
        for _ in range(8):
            a0 = float(np.exp(rng.uniform(np.log(0.01), np.log(0.9))))
            a1 = a0 * float(np.exp(rng.uniform(1e-3, 0.2)))
            la, lb = np.log(a0), np.log(a1)
            rows.append([om, ox, la, lb, ref.kick_loga(om, ox, la, lb), ref.drift_loga(om, ox, la, lb)])
    os.makedirs(os.path.join(HERE, "time"), exist_ok=True)
    path = os.path.join(HERE, "time", "loga_integrals.npz")
    np.savez_compressed(path, rows=np.array(rows))
    print("time/loga_integrals  %d rows" % len(rows))


def pm_cases():
    """(name, pos, boxsize, nside, rs, mass): a clump in a uniform box, and a
    perturbed grid on a mesh finer than its particle spacing."""
    rng = np.random.default_rng(3)
    L = 50.0
    pos = rng.random((1500, 3)) * L
    pos[:500] = (0.3 * L + rng.normal(scale=0.02 * L, size=(500, 3))) % L
    yield "pm_clump16", pos, L, 16, 1.25 * L / 16, 0.7
    g, p = ics.make("grid32", nside=12)
    yield "pm_grid12_mesh24", g, p["boxsize"], 24, 1.25 * p["boxsize"] / 24, p["mass"]


def pm_fixtures():
    """The reference's own PM (src/partmesh.c at one rank, the Fortran
    convolution replaced by oracle/pm_conv.c) -> pm/<name>.npz."""
    ref = oracle.RefOracle()
    os.makedirs(os.path.join(HERE, "pm"), exist_ok=True)
    for name, pos, L, N, rs, m in pm_cases():
        acc = ref.pm_force(pos, L, N, rs, m)
        path = os.path.join(HERE, "pm", name + ".npz")
        np.savez_compressed(path, pos=pos, acc_pm=acc, params=np.array([L, N, rs, m]))
        print("pm/%-16s N=%5d mesh %d  %6.1f KB" % (name, pos.shape[0], N, os.path.getsize(path) / 1024))


if __name__ == "__main__":
    # python make_golden.py [fixture names | time | pm]  (default: all)
    names = sys.argv[1:]
    main(names or None)
    if not names or "time" in names:
        time_integrals()
    if not names or "pm" in names:
        pm_fixtures()
