"""The multi-rank transport (photons_gb300/domains.py) across two and three
gloo ranks on CPU (127.0.0.1): particles move to their domains, and each
rank sends and receives the exported trees in fmm_ext's order.  The
exported trees and the walks on the received ones are the oracle's here
(no GPU), so each rank's counters must equal the oracle's multi-rank
pass emulated in one process and its forces agree with it to rounding
(the particles arrive in another order, so the sums within a leaf run in
another order), and its particles must be exactly those the
decomposition assigns to it."""
import json
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out, name, nside, maxleaf):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import __graft_entry__ as g
    import oracle

    ph = g.load_package()
    from photons_gb300 import domains, ics

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
        doms, split = ph.domain_split(world, p["boxsize"])
        # every rank starts with an arbitrary slab of the input
        slab = np.array_split(np.arange(pos.shape[0]), world)[rank]
        mine = domains.migrate(dist, pos[slab], split, world, rank, ph.domain_assign)
        port = oracle.PortOracle(build=False)
        d = doms[rank]
        port.prepare_domain(mine, p, list(d.lo), list(d.hi), d.axis)
        node_dt = np.dtype([("npart", "i4"), ("son", "i4", 2), ("width", "f8", 3), ("center", "f8", 3),
                            ("M", "f8", 20)], align=True)

        body_dt = np.dtype([("pos", "f8", 3)])

        def export(dom, shift):
            nodes, bodies = port.export(list(dom.lo), list(dom.hi), shift)
            return nodes, np.ascontiguousarray(bodies).view(body_dt).reshape(-1)

        sent = domains.exchange_trees(dist, rank, world, doms, p["boxsize"], export,
                                      lambda nodes, bodies: port.import_tree(nodes, bodies["pos"]), ph.let_schedule,
                                      node_dt, body_dt)
        acc, cnt = port.finish_domain(mine.shape[0])
        np.save(os.path.join(out, "pos%d.npy" % rank), mine)
        np.save(os.path.join(out, "acc%d.npy" % rank), acc)
        with open(os.path.join(out, "rank%d.json" % rank), "w") as f:
            json.dump({"counters": cnt, "sent": sent}, f)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,name,nside,maxleaf", [(2, "grid32", 16, 16), (3, "nfw128", 20, 8)])
def test_domain_exchange_gloo(tmp_path, port, ics, world, name, nside, maxleaf):
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path), name, nside, maxleaf), nprocs=world,
                       join=True, start_method="spawn")
    pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
    ref, rc, rank = port.run_domains(pos, p, world, nthreads=2)
    for r in range(world):
        mine = np.load(tmp_path / ("pos%d.npy" % r))
        acc = np.load(tmp_path / ("acc%d.npy" % r))
        info = json.load(open(tmp_path / ("rank%d.json" % r)))
        # exactly this rank's particles (as a set), forces equal to the emulation's
        want = pos[rank == r]
        order_m = np.lexsort(mine.T[::-1])
        order_w = np.lexsort(want.T[::-1])
        assert np.array_equal(mine[order_m], want[order_w])
        got, exp = acc[order_m], ref[rank == r][order_w]
        assert (np.linalg.norm(got - exp, axis=1) / np.linalg.norm(exp, axis=1)).max() <= 1e-12
        for k in ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "n_p2p_ext", "n_m2l_ext", "nleaf"):
            assert info["counters"][k] == rc[r][k], (r, k)
        assert info["sent"] > 0
