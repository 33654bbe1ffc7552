"""Several ranks, one GPU each, over torch.distributed: the transport of the
reference's multi-rank pass (src/domains.c:263-383 moves the particles to
their domains, src/remotes.c:684-751 moves the exported trees).

The library builds and uses the messages (photons_domain_*, photons_let_*);
this module moves them between ranks with point-to-point sends on the
process group the caller set up (gloo: host tensors; NCCL: the bytes are
staged through the rank's own GPU).  Every exchange pairs a send to
rank + i with a receive from rank - i, as fmm_remote's srank / rrank do,
so no rank waits on a message that is not on its way.
"""
from __future__ import annotations

import numpy as np


def _device(dist):
    import torch

    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def _send_recv(dist, payload: bytes, to: int, frm: int) -> bytes:
    """Send `payload` to rank `to` and receive the bytes rank `frm` sends."""
    import torch

    dev = _device(dist)
    n_out = torch.tensor([len(payload)], dtype=torch.int64, device=dev)
    n_in = torch.zeros(1, dtype=torch.int64, device=dev)
    req = dist.isend(n_out, to)
    dist.recv(n_in, frm)
    req.wait()
    out = torch.frombuffer(bytearray(payload), dtype=torch.uint8).to(dev) if payload else \
        torch.zeros(0, dtype=torch.uint8, device=dev)
    inn = torch.empty(int(n_in.item()), dtype=torch.uint8, device=dev)
    req = dist.isend(out, to) if out.numel() else None
    if inn.numel():
        dist.recv(inn, frm)
    if req is not None:
        req.wait()
    return inn.cpu().numpy().tobytes()


def migrate(dist, pos, split, nrank, rank, assign):
    """src/domains.c:263-383: every rank sends each of its particles to the
    rank whose domain holds it.  pos (n, 3) float64 on this rank; assign(
    nrank, split, pos) -> ranks.  Returns this rank's particles, ordered by
    sending rank (its own first, then rank - 1, rank - 2, ...)."""
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    dest = assign(nrank, split, pos)
    mine = [pos[dest == rank]]
    for i in range(1, nrank):
        to, frm = (rank + i) % nrank, (rank - i) % nrank
        got = _send_recv(dist, np.ascontiguousarray(pos[dest == to]).tobytes(), to, frm)
        mine.append(np.frombuffer(got, np.float64).reshape(-1, 3))
    return np.concatenate(mine)


def exchange_trees(dist, rank, nrank, domains, boxsize, export, import_, schedule, node_dtype, body_dtype):
    """src/fmm.c:1020-1045 / src/remotes.c:684-751: for each step of
    `schedule(rank, nrank)` -> (send_to, recv_from, shift unit), send this
    rank's tree exported for send_to's domain (shifted by unit * boxsize)
    and import the tree recv_from sends.  export(domain, shift) -> (nodes,
    bodies) arrays of the structured node_dtype / body_dtype;
    import_(nodes, bodies).
    Returns the bytes sent."""
    sent = 0
    for to, frm, unit in schedule(rank, nrank):
        nodes, bodies = export(domains[to], np.asarray(unit, np.float64) * boxsize)
        head = np.array([nodes.size, bodies.shape[0]], np.int64).tobytes()
        msg = head + np.ascontiguousarray(nodes).tobytes() + np.ascontiguousarray(bodies).tobytes()
        sent += len(msg)
        got = _send_recv(dist, msg, to, frm)
        nn, nb = np.frombuffer(got[:16], np.int64)
        off = 16 + int(nn) * node_dtype.itemsize
        bodies_in = np.frombuffer(got[off:], body_dtype)
        assert bodies_in.size == int(nb)
        import_(np.frombuffer(got[16:off], node_dtype), bodies_in)
    return sent


class DomainPass:
    """This rank's share of a force pass over several ranks (one GPU each):
    its particles' tree over its domain, the exchange of the locally
    essential trees, and the forces from its own, periodic and received
    trees.  fp: a ForcePass on this rank's GPU; dist: an initialised
    torch.distributed (NCCL or gloo)."""

    def __init__(self, ph, fp, dist):
        self.ph, self.fp, self.dist = ph, fp, dist
        self.rank, self.nrank = dist.get_rank(), dist.get_world_size()

    def run(self, pos_local, p, domains, precision=None):
        """pos_local: this rank's particles (all inside its domain).
        Returns their accelerations (n, 3) in the same order."""
        ph = self.ph
        precision = ph.FP32_SPLIT if precision is None else precision
        self.fp.domain_prepare(pos_local, p, domains[self.rank], precision=precision)
        exchange_trees(self.dist, self.rank, self.nrank, domains, p["boxsize"], self.fp.let_export,
                       self.fp.let_import, ph.let_schedule, ph.REMOTE_NODE, ph.REMOTE_BODY)
        return self.fp.domain_finish()
