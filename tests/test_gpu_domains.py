"""Several ranks, one GPU each, emulated here as several contexts in one
process on one GPU (the exchange between them goes through the host, so
no kernel waits on another).  Against the oracle's restatement of the
reference's domain decomposition (src/domains.c, src/toptree.c) and
locally essential trees (src/remotes.c:60-751):

* the exported trees (RemoteNode/RemoteBody in depth-first preorder) equal
  the oracle's node for node: counts, children and bodies exact, geometry
  to the last bits of the split means (1e-13 of the box; the GPU mean is a
  parallel sum), multipoles to 1e-12 of the largest;
* each rank's counters (its local and received P2P/M2L tasks and pairs)
  equal the oracle's emulated multi-rank pass, and its FP64 accelerations
  match it to 1e-10 relative; the FP32 split pass stays within the
  split-precision bar of the FP64 one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUNTERS = ("nleaf", "nnode", "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "n_p2p_ext", "n_m2l_ext")


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def gpu_domain_pass(ph, pos, p, nrank, precision):
    """The ranks' passes with the messages moved on the host, in the order
    of ph.let_schedule (each rank's own images are walked on the fly)."""
    doms, split = ph.domain_split(nrank, p["boxsize"])
    rank = ph.domain_assign(nrank, split, pos)
    ctx = [ph.ForcePass(0) for _ in range(nrank)]
    for r in range(nrank):
        ctx[r].domain_prepare(pos[rank == r], p, doms[r], precision=precision)
    for r in range(nrank):
        for _, src, unit in ph.let_schedule(r, nrank):
            nodes, bodies = ctx[src].let_export(doms[r], np.array(unit, float) * p["boxsize"])
            ctx[r].let_import(nodes, bodies)
    acc = np.empty_like(pos)
    counters = []
    for r in range(nrank):
        acc[rank == r] = ctx[r].domain_finish()
        counters.append(ctx[r].counters())
        ctx[r].close()
    return acc, counters, rank


@pytest.mark.parametrize("name,nside,maxleaf", [("grid32", 20, 16), ("nfw128", 24, 8)])
def test_export_equals_oracle(ph, ics, port, name, nside, maxleaf):
    pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
    doms, split = ph.domain_split(3, p["boxsize"])
    rank = ph.domain_assign(3, split, pos)
    fp = ph.ForcePass(0)
    for src, dst, unit in ((0, 1, (0, 0, 0)), (1, 2, (1, 0, -1)), (2, 0, (0, -1, 0)), (1, 1, (0, 0, 1))):
        sub = pos[rank == src]
        d = doms[src]
        fp.domain_prepare(sub, p, d, precision=ph.FP64)
        port.prepare_domain(sub, p, list(d.lo), list(d.hi), d.axis)
        shift = np.array(unit, float) * p["boxsize"]
        gn, gb = fp.let_export(doms[dst], shift)
        on, ob = port.export(list(doms[dst].lo), list(doms[dst].hi), shift)
        assert gn.size == on.size and gb.size == ob.shape[0], (src, dst)
        for k in ("npart", "son"):
            assert np.array_equal(gn[k], on[k]), k
        for k in ("width", "center"):
            assert np.allclose(gn[k], on[k], rtol=1e-13, atol=1e-13 * p["boxsize"]), k
        assert np.array_equal(gb["pos"], ob)
        assert np.abs(gn["M"] - on["M"]).max() <= 1e-12 * np.abs(on["M"]).max()
    fp.close()


@pytest.mark.parametrize("name,nside,maxleaf,nrank", [("grid32", 24, 16, 2), ("nfw128", 32, 8, 3),
                                                      ("nfw128", 32, 8, 4), ("zeldovich256", 32, 64, 2)])
def test_domain_pass_matches_oracle(ph, ics, port, name, nside, maxleaf, nrank):
    pos, p = ics.make(name, nside=nside, maxleaf=maxleaf)
    ref, rc, rrank = port.run_domains(pos, p, nrank, nthreads=8)
    acc, counters, rank = gpu_domain_pass(ph, pos, p, nrank, ph.FP64)
    assert np.array_equal(rank, rrank)
    for r in range(nrank):
        for k in COUNTERS:
            assert counters[r][k] == rc[r][k], (r, k, counters[r][k], rc[r][k])
    assert rel_err(acc, ref).max() <= 1e-10
    acc32, _, _ = gpu_domain_pass(ph, pos, p, nrank, ph.FP32_SPLIT)
    e = rel_err(acc32, acc)
    assert np.median(e) <= 2e-6 and np.percentile(e, 99) <= 2e-5, (np.median(e), np.percentile(e, 99))


def test_one_rank_domain_pass_is_the_plain_pass(ph, ics):
    """At one rank the domain is the whole box and nothing is received: the
    domain pass gives the plain pass's accelerations and counters."""
    pos, p = ics.make("nfw128", nside=24, maxleaf=8)
    fp = ph.ForcePass(0)
    plain = fp.run(pos, p, precision=ph.FP64)
    c0 = fp.counters()
    doms, _ = ph.domain_split(1, p["boxsize"])
    fp.domain_prepare(pos, p, doms[0], precision=ph.FP64)
    acc = fp.domain_finish()
    c1 = fp.counters()
    assert np.abs(acc - plain).max() <= 1e-12 * np.abs(plain).max()
    for k in COUNTERS:
        assert c0[k] == c1[k], k
    fp.close()


class _ThreadGroup:
    """A process-group stand-in for ranks run as threads of one process:
    point-to-point sends through queues (the library's exchange is
    host-staged, so the ranks' kernels never wait on one another)."""

    def __init__(self, world):
        import queue
        self.world = world
        self.q = {(a, b): queue.Queue() for a in range(world) for b in range(world)}

    def rank_view(self, rank):
        group = self

        class View:
            def get_rank(self):
                return rank

            def get_world_size(self):
                return group.world

            def get_backend(self):
                return "gloo"

            def isend(self, t, dst):
                group.q[(rank, dst)].put(t.clone())

                class Done:
                    def wait(self):
                        return True
                return Done()

            def recv(self, t, src):
                t.copy_(group.q[(src, rank)].get(timeout=120))

        return View()


def test_domain_pass_class_over_ranks_as_threads(ph, ics, port):
    """photons_gb300.domains.DomainPass, the per-rank driver a
    torch.distributed job calls, with two ranks as threads sharing this GPU
    (a context each): the same forces as the oracle's multi-rank pass."""
    import threading
    from photons_gb300 import domains
    pos, p = ics.make("nfw128", nside=28, maxleaf=8)
    nrank = 2
    doms, split = ph.domain_split(nrank, p["boxsize"])
    rank = ph.domain_assign(nrank, split, pos)
    group = _ThreadGroup(nrank)
    out, errs = {}, []

    def run(r):
        try:
            fp = ph.ForcePass(0)
            out[r] = domains.DomainPass(ph, fp, group.rank_view(r)).run(pos[rank == r], p, doms, ph.FP64)
            fp.close()
        except Exception as e:  # reported below
            errs.append(e)

    threads = [threading.Thread(target=run, args=(r,)) for r in range(nrank)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errs, errs
    ref, _, rref = port.run_domains(pos, p, nrank, nthreads=4)
    acc = np.empty_like(pos)
    for r in range(nrank):
        acc[rank == r] = out[r]
    assert rel_err(acc, ref).max() <= 1e-10
