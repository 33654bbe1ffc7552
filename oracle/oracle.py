"""ctypes access to the two CPU oracles.  TEST INFRASTRUCTURE ONLY.

* ``RefOracle``  -- the reference photoNs-2.0 FMM sources compiled in place
  (oracle/_ref/libphotons_ref.so, see oracle/Makefile and ref_harness.c).
  Exists only where the reference tree is present.
* ``PortOracle`` -- this project's own C restatement of the same pass
  (oracle/photons_oracle.c -> oracle/_build/libphotons_oracle.so).  It is
  pinned against ``RefOracle`` and the committed golden fixtures, and it is
  the CPU baseline on machines without the reference.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libphotons_ref.so")
REFROOT = os.environ.get("PHOTONS_REFERENCE", "/root/reference")  # the reference tree, where present
PORT_SO = os.path.join(HERE, "_build", "libphotons_oracle.so")

NMULTI = 20
LIST_KINDS = {"p2p": 0, "m2l": 1, "p2p_ext": 2, "m2l_ext": 3}
COUNTER_NAMES = [
    "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "NLEAF", "NNODE",
    "nleaf", "nnode", "first_leaf", "first_node", "direct_local_start",
    "n_p2p", "n_m2l", "n_p2p_ext", "n_m2l_ext", "n_images",
]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_longlong)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def build_ref():
    subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def ref_available():
    return os.path.exists(REF_SO)


class PassResult(dict):
    """pos (tree order), acc_task (after the local task phase), acc, counters, lists."""


class _Base:
    def _lists(self, lib, prefix):
        out = {}
        for name, k in LIST_KINDS.items():
            n = getattr(lib, prefix + "list_size")(k)
            t = np.empty(n, np.int32)
            s = np.empty(n, np.int32)
            im = np.empty(n, np.int32)
            if n:
                getattr(lib, prefix + "list_copy")(k, _ptr(t, _ip), _ptr(s, _ip), _ptr(im, _ip))
            out[name] = (t, s, im)
        return out

    def _tree(self, lib, prefix, counters):
        nl, nn = int(counters["nleaf"]), int(counters["nnode"])
        lip = np.empty((nl, 2), np.int32)
        lgeom = np.empty((nl, 6), np.float64)
        lM = np.empty((nl, NMULTI), np.float64)
        lL = np.empty((nl, NMULTI), np.float64)
        ninfo = np.empty((nn, 3), np.int32)
        ngeom = np.empty((nn, 7), np.float64)
        nM = np.empty((nn, NMULTI), np.float64)
        nL = np.empty((nn, NMULTI), np.float64)
        getattr(lib, prefix + "copy_leaves")(_ptr(lip, _ip), _ptr(lgeom), _ptr(lM), _ptr(lL))
        getattr(lib, prefix + "copy_nodes")(_ptr(ninfo, _ip), _ptr(ngeom), _ptr(nM), _ptr(nL))
        return dict(leaf_ipart=lip[:, 0].copy(), leaf_npart=lip[:, 1].copy(),
                    leaf_center=lgeom[:, :3].copy(), leaf_width=lgeom[:, 3:].copy(),
                    leaf_M=lM, leaf_L=lL,
                    node_npart=ninfo[:, 0].copy(), node_son=ninfo[:, 1:].copy(),
                    node_split=ngeom[:, 0].copy(), node_center=ngeom[:, 1:4].copy(),
                    node_width=ngeom[:, 4:].copy(), node_M=nM, node_L=nL)


class RefOracle(_Base):
    def __init__(self):
        if not ref_available():
            raise FileNotFoundError(REF_SO)
        # The GPU library defines the same FMM entry points and globals; bind
        # the reference's calls to its own definitions whatever was loaded first.
        lib = C.CDLL(REF_SO, mode=os.RTLD_LOCAL | getattr(os, "RTLD_DEEPBIND", 0))
        lib.ref_run.restype = C.c_double
        lib.ref_run.argtypes = [C.c_int, _dp, C.c_double, C.c_int, C.c_double, C.c_double,
                                C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _lp]
        lib.ref_list_size.restype = C.c_long
        lib.ref_list_size.argtypes = [C.c_int]
        lib.ref_list_copy.argtypes = [C.c_int, _ip, _ip, _ip]
        lib.ref_copy_leaves.argtypes = [_ip, _dp, _dp, _dp]
        lib.ref_copy_nodes.argtypes = [_ip, _dp, _dp, _dp]
        lib.ref_m2l.argtypes = [C.c_double] * 3 + [_dp, _dp, C.c_double]
        lib.ref_m2m.argtypes = [C.c_double] * 3 + [_dp, _dp]
        lib.ref_l2l.argtypes = [C.c_double] * 3 + [_dp, _dp]
        lib.ref_acceptance.restype = C.c_int
        lib.ref_acceptance.argtypes = [_dp, _dp, _dp, C.c_double, C.c_double]
        for name in ("ref_kick_loga", "ref_drift_loga"):
            getattr(lib, name).restype = C.c_double
            getattr(lib, name).argtypes = [C.c_double] * 4
        self.lib = lib

    def gadget(self, path):
        """(header values, pos, vel) read by the reference's own Gadget-2 readers."""
        lib = self.lib
        lib.ref_gadget_header.argtypes = [C.c_char_p, _dp]
        lib.ref_gadget_read.argtypes = [C.c_char_p, C.c_int, _dp, _dp]
        h = np.zeros(7)
        lib.ref_gadget_header(path.encode(), _ptr(h))
        n = int(h[1])
        pos = np.empty((n, 3))
        vel = np.empty((n, 3))
        lib.ref_gadget_read(path.encode(), n, _ptr(pos), _ptr(vel))
        keys = ("boxsize", "npart_total", "mass", "omega0", "omega_lambda", "hubble", "redshift")
        return dict(zip(keys, h.tolist())), pos, vel

    def pm_force(self, pos, boxsize, nside, rs, mass):
        """acc_pm (n, 3) of the reference's own PM (src/partmesh.c, one rank),
        with the Fortran convolution replaced by oracle/pm_conv.c."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        out = np.empty_like(pos)
        self.lib.ref_pm_force.argtypes = [C.c_int, _dp, C.c_double, C.c_int, C.c_double, C.c_double, _dp]
        self.lib.ref_pm_force(pos.shape[0], _ptr(pos), float(boxsize), int(nside), float(rs), float(mass), _ptr(out))
        return out

    def kick_loga(self, om, ox, la, lb):
        return self.lib.ref_kick_loga(om, ox, la, lb)

    def drift_loga(self, om, ox, la, lb):
        return self.lib.ref_drift_loga(om, ox, la, lb)

    def run(self, pos, p, capture=True, tree=True):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        pos_out = np.empty_like(pos)
        acc_task = np.empty_like(pos)
        acc = np.empty_like(pos)
        cnt = np.zeros(16, np.int64)
        secs = self.lib.ref_run(n, _ptr(pos), p["boxsize"], p["maxleaf"], p["theta"], p["rs"],
                                p["rcut"], p["eps"], p["mass"], int(capture), _ptr(pos_out),
                                _ptr(acc_task), _ptr(acc), _ptr(cnt, _lp))
        counters = dict(zip(COUNTER_NAMES, (int(c) for c in cnt)))
        r = PassResult(pos=pos_out, acc_task=acc_task, acc=acc, counters=counters, seconds=secs)
        if capture:
            r["lists"] = self._lists(self.lib, "ref_")
        if tree:
            r["tree"] = self._tree(self.lib, "ref_", counters)
        return r

    def m2l(self, d, M, rs):
        L = np.zeros(NMULTI)
        M = np.ascontiguousarray(M, np.float64)
        self.lib.ref_m2l(d[0], d[1], d[2], _ptr(M), _ptr(L), rs)
        return L

    def m2m(self, d, M):
        out = np.zeros(NMULTI)
        M = np.ascontiguousarray(M, np.float64)
        self.lib.ref_m2m(d[0], d[1], d[2], _ptr(M), _ptr(out))
        return out

    def l2l(self, d, L):
        out = np.zeros(NMULTI)
        L = np.ascontiguousarray(L, np.float64)
        self.lib.ref_l2l(d[0], d[1], d[2], _ptr(L), _ptr(out))
        return out

    def acceptance(self, wi, wj, dist, theta, rcut):
        a = [np.ascontiguousarray(x, np.float64) for x in (wi, wj, dist)]
        return self.lib.ref_acceptance(_ptr(a[0]), _ptr(a[1]), _ptr(a[2]), theta, rcut)


class PortOracle(_Base):
    """This project's C restatement (oracle/photons_oracle.c)."""

    def __init__(self, build=True):
        if build and not os.path.exists(PORT_SO):
            build_port()
        lib = C.CDLL(PORT_SO)
        lib.po_create.restype = C.c_void_p
        lib.po_destroy.argtypes = [C.c_void_p]
        lib.po_run.restype = C.c_int
        lib.po_run.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _dp, _dp]
        lib.po_counters.argtypes = [C.c_void_p, _lp]
        lib.po_particles.argtypes = [C.c_void_p, _dp, _dp, _dp, _ip]
        lib.po_run_sample.restype = C.c_int
        lib.po_run_sample.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _dp, C.c_int, _ip, _dp, _dp]
        lib.po_pairs.argtypes = [C.c_void_p, _lp, _lp]
        lib.po_run_domains.restype = C.c_int
        lib.po_run_domains.argtypes = [C.c_int, C.c_void_p, C.c_int, _dp, C.c_int, _dp, _lp, _ip]
        lib.po_domains.restype = C.c_int
        lib.po_domains.argtypes = [C.c_int, C.c_double, _dp, _ip, _dp]
        lib.po_prepare_domain.restype = C.c_int
        lib.po_prepare_domain.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, C.c_int, C.c_int, _dp]
        lib.po_export.restype = C.c_int
        lib.po_export.argtypes = [C.c_void_p, _dp, _dp, _dp, _ip, _ip, C.c_int, C.c_int, C.c_void_p, _dp]
        lib.po_import.restype = C.c_int
        lib.po_import.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, _dp]
        lib.po_finish_domain.restype = C.c_int
        lib.po_finish_domain.argtypes = [C.c_void_p, _dp]
        lib.po_forces_sample.restype = C.c_int
        lib.po_forces_sample.argtypes = [C.c_void_p, C.c_int, _ip, _dp, _dp]
        lib.po_list_size.restype = C.c_long
        lib.po_list_size.argtypes = [C.c_void_p, C.c_int]
        lib.po_list_copy.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip]
        lib.po_copy_leaves.argtypes = [C.c_void_p, _ip, _dp, _dp, _dp]
        lib.po_copy_nodes.argtypes = [C.c_void_p, _ip, _dp, _dp, _dp]
        lib.po_m2l.argtypes = [C.c_double] * 3 + [_dp, _dp, C.c_double]
        lib.po_m2m.argtypes = [C.c_double] * 3 + [_dp, _dp]
        lib.po_l2l.argtypes = [C.c_double] * 3 + [_dp, _dp]
        lib.po_p2m.argtypes = [C.c_int, _dp, C.c_double, _dp, _dp]
        lib.po_l2p.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        lib.po_acceptance.restype = C.c_int
        lib.po_acceptance.argtypes = [_dp, _dp, _dp, C.c_double, C.c_double]
        lib.po_direct_sum.restype = C.c_int
        lib.po_direct_sum.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, C.c_double, _dp]
        for name in ("po_kick_loga", "po_drift_loga"):
            getattr(lib, name).restype = C.c_double
            getattr(lib, name).argtypes = [C.c_double] * 4
        lib.po_kick.argtypes = [C.c_longlong, _dp, _dp, C.c_double]
        lib.po_drift.argtypes = [C.c_longlong, _dp, _dp, C.c_double, C.c_double]
        self.lib = lib
        self.state = C.c_void_p(lib.po_create())

    def __del__(self):
        try:
            self.lib.po_destroy(self.state)
        except Exception:
            pass

    @staticmethod
    def _params(p, nthreads=1, capture=True, images=True):
        class P(C.Structure):
            _fields_ = [("boxsize", C.c_double), ("theta", C.c_double), ("rs", C.c_double),
                        ("rcut", C.c_double), ("eps", C.c_double), ("mass", C.c_double),
                        ("maxleaf", C.c_int), ("nthreads", C.c_int), ("capture", C.c_int),
                        ("images", C.c_int)]
        return P(p["boxsize"], p["theta"], p["rs"], p["rcut"], p["eps"], p["mass"],
                 int(p["maxleaf"]), int(nthreads), int(capture), int(images))

    def run(self, pos, p, capture=True, tree=True, nthreads=1, images=True):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        prm = self._params(p, nthreads, capture, images)
        secs = C.c_double(0.0)
        rc = self.lib.po_run(self.state, C.byref(prm), n, _ptr(pos), C.byref(secs))
        if rc != 0:
            raise RuntimeError(f"oracle pass failed with code {rc}")
        cnt = np.zeros(16, np.int64)
        self.lib.po_counters(self.state, _ptr(cnt, _lp))
        counters = dict(zip(COUNTER_NAMES, (int(c) for c in cnt)))
        pos_out = np.empty_like(pos)
        acc_task = np.empty_like(pos)
        acc = np.empty_like(pos)
        perm = np.empty(n, np.int32)
        self.lib.po_particles(self.state, _ptr(pos_out), _ptr(acc_task), _ptr(acc), _ptr(perm, _ip))
        r = PassResult(pos=pos_out, acc_task=acc_task, acc=acc, perm=perm, counters=counters,
                       seconds=secs.value)
        if capture:
            out = {}
            for name, k in LIST_KINDS.items():
                m = self.lib.po_list_size(self.state, k)
                t = np.empty(m, np.int32); s = np.empty(m, np.int32); im = np.empty(m, np.int32)
                if m:
                    self.lib.po_list_copy(self.state, k, _ptr(t, _ip), _ptr(s, _ip), _ptr(im, _ip))
                out[name] = (t, s, im)
            r["lists"] = out
        if tree:
            r["tree"] = self._tree_port(counters)
        return r

    def run_sample(self, pos, p, targets, nthreads=1, images=True, lists=False, perm=False):
        """The pass with forces only for ``targets`` (input indices): complete
        tree, walks and counters; the targets' accelerations equal the full
        pass's.  Returns acc (len(targets), 3), counters (with pairs_local,
        pairs_image), times {tree, multipoles, walk, forces} in seconds and,
        on request, the lists (reference index space) and the permutation."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        targets = np.ascontiguousarray(targets, np.int32)
        n = pos.shape[0]
        prm = self._params(p, nthreads, True, images)
        acc = np.empty((targets.size, 3))
        t = np.zeros(4)
        rc = self.lib.po_run_sample(self.state, C.byref(prm), n, _ptr(pos), targets.size, _ptr(targets, _ip),
                                    _ptr(acc), _ptr(t))
        if rc != 0:
            raise RuntimeError(f"oracle sampled pass failed with code {rc}")
        cnt = np.zeros(16, np.int64)
        self.lib.po_counters(self.state, _ptr(cnt, _lp))
        counters = dict(zip(COUNTER_NAMES, (int(c) for c in cnt)))
        a, b = C.c_longlong(0), C.c_longlong(0)
        self.lib.po_pairs(self.state, C.byref(a), C.byref(b))
        counters["pairs_local"], counters["pairs_image"] = a.value, b.value
        r = PassResult(acc=acc, counters=counters,
                       times=dict(zip(("tree", "multipoles", "walk", "forces"), t.tolist())))
        if perm:
            pm = np.empty(n, np.int32)
            self.lib.po_particles(self.state, None, None, None, _ptr(pm, _ip))
            r["perm"] = pm
        if lists:
            out = {}
            for name, k in LIST_KINDS.items():
                m = self.lib.po_list_size(self.state, k)
                tt = np.empty(m, np.int32); ss = np.empty(m, np.int32); im = np.empty(m, np.int32)
                if m:
                    self.lib.po_list_copy(self.state, k, _ptr(tt, _ip), _ptr(ss, _ip), _ptr(im, _ip))
                out[name] = (tt, ss, im)
            r["lists"] = out
        return r

    def domains(self, nrank, boxsize):
        """The reference's first domain decomposition: (box (P, 2, 3) lo/hi,
        first split axis (P,), split planes (P-1,) in heap order)."""
        box = np.empty((nrank, 2, 3))
        axis = np.empty(nrank, np.int32)
        split = np.empty(max(nrank - 1, 1))
        rc = self.lib.po_domains(nrank, float(boxsize), _ptr(box), _ptr(axis, _ip), _ptr(split))
        if rc != 0:
            raise RuntimeError(f"oracle domains failed with code {rc}")
        return box, axis, split[:nrank - 1]

    def import_tree(self, nodes, bodies):
        """Keep a received tree (nodes as export returns them, bodies (n, 3))."""
        nodes = np.ascontiguousarray(nodes)
        bodies = np.ascontiguousarray(bodies, np.float64).reshape(-1, 3)
        rc = self.lib.po_import(self.state, nodes.size, nodes.ctypes.data, bodies.shape[0], _ptr(bodies))
        if rc != 0:
            raise RuntimeError(f"oracle import failed with code {rc}")

    def finish_domain(self, n):
        """The prepared domain's pass over the received trees: acc (n, 3)
        and the counters."""
        acc = np.empty((n, 3))
        rc = self.lib.po_finish_domain(self.state, _ptr(acc))
        if rc != 0:
            raise RuntimeError(f"oracle domain finish failed with code {rc}")
        cnt = np.zeros(16, np.int64)
        self.lib.po_counters(self.state, _ptr(cnt, _lp))
        return acc, dict(zip(COUNTER_NAMES, (int(c) for c in cnt)))

    def run_domains(self, pos, p, nrank, nthreads=1, explicit_self=False):
        """One pass over `nrank` ranks emulated here: acc (n, 3) input
        order, per-rank counters, each particle's rank."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        prm = self._params(p, nthreads, True, True)
        acc = np.empty_like(pos)
        cnt = np.zeros((nrank, 16), np.int64)
        rank = np.empty(n, np.int32)
        rc = self.lib.po_run_domains(nrank, C.byref(prm), n, _ptr(pos), int(explicit_self), _ptr(acc),
                                     _ptr(cnt, _lp), _ptr(rank, _ip))
        if rc != 0:
            raise RuntimeError(f"oracle domain pass failed with code {rc}")
        return acc, [dict(zip(COUNTER_NAMES, (int(c) for c in row))) for row in cnt], rank

    def prepare_domain(self, pos, p, lo, hi, axis, nthreads=1):
        """fmm_prepare of one rank: its tree over the domain box (lo, hi)."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        prm = self._params(p, nthreads, True, True)
        lo = np.ascontiguousarray(lo, np.float64)
        hi = np.ascontiguousarray(hi, np.float64)
        rc = self.lib.po_prepare_domain(self.state, C.byref(prm), _ptr(lo), _ptr(hi), int(axis), pos.shape[0],
                                        _ptr(pos))
        if rc != 0:
            raise RuntimeError(f"oracle domain prepare failed with code {rc}")

    def export(self, recv_lo, recv_hi, shift):
        """The prepared tree shifted and pruned for the receiving domain
        (its top-tree box recv_lo..recv_hi): nodes (structured: npart, son,
        width, center, M), bodies (n, 3)."""
        lo = np.asarray(recv_lo, np.float64)
        hi = np.asarray(recv_hi, np.float64)
        tc, tw = 0.5 * (hi + lo), hi - lo                  # the receiver's top-tree box
        rlo, rhi = tc - 0.5 * tw, tc + 0.5 * tw             # its root's bounds
        rc_, rw = np.ascontiguousarray(0.5 * (rhi + rlo)), np.ascontiguousarray(rhi - rlo)
        sh = np.ascontiguousarray(shift, np.float64)
        nn, nb = C.c_int(0), C.c_int(0)
        self.lib.po_export(self.state, _ptr(rc_), _ptr(rw), _ptr(sh), C.byref(nn), C.byref(nb), 0, 0, None, None)
        dt = np.dtype([("npart", "i4"), ("son", "i4", 2), ("width", "f8", 3), ("center", "f8", 3),
                       ("M", "f8", NMULTI)], align=True)
        nodes = np.zeros(nn.value, dt)
        bodies = np.zeros((nb.value, 3))
        rc = self.lib.po_export(self.state, _ptr(rc_), _ptr(rw), _ptr(sh), C.byref(nn), C.byref(nb), nodes.size,
                                nb.value, nodes.ctypes.data, _ptr(bodies))
        if rc != 0:
            raise RuntimeError(f"oracle export failed with code {rc}")
        return nodes, bodies

    def forces_sample(self, targets):
        """Forces for another target set on the last pass's tree and lists:
        (acc (len(targets), 3), seconds)."""
        targets = np.ascontiguousarray(targets, np.int32)
        acc = np.empty((targets.size, 3))
        secs = C.c_double(0.0)
        rc = self.lib.po_forces_sample(self.state, targets.size, _ptr(targets, _ip), _ptr(acc), C.byref(secs))
        if rc != 0:
            raise RuntimeError(f"oracle sampled forces failed with code {rc}")
        return acc, secs.value

    def _tree_port(self, counters):
        class Shim:
            pass
        shim = Shim()
        shim.po_copy_leaves = lambda *a: self.lib.po_copy_leaves(self.state, *a)
        shim.po_copy_nodes = lambda *a: self.lib.po_copy_nodes(self.state, *a)
        return self._tree(shim, "po_", counters)

    def kick_loga(self, om, ox, la, lb):
        return self.lib.po_kick_loga(om, ox, la, lb)

    def drift_loga(self, om, ox, la, lb):
        return self.lib.po_drift_loga(om, ox, la, lb)

    def kick(self, vel, acc, dkh):
        """vel += acc dkh in place (float64 arrays of equal size)."""
        assert vel.dtype == np.float64 and vel.flags.c_contiguous
        acc = np.ascontiguousarray(acc, np.float64)
        self.lib.po_kick(vel.size, _ptr(vel), _ptr(acc), dkh)

    def drift(self, pos, vel, dd, L):
        """pos += vel dd in place, wrapped into [0, L)."""
        assert pos.dtype == np.float64 and pos.flags.c_contiguous
        vel = np.ascontiguousarray(vel, np.float64)
        self.lib.po_drift(pos.size, _ptr(pos), _ptr(vel), dd, L)

    def direct_sum(self, pos, p, targets, rmax=None, nthreads=1):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        targets = np.ascontiguousarray(targets, np.int32)
        prm = self._params(p, nthreads)
        out = np.empty((targets.size, 3))
        rmax = rmax if rmax is not None else 2.0 * p["rcut"]
        rc = self.lib.po_direct_sum(C.byref(prm), pos.shape[0], _ptr(pos), targets.size,
                                    _ptr(targets, _ip), rmax, _ptr(out))
        if rc != 0:
            raise RuntimeError(f"direct sum failed with code {rc}")
        return out

    def m2l(self, d, M, rs):
        L = np.zeros(NMULTI)
        M = np.ascontiguousarray(M, np.float64)
        self.lib.po_m2l(d[0], d[1], d[2], _ptr(M), _ptr(L), rs)
        return L

    def m2m(self, d, M):
        out = np.zeros(NMULTI)
        M = np.ascontiguousarray(M, np.float64)
        self.lib.po_m2m(d[0], d[1], d[2], _ptr(M), _ptr(out))
        return out

    def l2l(self, d, L):
        out = np.zeros(NMULTI)
        L = np.ascontiguousarray(L, np.float64)
        self.lib.po_l2l(d[0], d[1], d[2], _ptr(L), _ptr(out))
        return out

    def p2m(self, pos, mass, center):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        c = np.ascontiguousarray(center, np.float64)
        M = np.zeros(NMULTI)
        self.lib.po_p2m(pos.shape[0], _ptr(pos), mass, _ptr(c), _ptr(M))
        return M

    def l2p(self, pos, center, L):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        c = np.ascontiguousarray(center, np.float64)
        L = np.ascontiguousarray(L, np.float64)
        acc = np.zeros_like(pos)
        self.lib.po_l2p(pos.shape[0], _ptr(pos), _ptr(c), _ptr(L), _ptr(acc))
        return acc

    def acceptance(self, wi, wj, dist, theta, rcut):
        a = [np.ascontiguousarray(x, np.float64) for x in (wi, wj, dist)]
        return self.lib.po_acceptance(_ptr(a[0]), _ptr(a[1]), _ptr(a[2]), theta, rcut)
