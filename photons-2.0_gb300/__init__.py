"""Python host interface to libphotons_fmm.so -- the GB300 FMM short-range
force pass of photoNs-2.0 (include/photons_fmm.h).

Two ways in, mirroring the C ABI:

* ``ForcePass``   -- the context-based pass on plain arrays
  (photons_force_pass): positions in, accelerations out, plus counters,
  timings, the tree and the interaction lists for inspection.
* ``Reference``   -- the reference's own entry points (fmm_construct,
  fmm_prepare, fmm_task, fmm_ext, fmm_deconstruct, ...) driven through the
  reference's globals, exactly as src/photoNs.c drives the CPU FMM.

The CUDA library is required: every call fails loudly when it is missing.
There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libphotons_fmm.so")

FP32_SPLIT = 0
FP64 = 1

F_DEVICE_IO = 1
F_TREE_ORDER = 2
F_NO_FARFIELD = 4
F_MULTIPOLES = 8
F_KEEP_LISTS = 16
F_ONE_WAY = 32
F_P2P_BULK = 64  # FP32 mutual kernel: source leaves staged by TMA bulk copies
P2P_SHAPES = 5


def F_P2P_SHAPE(shape):
    """Flag bits naming the FP32 mutual P2P kernel build (0: chosen by MAXLEAF)."""
    return int(shape) << 8

NMULTI = 20
LIST_KINDS = {"p2p": 0, "m2l": 1, "p2p_ext": 2, "m2l_ext": 3}
COUNTER_NAMES = [
    "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "NLEAF", "NNODE",
    "nleaf", "nnode", "first_leaf", "first_node", "direct_local_start",
    "n_p2p", "n_m2l", "n_p2p_ext", "n_m2l_ext", "n_images",
    "pairs_local", "pairs_image", "depth", "max_stack", "max_stage", "pd_peak",
    "p2p_entries", "m2l_entries",
]
TIMING_NAMES = ["total", "upload", "tree", "walk", "p2p", "farfield", "download"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_longlong)


class Params(C.Structure):
    _fields_ = [("boxsize", C.c_double), ("theta", C.c_double), ("rs", C.c_double), ("rcut", C.c_double),
                ("eps", C.c_double), ("mass", C.c_double), ("maxleaf", C.c_int), ("precision", C.c_int),
                ("image_mask", C.c_uint), ("flags", C.c_int)]


class PhotonsError(RuntimeError):
    pass


class Domain(C.Structure):
    """A rank's domain: its box and its tree's first split axis."""
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3), ("axis", C.c_int)]


# inc/photoNs.h:177-189: RemoteNode (a node of an exported tree) and RemoteBody
REMOTE_NODE = np.dtype([("npart", "i4"), ("son", "i4", 2), ("width", "f8", 3), ("center", "f8", 3),
                        ("M", "f8", NMULTI)], align=True)
REMOTE_BODY = np.dtype([("pos", "f8", 3), ("replenish", "f8")])


_lib = None


def library_path():
    return LIB_PATH


def load_library():
    """Load the CUDA library (build it with build.py / __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise PhotonsError(f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH, mode=C.RTLD_GLOBAL)
    lib.photons_create.restype = C.c_void_p
    lib.photons_create.argtypes = [C.c_int]
    lib.photons_destroy.argtypes = [C.c_void_p]
    lib.photons_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    lib.photons_force_pass.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int, C.c_void_p, C.c_void_p]
    lib.photons_force_pass_boxes.argtypes = [C.c_void_p, C.c_int, C.POINTER(Params), _ip, C.c_void_p, C.c_void_p]
    lib.photons_get_counters.argtypes = [C.c_void_p, _lp, C.c_int]
    lib.photons_get_timings.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int]
    lib.photons_get_perm.argtypes = [C.c_void_p, _ip]
    lib.photons_get_positions.argtypes = [C.c_void_p, _dp]
    lib.photons_copy_leaves.argtypes = [C.c_void_p, _ip, _dp, _dp, _dp]
    lib.photons_copy_nodes.argtypes = [C.c_void_p, _ip, _dp, _dp, _dp]
    lib.photons_list_size.restype = C.c_longlong
    lib.photons_list_size.argtypes = [C.c_void_p, C.c_int]
    lib.photons_list_copy.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip]
    lib.photons_op_batch.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_double]
    lib.photons_direct_sum.argtypes = [C.POINTER(Params), C.c_int, _dp, C.c_int, _ip, C.c_double, _dp]
    lib.photons_launch_count.restype = C.c_ulonglong
    lib.photons_launch_count.argtypes = []
    lib.photons_fp32_fma_peak.restype = C.c_double
    lib.photons_fp32_fma_peak.argtypes = [C.c_int]
    lib.photons_fp64_fma_peak.restype = C.c_double
    lib.photons_fp64_fma_peak.argtypes = [C.c_int]
    lib.photons_split_factor_fp64.argtypes = [_dp, C.c_int, C.c_int, _dp]
    lib.photons_host_alloc.restype = C.c_void_p
    lib.photons_host_alloc.argtypes = [C.c_size_t]
    lib.photons_host_free.argtypes = [C.c_void_p]
    lib.photons_gpu_error.restype = C.c_char_p
    lib.photons_gpu_status.restype = C.c_int
    for name in ("fmm_construct", "fmm_prepare", "fmm_task", "fmm_ext", "fmm_deconstruct", "build_localtree",
                 "partmesh_thread", "partmesh"):
        getattr(lib, name).restype = None
        getattr(lib, name).argtypes = []
    lib.pm_thread.restype = C.c_void_p
    lib.pm_thread.argtypes = [C.c_void_p]
    lib.acceptance.restype = C.c_int
    lib.acceptance.argtypes = [_dp, _dp, _dp]
    lib.fmm_remote.argtypes = [C.c_int, _dp]
    for name in ("photons_kick_loga", "photons_drift_loga"):
        getattr(lib, name).restype = C.c_double
        getattr(lib, name).argtypes = [C.c_double] * 4
    lib.photons_kick.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    lib.photons_drift.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    lib.photons_pm_force.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.photons_kdk_step_pm.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int, C.c_int] + [C.c_void_p] * 4 + \
        [C.c_double, C.c_double]
    lib.photons_kdk_step.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_double, C.c_double]
    lib.photons_kdk_step_ordered.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int] + [C.c_void_p] * 4 + \
        [C.c_double, C.c_double]
    lib.photons_kdk_step_pm_ordered.argtypes = [C.c_void_p, C.POINTER(Params), C.c_int, C.c_int] + \
        [C.c_void_p] * 5 + [C.c_double, C.c_double]
    lib.photons_domain_split.argtypes = [C.c_int, C.c_double, C.POINTER(Domain), _dp]
    lib.photons_domain_assign.argtypes = [C.c_int, _dp, C.c_int, _dp, _ip]
    lib.photons_domain_rebalance.argtypes = [C.c_int, C.c_double, _dp, _dp, C.POINTER(Domain)]
    lib.photons_domain_prepare.argtypes = [C.c_void_p, C.POINTER(Params), C.POINTER(Domain), C.c_int, C.c_void_p]
    lib.photons_let_export.argtypes = [C.c_void_p, C.POINTER(Domain), _dp, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                       _ip, _ip]
    lib.photons_let_import.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    lib.photons_domain_finish.argtypes = [C.c_void_p, C.c_void_p]
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        msg = _lib.photons_gpu_error().decode(errors="replace")
        raise PhotonsError(f"photons error {rc}: {msg}")


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def make_params(p, precision=FP32_SPLIT, image_mask=0, flags=0):
    """photons_params from a dict with boxsize, theta, rs, rcut, eps, mass, maxleaf."""
    return Params(float(p["boxsize"]), float(p["theta"]), float(p["rs"]), float(p["rcut"]), float(p["eps"]),
                  float(p["mass"]), int(p["maxleaf"]), int(precision), int(image_mask), int(flags))


class ForcePass:
    """One GPU context; run() evaluates the short-range force pass."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = self.lib.photons_create(device)
        if not h:
            raise PhotonsError(self.lib.photons_gpu_error().decode(errors="replace"))
        self.h = C.c_void_p(h)
        self.n = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.photons_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        _check(self.lib.photons_set_stream(self.h, C.c_void_p(stream_ptr)))

    def run(self, pos, p, precision=FP32_SPLIT, image_mask=0, flags=0, out=None):
        """Host arrays: pos (N,3) float64 -> acc (N,3) float64."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        acc = out if out is not None else np.empty_like(pos)
        prm = make_params(p, precision, image_mask, flags & ~F_DEVICE_IO)
        _check(self.lib.photons_force_pass(self.h, C.byref(prm), n, pos.ctypes.data, acc.ctypes.data))
        self.n = n
        return acc

    def run_boxes(self, boxes, precision=FP32_SPLIT, image_mask=0, flags=0):
        """Independent periodic boxes in one pass: boxes = [(pos (n_b,3), params_b), ...]
        -> list of acc (n_b,3).  theta and maxleaf are taken from the first box."""
        nb = len(boxes)
        counts = np.array([b[0].shape[0] for b in boxes], np.int32)
        pos = np.ascontiguousarray(np.concatenate([np.asarray(b[0], np.float64).reshape(-1, 3) for b in boxes]))
        acc = np.empty_like(pos)
        p0 = boxes[0][1]
        prm = (Params * nb)()
        for i, (_, p) in enumerate(boxes):
            q = dict(p, theta=p0["theta"], maxleaf=p0["maxleaf"])
            prm[i] = make_params(q, precision, image_mask, flags & ~F_DEVICE_IO)
        _check(self.lib.photons_force_pass_boxes(self.h, nb, prm, _p(counts, _ip), pos.ctypes.data, acc.ctypes.data))
        self.n = pos.shape[0]
        return np.split(acc, np.cumsum(counts)[:-1])

    def run_device(self, pos_ptr, acc_ptr, n, p, precision=FP32_SPLIT, image_mask=0, flags=0):
        """Device pointers (e.g. torch tensors' data_ptr()), AoS (n,3) float64."""
        prm = make_params(p, precision, image_mask, flags | F_DEVICE_IO)
        _check(self.lib.photons_force_pass(self.h, C.byref(prm), int(n), C.c_void_p(pos_ptr), C.c_void_p(acc_ptr)))
        self.n = n

    def kdk_step_device(self, pos_ptr, vel_ptr, acc_ptr, n, p, dkh, dd, precision=FP32_SPLIT, image_mask=0, flags=0):
        """One kick-drift-kick step on device arrays (n,3) float64: vel += acc dkh,
        pos += vel dd (wrapped), acc = forces at the new positions, vel += acc dkh."""
        prm = make_params(p, precision, image_mask, flags | F_DEVICE_IO)
        _check(self.lib.photons_kdk_step(self.h, C.byref(prm), int(n), C.c_void_p(pos_ptr), C.c_void_p(vel_ptr),
                                         C.c_void_p(acc_ptr), float(dkh), float(dd)))
        self.n = n

    def kdk_step_pm_device(self, pos_ptr, vel_ptr, acc_ptr, acc_pm_ptr, n, p, nside, dkh, dd, precision=FP32_SPLIT,
                           flags=0):
        """The reference's step with both force halves on device arrays (n,3) float64."""
        prm = make_params(p, precision, 0, flags | F_DEVICE_IO)
        _check(self.lib.photons_kdk_step_pm(self.h, C.byref(prm), int(nside), int(n), C.c_void_p(pos_ptr),
                                            C.c_void_p(vel_ptr), C.c_void_p(acc_ptr), C.c_void_p(acc_pm_ptr),
                                            float(dkh), float(dd)))
        self.n = n

    def kdk_step_ordered_device(self, pos_ptr, vel_ptr, acc_ptr, ids_ptr, n, p, dkh, dd, precision=FP32_SPLIT,
                                flags=0, nside=0, acc_pm_ptr=0):
        """The KDK step (with the PM half when nside > 0) keeping pos, vel,
        acc (acc_pm) and ids (int64, may be 0) in the order of the pass's
        tree, as the reference keeps part[]; device arrays."""
        prm = make_params(p, precision, 0, flags | F_DEVICE_IO)
        if nside:
            _check(self.lib.photons_kdk_step_pm_ordered(self.h, C.byref(prm), int(nside), int(n), C.c_void_p(pos_ptr),
                                                        C.c_void_p(vel_ptr), C.c_void_p(acc_ptr),
                                                        C.c_void_p(acc_pm_ptr), C.c_void_p(ids_ptr or None),
                                                        float(dkh), float(dd)))
        else:
            _check(self.lib.photons_kdk_step_ordered(self.h, C.byref(prm), int(n), C.c_void_p(pos_ptr),
                                                     C.c_void_p(vel_ptr), C.c_void_p(acc_ptr),
                                                     C.c_void_p(ids_ptr or None), float(dkh), float(dd)))
        self.n = n

    # ---- a rank's domain pass (several ranks, one GPU each) ----
    def domain_prepare(self, pos, p, dom, precision=FP32_SPLIT, flags=0):
        """Start this rank's pass: the tree of its particles over its domain."""
        self._dom_pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)  # must outlive the pass
        prm = make_params(p, precision, 0, flags & ~F_DEVICE_IO)
        _check(self.lib.photons_domain_prepare(self.h, C.byref(prm), C.byref(dom), self._dom_pos.shape[0],
                                               self._dom_pos.ctypes.data))
        self.n = self._dom_pos.shape[0]

    def let_export(self, receiver, shift=(0.0, 0.0, 0.0)):
        """This rank's tree shifted and pruned for `receiver` (a Domain):
        (nodes, bodies) as REMOTE_NODE / REMOTE_BODY arrays."""
        sh = np.ascontiguousarray(shift, np.float64)
        nn, nb = C.c_int(0), C.c_int(0)
        _check(self.lib.photons_let_export(self.h, C.byref(receiver), _p(sh), None, 0, None, 0, C.byref(nn),
                                           C.byref(nb)))
        nodes = np.zeros(nn.value, REMOTE_NODE)
        bodies = np.zeros(nb.value, REMOTE_BODY)
        _check(self.lib.photons_let_export(self.h, C.byref(receiver), _p(sh), nodes.ctypes.data, nodes.size,
                                           bodies.ctypes.data, bodies.size, C.byref(nn), C.byref(nb)))
        return nodes, bodies

    def let_import(self, nodes, bodies):
        """Keep a received tree for domain_finish."""
        nodes = np.ascontiguousarray(nodes, REMOTE_NODE)
        bodies = np.ascontiguousarray(bodies, REMOTE_BODY)
        _check(self.lib.photons_let_import(self.h, nodes.ctypes.data, nodes.size, bodies.ctypes.data, bodies.size))

    def domain_finish(self):
        """Walks, P2P and far field over the local, periodic and received
        trees: the accelerations (n, 3) in the prepared positions' order."""
        acc = np.empty((self.n, 3))
        _check(self.lib.photons_domain_finish(self.h, acc.ctypes.data))
        return acc

    def pm_force(self, pos, p, nside):
        """PM long-range acceleration (n,3) on an nside^3 mesh (host arrays)."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        acc = np.empty_like(pos)
        prm = make_params(p, FP64, 0, 0)
        _check(self.lib.photons_pm_force(self.h, C.byref(prm), int(nside), pos.shape[0], pos.ctypes.data,
                                         acc.ctypes.data))
        return acc

    def counters(self):
        v = np.zeros(32, np.int64)
        _check(self.lib.photons_get_counters(self.h, _p(v, _lp), 32))
        return dict(zip(COUNTER_NAMES, (int(x) for x in v)))

    def timings(self):
        v = (C.c_float * 8)()
        _check(self.lib.photons_get_timings(self.h, v, 8))
        return dict(zip(TIMING_NAMES, list(v)))

    def perm(self):
        out = np.empty(self.n, np.int32)
        _check(self.lib.photons_get_perm(self.h, _p(out, _ip)))
        return out

    def positions(self):
        out = np.empty((self.n, 3))
        _check(self.lib.photons_get_positions(self.h, _p(out)))
        return out

    def tree(self):
        c = self.counters()
        nl, nn = c["nleaf"], c["nnode"]
        lip = np.empty((nl, 2), np.int32)
        lg = np.empty((nl, 6))
        lM = np.empty((nl, NMULTI))
        lL = np.empty((nl, NMULTI))
        ni = np.empty((nn, 3), np.int32)
        ng = np.empty((nn, 7))
        nM = np.empty((nn, NMULTI))
        nL = np.empty((nn, NMULTI))
        _check(self.lib.photons_copy_leaves(self.h, _p(lip, _ip), _p(lg), _p(lM), _p(lL)))
        _check(self.lib.photons_copy_nodes(self.h, _p(ni, _ip), _p(ng), _p(nM), _p(nL)))
        return dict(leaf_ipart=lip[:, 0].copy(), leaf_npart=lip[:, 1].copy(), leaf_center=lg[:, :3].copy(),
                    leaf_width=lg[:, 3:].copy(), leaf_M=lM, leaf_L=lL, node_npart=ni[:, 0].copy(),
                    node_son=ni[:, 1:].copy(), node_split=ng[:, 0].copy(), node_center=ng[:, 1:4].copy(),
                    node_width=ng[:, 4:].copy(), node_M=nM, node_L=nL)

    def lists(self):
        out = {}
        for name, k in LIST_KINDS.items():
            m = self.lib.photons_list_size(self.h, k)
            if m < 0:
                _check(self.lib.photons_gpu_status() or 6)
            t = np.empty(m, np.int32)
            s = np.empty(m, np.int32)
            im = np.empty(m, np.int32)
            if m:
                _check(self.lib.photons_list_copy(self.h, k, _p(t, _ip), _p(s, _ip), _p(im, _ip)))
            out[name] = (t, s, im)
        return out


def domain_split(nrank, boxsize):
    """The reference's first decomposition over nrank ranks: (domains, split planes)."""
    lib = load_library()
    doms = (Domain * nrank)()
    split = np.zeros(max(nrank - 1, 1))
    _check(lib.photons_domain_split(int(nrank), float(boxsize), doms, _p(split)))
    return list(doms), split[:nrank - 1].copy()


def domain_assign(nrank, split, pos):
    """The rank of each position under the split planes."""
    lib = load_library()
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    split = np.ascontiguousarray(split if len(split) else [0.0], np.float64)
    rank = np.empty(pos.shape[0], np.int32)
    _check(lib.photons_domain_assign(int(nrank), _p(split), pos.shape[0], _p(pos), _p(rank, _ip)))
    return rank


def domain_rebalance(nrank, boxsize, split, rank_time):
    """Split planes moved by the ranks' measured times: (domains, split)."""
    lib = load_library()
    split = np.array(split if len(split) else [0.0], np.float64)
    t = np.ascontiguousarray(rank_time, np.float64)
    doms = (Domain * nrank)()
    _check(lib.photons_domain_rebalance(int(nrank), float(boxsize), _p(split), _p(t), doms))
    return list(doms), split[:nrank - 1].copy()


IMAGE_SHIFTS = [(mi, mj, mk) for mi in (-1, 0, 1) for mj in (-1, 0, 1) for mk in (-1, 0, 1) if (mi, mj, mk) != (0, 0, 0)]


def let_schedule(rank, nrank):
    """The exchanges of one rank's pass in fmm_ext's order
    (src/fmm.c:1020-1045, fmm_remote's srank/rrank, src/remotes.c:690-691):
    [(send_to, recv_from, shift unit)]: the other ranks unshifted, then for
    every periodic image every other rank.  A rank's own images are walked
    on the fly, not exchanged."""
    out = [((rank + i) % nrank, (rank - i) % nrank, (0, 0, 0)) for i in range(1, nrank)]
    for s in IMAGE_SHIFTS:
        out += [((rank + i) % nrank, (rank - i) % nrank, s) for i in range(1, nrank)]
    return out


def op_batch(op, d, inp, inout, rs=1.0):
    """Batched operators on the GPU: op 'm2l' (L += M2L(d, M)), 'm2m', 'l2l'."""
    lib = load_library()
    code = {"m2l": 0, "m2m": 1, "l2l": 2}[op]
    d = np.ascontiguousarray(d, np.float64).reshape(-1, 3)
    inp = np.ascontiguousarray(inp, np.float64).reshape(-1, NMULTI)
    out = np.ascontiguousarray(inout, np.float64).reshape(-1, NMULTI).copy()
    _check(lib.photons_op_batch(code, d.shape[0], _p(d), _p(inp), _p(out), float(rs)))
    return out


def direct_sum(pos, p, targets, rmax=None):
    """FP64 GPU direct sum of the untruncated split kernel for the target subset."""
    lib = load_library()
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    targets = np.ascontiguousarray(targets, np.int32)
    out = np.empty((targets.size, 3))
    prm = make_params(p)
    rmax = 2.0 * p["rcut"] if rmax is None else rmax
    _check(lib.photons_direct_sum(C.byref(prm), pos.shape[0], _p(pos), targets.size, _p(targets, _ip),
                                  float(rmax), _p(out)))
    return out


class GadgetHeader(C.Structure):
    _fields_ = [("npart", C.c_int * 6), ("mass", C.c_double * 6), ("time", C.c_double), ("redshift", C.c_double),
                ("flag_sfr", C.c_int), ("flag_feedback", C.c_int), ("npart_total", C.c_int * 6),
                ("flag_cooling", C.c_int), ("num_files", C.c_int), ("boxsize", C.c_double), ("omega0", C.c_double),
                ("omega_lambda", C.c_double), ("hubble", C.c_double)]


def gadget_read(path, first=0, count=None):
    """Gadget-2 snapshot -> (header dict, pos (n,3), vel (n,3)); velocities
    scaled by (1/(1+z))^1.5 as the reference reads them."""
    lib = load_library()
    lib.photons_gadget_read_header.argtypes = [C.c_char_p, C.POINTER(GadgetHeader)]
    lib.photons_gadget_read.argtypes = [C.c_char_p, C.c_longlong, C.c_longlong, C.c_void_p, C.c_void_p]
    h = GadgetHeader()
    _check(lib.photons_gadget_read_header(str(path).encode(), C.byref(h)))
    n = sum(h.npart) - first if count is None else count
    pos = np.empty((n, 3))
    vel = np.empty((n, 3))
    _check(lib.photons_gadget_read(str(path).encode(), first, n, pos.ctypes.data, vel.ctypes.data))
    hd = {f: (list(getattr(h, f)) if f in ("npart", "mass", "npart_total") else getattr(h, f)) for f, _ in h._fields_}
    return hd, pos, vel


def gadget_write(path, header, pos, vel):
    """Write one Gadget-2 file (header dict as gadget_read returns)."""
    lib = load_library()
    lib.photons_gadget_write.argtypes = [C.c_char_p, C.POINTER(GadgetHeader), C.c_longlong, C.c_void_p, C.c_void_p]
    h = GadgetHeader()
    for f, _ in h._fields_:
        v = header.get(f, 0)
        if f in ("npart", "mass", "npart_total"):
            arr = getattr(h, f)
            for i, x in enumerate(v if v else [0] * 6):
                arr[i] = x
        else:
            setattr(h, f, v)
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    _check(lib.photons_gadget_write(str(path).encode(), C.byref(h), pos.shape[0], pos.ctypes.data, vel.ctypes.data))


def kick_loga(omega_m, omega_x, loga_i, loga_f):
    """The reference's kick factor over [loga_i, loga_f] (src/initial.c:639-660)."""
    return load_library().photons_kick_loga(float(omega_m), float(omega_x), float(loga_i), float(loga_f))


def drift_loga(omega_m, omega_x, loga_i, loga_f):
    """The reference's drift factor over [loga_i, loga_f] (src/initial.c:662-683)."""
    return load_library().photons_drift_loga(float(omega_m), float(omega_x), float(loga_i), float(loga_f))


def kick(n, vel_ptr, acc_ptr, dkh, stream_ptr=0):
    """vel += acc dkh on device arrays (n,3) float64 (asynchronous on the stream)."""
    _check(load_library().photons_kick(int(n), C.c_void_p(vel_ptr), C.c_void_p(acc_ptr), float(dkh),
                                       C.c_void_p(stream_ptr)))


def drift(n, pos_ptr, vel_ptr, dd, boxsize, stream_ptr=0):
    """pos += vel dd, wrapped into [0, boxsize), on device arrays (asynchronous)."""
    _check(load_library().photons_drift(int(n), C.c_void_p(pos_ptr), C.c_void_p(vel_ptr), float(dd),
                                        float(boxsize), C.c_void_p(stream_ptr)))


def fp64_fma_peak(iters=256):
    lib = load_library()
    v = lib.photons_fp64_fma_peak(int(iters))
    if v <= 0:
        raise PhotonsError("FP64 FMA probe failed: " + lib.photons_gpu_error().decode(errors="replace"))
    return v


def host_array(shape, dtype=np.float64):
    """A numpy array in pinned host memory from photons_host_alloc (freed
    with the array), for the host-buffer pass: the pass's kernels read and
    write it over the host link, at the link's rate."""
    import weakref

    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    nbytes = max(1, count * dtype.itemsize)
    lib = load_library()
    ptr = lib.photons_host_alloc(nbytes)
    if not ptr:
        raise PhotonsError("pinned host allocation failed: " + lib.photons_gpu_error().decode(errors="replace"))
    buf = (C.c_char * nbytes).from_address(ptr)
    weakref.finalize(buf, lib.photons_host_free, C.c_void_p(ptr))
    return np.frombuffer(buf, dtype=dtype, count=count).reshape(shape)


def split_factor_fp64(u, exact=False):
    """The FP64 kernels' split factor erfc(u) + (2/sqrt(pi)) u exp(-u^2) at
    the points u >= 0, on the device: their piecewise polynomials, or with
    exact=True erfc and exp."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    g = np.empty_like(u)
    _check(load_library().photons_split_factor_fp64(_p(u, _dp), int(u.size), int(bool(exact)), _p(g, _dp)))
    return g


def fp32_fma_peak(iters=4096):
    lib = load_library()
    v = lib.photons_fp32_fma_peak(int(iters))
    if v <= 0:
        raise PhotonsError("FMA probe failed: " + lib.photons_gpu_error().decode(errors="replace"))
    return v


class Reference:
    """The reference's entry points on the reference's globals."""

    BODY = np.dtype([("pos", "f8", 3), ("acc", "f8", 3), ("vel", "f8", 3), ("acc_pm", "f8", 3)])

    def __init__(self):
        self.lib = load_library()
        self._part = None

    def _set(self, ctype, name, value):
        ctype.in_dll(self.lib, name).value = value

    def _get(self, ctype, name):
        return ctype.in_dll(self.lib, name).value

    def setup(self, pos, p):
        """Fill part[] and the parameter globals as src/initial.c would."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        body = np.zeros(n, self.BODY)
        body["pos"] = pos
        self._part = body
        C.c_void_p.in_dll(self.lib, "part").value = body.ctypes.data
        self._set(C.c_int, "NPART", n)
        self._set(C.c_long, "NPART_TOTAL", n)
        self._set(C.c_int, "PROC_SIZE", 1)
        self._set(C.c_int, "PROC_RANK", 0)
        self._set(C.c_double, "BOXSIZE", p["boxsize"])
        self._set(C.c_int, "MAXLEAF", int(p["maxleaf"]))
        self._set(C.c_double, "open_angle", p["theta"])
        self._set(C.c_double, "splitRadius", p["rs"])
        self._set(C.c_double, "cutoffRadius", p["rcut"])
        self._set(C.c_double, "SoftenScale", p["eps"])
        self._set(C.c_double, "MASSPART", p["mass"])
        for name in ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote"):
            self._set(C.c_ulong, name, 0)

    def force_pass(self, pm_nside=0):
        """The driver sequence of src/photoNs.c:97-116.  With pm_nside, the PM
        runs as the driver runs it: pm_thread on a second thread from after
        fmm_prepare until before fmm_ext, beside fmm_task (PMTHREAD)."""
        import threading
        lib = self.lib
        lib.fmm_construct()
        lib.fmm_prepare()
        pm = None
        if pm_nside:
            self._set(C.c_int, "NSIDE", int(pm_nside))
            pm = threading.Thread(target=lib.pm_thread, args=(None,))
            pm.start()
        lib.fmm_task()
        if pm:
            pm.join()
        acc_task = self._part["acc"].copy()
        lib.fmm_ext()
        return acc_task

    def pm(self, nside):
        """partmesh_thread() on the current part[]: acc_pm (n, 3)."""
        self._set(C.c_int, "NSIDE", int(nside))
        self.lib.partmesh_thread()
        return self._part["acc_pm"].copy()

    def part(self):
        return self._part

    def counters(self):
        return {k: int(self._get(C.c_ulong, k)) for k in ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote")}

    def deconstruct(self):
        self.lib.fmm_deconstruct()


def autotune_leaf(fp, pos, p, candidates=(16, 24, 32, 48, 64), error_bound=1e-4, sample=2000, repeats=2,
                  precision=FP32_SPLIT, seed=11, shapes=True):
    """Pick MAXLEAF and the FP32 P2P kernel for this input.

    Leaf size: the fastest candidate whose median relative force error
    against the FP64 direct sum (untruncated split kernel within 2 rcut,
    `sample` random particles) is within `error_bound`; if none qualifies,
    the most accurate one.  From leaf 48 the pass evaluates each symmetric
    leaf pair once by default; halo-dominated inputs can run faster one way
    (F_ONE_WAY), so both are timed there.  Kernel shape (with `shapes`): at
    the chosen leaf size, when the mutual kernel won, each of its builds
    (resident blocks per SM, interleaved dependency chains, the 6-target
    path; F_P2P_SHAPE), with source leaves staged by per-lane cp.async or by
    TMA bulk copies (F_P2P_BULK), is timed and the fastest kept.  All of
    these give the same forces to FP32 rounding (the two stagings, the same
    bits).

    Returns (best_leaf, table, flags): table lists, per candidate, the pass
    time on the device (ms, CUDA events: tree, walk, P2P, far field,
    gather), pairs per particle, the median / 99th-percentile error, the
    kernel and its flags; flags are those of the chosen candidate."""
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    tgt = rng.choice(pos.shape[0], min(sample, pos.shape[0]), replace=False).astype(np.int32)
    ref = direct_sum(pos, p, tgt)
    nref = np.linalg.norm(ref, axis=1)
    table = []

    def trial(leaf, flags, kernel):
        q = dict(p)
        q["maxleaf"] = int(leaf)
        ms = []
        acc = None
        for _ in range(repeats):
            acc = fp.run(pos, q, precision=precision, flags=flags)
            t = fp.timings()
            ms.append(t["total"] - t["upload"] - t["download"])  # the device part of the pass
        c = fp.counters()
        err = np.linalg.norm(acc[tgt] - ref, axis=1) / np.maximum(nref, 1e-300)
        row = dict(maxleaf=int(leaf), ms=float(min(ms)), median=float(np.median(err)),
                   p99=float(np.percentile(err, 99)),
                   pairs_per_particle=(c["pairs_local"] + c["pairs_image"]) / pos.shape[0], kernel=kernel,
                   flags=int(flags))
        table.append(row)
        return row

    for leaf in candidates:
        mutual = precision == FP32_SPLIT and 48 <= leaf <= 64
        trial(leaf, 0, "mutual" if mutual else "one-way")
        if mutual:
            trial(leaf, F_ONE_WAY, "one-way")
    ok = [t for t in table if t["median"] <= error_bound]
    best = min(ok, key=lambda t: t["ms"]) if ok else min(table, key=lambda t: t["median"])
    if shapes and precision == FP32_SPLIT and best["kernel"] == "mutual":
        leaf = best["maxleaf"]
        builds = [(F_P2P_SHAPE(sh) | bulk, "mutual shape %d%s" % (sh, " bulk" if bulk else ""))
                  for sh in range(1, P2P_SHAPES) for bulk in (0, F_P2P_BULK)]
        for flags, kernel in builds:
            row = trial(leaf, flags, kernel)
            if row["ms"] < best["ms"] and row["median"] <= max(error_bound, best["median"]):
                best = row
    return best["maxleaf"], table, best["flags"]
