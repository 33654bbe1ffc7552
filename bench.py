"""Benchmark: photoNs-2.0 FMM short-range force pass on GB300.

Workload (the headline configuration): 256^3 = 16,777,216 particles in a
periodic box L = 500 Mpc/h, grid + Zel'dovich displacement of a Gaussian
field with P(k) ~ k^-2 (rms displacement 0.5 spacing, seed 3), mesh 256,
rs = 1.25 cells, rcut = 4.5 rs, theta = 0.5, softening 0.03 spacing.
Synthetic, seeded; forces exclude G as in the reference.

One step = one full short-range force pass (tree build, dual-tree walk with
26 periodic images, P2P, far field when any M2L occurs, gather) over the
resident particles, FP32 split precision.  value = particle-forces/s =
N / (time per pass).  Inputs (400 MB of FP64 positions) exceed the 126 MB
L2, so no flush is needed between steps.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
Under torchrun each rank runs an independent box (seed 3 + rank): replicas,
weak scaling, no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-forces/s at 256^3 clustered: FP32-split vs FP64 GPU at rel err <=1e-4"
UNIT = "particle-forces/s"
# fixed work unit per pair interaction of the reference's pair set (the
# conventional count for a softened, erfc-truncated pair force); the P2P
# roofline is this times the pairs, over the P2P phase time
FLOPS_PER_PAIR = 36
# DRAM traffic of one launch of the dominant kernel at 256^3 leaf 64 (bytes
# read + written): ncu dram__bytes_read.sum + dram__bytes_write.sum of one
# launch on the 128^3 workload of the same density, scaled by the particle
# count (x8; traffic grows in proportion).  The capture command and figures
# are kept with the kernel's profile summary.
TRAFFIC_PER_LAUNCH_256 = {"k_p2p_mutual": 13.12e9, "k_p2p_split_packed": 1.27e9}
# MAXLEAF the GPU arm's autotuner picks for each workload on GB300 (the
# fastest leaf within the 1e-4 median error bound); the CPU baselines run
# the same leaf so that both arms compute the same lists at the same error
CHOSEN_LEAF = {"zeldovich256": 64, "zeldovich512": 64, "nfw128": 24, "grid32": 16}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nside", type=int, default=256)
    ap.add_argument("--maxleaf", type=int, default=0, help="0: pick by the autotuner (error <= 1e-4)")
    ap.add_argument("--error-bound", type=float, default=1e-4)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison pass")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the parity leg (tree, lists, counters and FP64 forces against the oracle)")
    ap.add_argument("--workload", default="zeldovich256",
                    choices=["zeldovich256", "zeldovich512", "nfw128", "boxes256"],
                    help="zeldovich256: the headline (P(k)~k^-2, seed 3); zeldovich512: P(k)~k^-1.5, seed 5, "
                         "L=1000 at 512^3; nfw128: 50%% uniform + 50%% in NFW halos, L=200 at 128^3; "
                         "boxes256: 256 independent Plummer + uniform boxes of 16^3-64^3 particles in one pass")
    ap.add_argument("--kdk", action="store_true", help="also time device-resident kick-drift-kick steps")
    ap.add_argument("--pass-flags", type=int, default=0,
                    help="with --maxleaf: PHOTONS_F_* flags of the timed pass (e.g. 512: mutual build 2, "
                         "64: sources staged by TMA bulk copies)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms, dist, device="cpu"):
    """The slowest rank's time: a step of the whole job ends when every
    rank's step has ended (replicas: each rank runs its own box)."""
    if not dist:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def broadcast_from_rank0(v, dist, device="cpu"):
    """Rank 0's integer on every rank (the leaf size all replicas run)."""
    if not dist:
        return v
    import torch

    t = torch.tensor([int(v)], dtype=torch.int64, device=device)
    dist.broadcast(t, 0)
    return int(t.item())


def workload(nside, maxleaf, seed_offset=0, name="zeldovich256"):
    import __graft_entry__ as g

    g.load_package()
    from photons_gb300 import ics

    if name != "zeldovich256":
        return ics.make(name, nside=nside, maxleaf=maxleaf)
    L = 500.0 * nside / 256
    pos = ics.zeldovich(nside, L, -2.0, seed=3 + seed_offset)
    p = ics.force_params(pos.shape[0], L, nside, theta=0.5, maxleaf=maxleaf)
    return pos, p


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower().startswith("active")})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(nthreads=None, target_s=10.0, maxleaf=64, name="zeldovich256"):
    """The oracle's CPU restatement of the pass, all host threads, on a bounded
    sample of the same workload (same density, clustering and MAXLEAF,
    smaller box)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build_port()
    port = oracle.PortOracle(build=False)
    nthreads = nthreads or os.cpu_count() or 1
    nside = 48
    while True:
        pos, p = workload(nside, maxleaf, name=name)
        r = port.run(pos, p, capture=False, tree=False, nthreads=nthreads)
        secs = r["seconds"]
        if secs * 2.5 > target_s or nside >= 96:
            break
        nside = min(96, int(nside * (target_s / max(secs, 1e-3)) ** (1 / 3.0) * 0.9) // 8 * 8 or nside + 16)
    return {"value": pos.shape[0] / secs, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "one full pass of the same workload at %d^3 (L=%.1f, leaf %d, reference rules) "
                      "on the host: %.2f s" % (nside, p["boxsize"], maxleaf, secs)}


def workload_config(args, p, n):
    """The workload description both arms print (identical keys and values)."""
    return {"workload": args.workload, "n": int(n), "boxsize": p["boxsize"], "mesh": args.nside,
            "maxleaf": int(p["maxleaf"]), "theta": p["theta"], "rs": p["rs"], "rcut": p["rcut"], "eps": p["eps"],
            "l2": "inputs larger than L2 (positions %.0f MB), no flush" % (n * 24 / 1e6)}


def tree_blocks(perm, k, rng, nblocks=8):
    """k particles (input indices) in nblocks runs of consecutive tree
    positions: whole leaves of spatially compact regions, drawn at random."""
    n = perm.size
    per = max(1, k // nblocks)
    starts = rng.choice(max(1, n - per), nblocks, replace=False)
    return np.unique(np.concatenate([perm[s0:s0 + per] for s0 in starts])).astype(np.int32)


def run_reference_arm(args):
    """The reference's algorithm (the oracle's C restatement, pinned bit for
    bit to the reference's own fmm.c/operator.c/remotes.c) on the host cores,
    on the same workload and leaf size as the GPU arm.  Setup: the tree
    build, multipoles and dual-tree walks of the whole input, timed once.
    Each step: the forces (P2P, M2L, L2L, L2P) of a sample of the particles
    (runs of whole leaves at random places in tree order), timed; the step's
    time adds the setup's share for the sample (setup x sample / N), so the
    rate is particles per second of the whole pass."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build_port()
    port = oracle.PortOracle(build=False)
    nthreads = os.cpu_count() or 1
    name = args.workload if args.workload in CHOSEN_LEAF else "zeldovich256"
    leaf = args.maxleaf or CHOSEN_LEAF[name]
    pos, p = workload(args.nside, leaf, name=name)
    n = pos.shape[0]
    rng = np.random.default_rng(5)
    probe = rng.choice(n, 4096, replace=False).astype(np.int32)
    r = port.run_sample(pos, p, probe, nthreads=nthreads, perm=True)
    perm = r["perm"]
    setup_s = r["times"]["tree"] + r["times"]["multipoles"] + r["times"]["walk"]
    # size the sample to about 2 s of force work per step
    k = 16384
    _, secs = port.forces_sample(tree_blocks(perm, k, rng))
    k = int(min(n, max(4096, k * 2.0 / max(secs, 1e-3))))
    for _ in range(max(0, args.warmup)):
        port.forces_sample(tree_blocks(perm, k, rng))
    t, ks = [], []
    for _ in range(max(1, args.steps)):
        tg = tree_blocks(perm, k, rng)
        _, secs = port.forces_sample(tg)
        t.append(secs + setup_s * tg.size / n)
        ks.append(tg.size)
    secs = float(np.sum(t))
    v = float(np.sum(ks)) / secs
    c = r["counters"]
    pairs = c["pairs_local"] + c["pairs_image"]
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs * 1e3 / len(t), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, p, n),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "setup once: tree, multipoles and walks of all %d particles on %d host "
                                       "threads (%.2f s); each step: forces of %d particles (8 runs of whole "
                                       "leaves in tree order) plus the setup's share for them; the reference's "
                                       "algorithm restated in C and pinned bit-exact to its sources (which are "
                                       "not on this host)" % (n, nthreads, setup_s, k)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": r["times"], "sample_particles_per_step": k,
            "counters": {kk: c[kk] for kk in ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "nleaf",
                                              "nnode", "n_p2p_ext", "n_m2l_ext", "pairs_local", "pairs_image")},
            "pairs_per_particle": pairs / n}
    print(json.dumps(line))


def list_digest(t, s, im):
    """SHA-256 of a list's (target, source, image) entries as a sorted multiset."""
    import hashlib

    key = (t.astype(np.int64) << 34) | (s.astype(np.int64) << 5) | im.astype(np.int64)
    key.sort()
    return hashlib.sha256(key.tobytes()).hexdigest()


PARITY_COUNTERS = ("nleaf", "nnode", "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "n_p2p_ext",
                   "n_m2l_ext", "pairs_local", "pairs_image")


def parity_leg(fp, pos, p, tgt, acc64_tgt, acc32_tgt, nthreads):
    """The GPU pass against the oracle's restatement (pinned bit for bit to
    the reference's sources) on the same input and leaf size, outside the
    timed region: tree and walk counters, the tree-order permutation, every
    interaction list as a multiset, and the FP64 accelerations of the target
    subset (relative bar 1e-10).  fp holds the last FP64 pass (lists kept)."""
    import hashlib

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    t0 = time.time()
    port = oracle.PortOracle()
    r = port.run_sample(pos, p, tgt, nthreads=nthreads, lists=True, perm=True)
    gc = fp.counters()
    oc = r["counters"]
    counts = {k: [int(gc[k]), int(oc[k])] for k in PARITY_COUNTERS}
    gperm = fp.perm()
    lists = {}
    glists = fp.lists()
    for kind, (t, s, im) in r["lists"].items():
        lists[kind] = list_digest(*glists[kind]) == list_digest(t, s, im)
    a_ref = r["acc"]
    nref = np.maximum(np.linalg.norm(a_ref, axis=1), 1e-300)
    e64 = np.linalg.norm(acc64_tgt - a_ref, axis=1) / nref
    e32 = np.linalg.norm(acc32_tgt - a_ref, axis=1) / nref
    return {"oracle": "the C restatement of the reference's pass (oracle/photons_oracle.c), bit-identical to the "
                      "reference's compiled sources on the golden inputs; %d host threads" % nthreads,
            "counts_equal": all(a == b for a, b in counts.values()), "counters_gpu_oracle": counts,
            "perm_equal": bool(np.array_equal(gperm, r["perm"])),
            "perm_sha256": hashlib.sha256(np.ascontiguousarray(gperm, np.int32).tobytes()).hexdigest(),
            "lists_equal": lists,
            "fp64_max_rel": float(e64.max()), "fp64_bar": 1e-10, "fp64_ok": bool(e64.max() <= 1e-10),
            "fp32_vs_oracle_median": float(np.median(e32)), "fp32_vs_oracle_p99": float(np.percentile(e32, 99)),
            "targets": int(tgt.size), "oracle_times_s": r["times"], "seconds": time.time() - t0}


def kdk_measure(ph, fp, torch, stream, dpos, dacc, n, p, steps, pflags=0):
    """Device-resident kick-drift-kick steps at a = 0.5 -> 0.505 (the
    reference's kick_loga / drift_loga factors, G = 43007.105732), and the
    kick and drift kernels alone against the measured HBM copy bandwidth."""
    om, ox, G = 0.3, 0.7, 43007.105732
    la, lb = math.log(0.5), math.log(0.505)
    dkh = 0.5 * ph.kick_loga(om, ox, la, lb) * G
    dd = ph.drift_loga(om, ox, la, lb)
    pos = dpos.clone()
    acc = dacc.clone()
    vel = torch.zeros_like(pos)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    fp.kdk_step_device(pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), n, p, dkh, dd, precision=ph.FP32_SPLIT,
                       flags=pflags)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fp.kdk_step_device(pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), n, p, dkh, dd, precision=ph.FP32_SPLIT,
                           flags=pflags)
    e1.record(stream)
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / steps
    s = stream.cuda_stream
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        ph.kick(n, vel.data_ptr(), acc.data_ptr(), 1e-9, s)
    e1.record(stream)
    torch.cuda.synchronize()
    kick_ms = e0.elapsed_time(e1) / reps
    e0.record(stream)
    for _ in range(reps):
        ph.drift(n, pos.data_ptr(), vel.data_ptr(), 1e-9, p["boxsize"], s)
    e1.record(stream)
    torch.cuda.synchronize()
    drift_ms = e0.elapsed_time(e1) / reps
    # PM long-range force on the configuration's mesh, and the step with both halves
    import ctypes as C
    nside = int(round(p["boxsize"] / (p["rs"] / 1.25)))
    acc_pm = torch.zeros_like(pos)
    prm = ph.make_params(p, ph.FP64, 0, ph.F_DEVICE_IO)

    def pm():
        rc = fp.lib.photons_pm_force(fp.h, C.byref(prm), nside, n, C.c_void_p(pos.data_ptr()),
                                     C.c_void_p(acc_pm.data_ptr()))
        if rc:
            raise RuntimeError(fp.lib.photons_gpu_error().decode())

    pm()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        pm()
    e1.record(stream)
    torch.cuda.synchronize()
    pm_ms = e0.elapsed_time(e1) / reps
    fp.kdk_step_pm_device(pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), acc_pm.data_ptr(), n, p, nside, dkh, dd,
                          flags=pflags)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fp.kdk_step_pm_device(pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), acc_pm.data_ptr(), n, p, nside, dkh, dd,
                              flags=pflags)
    e1.record(stream)
    torch.cuda.synchronize()
    step_pm_ms = e0.elapsed_time(e1) / steps
    # the same steps keeping the state in tree order (the reference's part[]
    # ordering): each build starts from the previous step's tree order
    opos, ovel, oacc, opm = pos.clone(), vel.clone(), acc.clone(), acc_pm.clone()
    oids = torch.arange(n, dtype=torch.int64, device=pos.device)

    def ordered(with_pm):
        fp.kdk_step_ordered_device(opos.data_ptr(), ovel.data_ptr(), oacc.data_ptr(), oids.data_ptr(), n, p, dkh, dd,
                                   precision=ph.FP32_SPLIT, flags=pflags, nside=nside if with_pm else 0,
                                   acc_pm_ptr=opm.data_ptr())

    ordered(False)
    ordered(False)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        ordered(False)
    e1.record(stream)
    torch.cuda.synchronize()
    step_ordered_ms = e0.elapsed_time(e1) / steps
    e0.record(stream)
    for _ in range(steps):
        ordered(True)
    e1.record(stream)
    torch.cuda.synchronize()
    step_ordered_pm_ms = e0.elapsed_time(e1) / steps
    bytes_each = 3 * n * 24  # read two arrays, write one, 3n doubles
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs")
    out = {"step_ms": step_ms, "step_with_pm_ms": step_pm_ms, "pm_ms": pm_ms, "pm_mesh": nside,
           "step_tree_order_ms": step_ordered_ms, "step_tree_order_with_pm_ms": step_ordered_pm_ms,
           "a": [0.5, 0.505], "dkh": dkh, "dd": dd,
           "kick_ms": kick_ms, "drift_ms": drift_ms,
           "kick_gbs": bytes_each / (kick_ms * 1e-3) / 1e9, "drift_gbs": bytes_each / (drift_ms * 1e-3) / 1e9,
           "bytes_per_kernel": bytes_each}
    if hbm:
        out["kick_frac_of_measured_hbm"] = out["kick_gbs"] / hbm
        out["drift_frac_of_measured_hbm"] = out["drift_gbs"] / hbm
    return out


def run_boxes_bench(args):
    """Many independent periodic boxes (70% Plummer a = 0.05 L_b + 30% uniform,
    N_b log-uniform in [16^3, 64^3], L_b in [20, 100], seed 4) in one batched
    pass, against looping over the boxes one pass at a time (FP32 and FP64)."""
    import ctypes as C
    import torch
    import __graft_entry__ as g

    ph = g.load_package()
    from photons_gb300 import ics

    torch.cuda.set_device(0)
    leaf = args.maxleaf or 32
    boxes = [(pos, dict(p, maxleaf=leaf)) for pos, p in ics.plummer_boxes(nbox=256, seed=4)]
    counts = np.array([b[0].shape[0] for b in boxes], np.int32)
    offs = np.concatenate([[0], np.cumsum(counts)])
    n = int(offs[-1])
    pos = np.ascontiguousarray(np.concatenate([b[0] for b in boxes]))
    fp = ph.ForcePass(0)
    stream = torch.cuda.current_stream()
    fp.set_stream(stream.cuda_stream)
    dpos = torch.from_numpy(pos).cuda()
    dacc = torch.empty_like(dpos)
    lib = fp.lib

    def params(prec):
        arr = (ph.Params * len(boxes))()
        for i, (_, p) in enumerate(boxes):
            arr[i] = ph.make_params(p, prec, 0, ph.F_DEVICE_IO)
        return arr

    p32, p64 = params(ph.FP32_SPLIT), params(ph.FP64)
    cptr = counts.ctypes.data_as(C.POINTER(C.c_int))

    def batched(prm):
        rc = lib.photons_force_pass_boxes(fp.h, len(boxes), prm, cptr, C.c_void_p(dpos.data_ptr()),
                                          C.c_void_p(dacc.data_ptr()))
        if rc:
            raise RuntimeError(lib.photons_gpu_error().decode())

    # the loop gives each box its own context, so each keeps its captured pass
    ctxs = [ph.ForcePass(0) for _ in boxes]
    for cx in ctxs:
        cx.set_stream(stream.cuda_stream)

    def loop(prec):
        for i, (_, p) in enumerate(boxes):
            ctxs[i].run_device(dpos.data_ptr() + 24 * int(offs[i]), dacc.data_ptr() + 24 * int(offs[i]),
                               int(counts[i]), p, precision=prec)

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for _ in range(max(3, args.warmup)):
        batched(p32)
    sampler = ClockSampler(0)
    sampler.start()
    launches0 = lib.photons_launch_count()
    ms = timed(lambda: batched(p32), args.steps)
    launches = lib.photons_launch_count() - launches0
    clocks = sampler.stop()
    t = fp.timings()
    c = fp.counters()
    pairs = c["pairs_local"] + c["pairs_image"]
    acc32 = dacc.cpu().numpy()
    loop(ph.FP32_SPLIT)
    ms_loop32 = timed(lambda: loop(ph.FP32_SPLIT), 1)
    batched(p64)
    ms64 = timed(lambda: batched(p64), 1)
    acc64 = dacc.cpu().numpy()
    loop(ph.FP64)
    ms_loop64 = timed(lambda: loop(ph.FP64), 1)
    # errors: FP32 vs FP64 everywhere, and both vs the direct sum on ~40 particles per box
    e = rel_err(acc32, acc64)
    rng = np.random.default_rng(7)
    a32, a64 = [], []
    for i, (bp, p) in enumerate(boxes):
        tg = rng.choice(counts[i], min(40, counts[i]), replace=False).astype(np.int32)
        ds = ph.direct_sum(bp, p, tg)
        a32.append(rel_err(acc32[offs[i] + tg], ds))
        a64.append(rel_err(acc64[offs[i] + tg], ds))
    a32, a64 = np.concatenate(a32), np.concatenate(a64)
    # end to end: host arrays through the batched C-ABI call
    hpos = ph.host_array(pos.shape)  # pinned by the library (cudaHostAlloc)
    hpos[:] = pos
    hacc = ph.host_array(pos.shape)
    hp32 = (ph.Params * len(boxes))()
    for i, (_, p) in enumerate(boxes):
        hp32[i] = ph.make_params(p, ph.FP32_SPLIT, 0, 0)

    def e2e():
        rc = lib.photons_force_pass_boxes(fp.h, len(boxes), hp32, cptr, C.c_void_p(hpos.ctypes.data),
                                          C.c_void_p(hacc.ctypes.data))
        if rc:
            raise RuntimeError(lib.photons_gpu_error().decode())

    e2e()
    t0 = time.time()
    for _ in range(3):
        e2e()
    e2e_ms = (time.time() - t0) * 1e3 / 3
    peak = ph.fp32_fma_peak(8192)
    achieved = FLOPS_PER_PAIR * pairs / (t["p2p"] * 1e-3) / 1e12
    line = {
        "metric": "particle-forces/s, 256 independent boxes in one batched pass", "value": n / (ms * 1e-3),
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "boxes256", "n": n, "nbox": len(boxes), "maxleaf": leaf,
                   "n_box_min": int(counts.min()), "n_box_max": int(counts.max()),
                   "precision": "fp32-split", "l2": "inputs larger than L2 (positions %.0f MB)" % (n * 24 / 1e6)},
        "roofline": {"bound": "fp32", "kernel": "k_p2p_split_packed", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "p2p_ms": t["p2p"]},
        "e2e": {"value": n / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": n * 24, "d2h_bytes_per_step": n * 24,
                "ms_per_step": e2e_ms},
        "gpu_launches": int(launches), "clocks": clocks,
        "phases_ms": t,
        "boxes": {"batched_fp32_ms": ms, "loop_fp32_ms": ms_loop32, "batched_fp64_ms": ms64,
                  "loop_fp64_ms": ms_loop64, "speedup_batched_fp32_vs_loop_fp64": ms_loop64 / ms,
                  "speedup_batched_vs_loop_fp32": ms_loop32 / ms},
        "errors": {"precision_fp32_vs_fp64gpu": {"median": float(np.median(e)), "p99": float(np.percentile(e, 99))},
                   "algorithmic_vs_direct_sum": {"fp32_median": float(np.median(a32)),
                                                 "fp32_p99": float(np.percentile(a32, 99)),
                                                 "fp64_median": float(np.median(a64)),
                                                 "sample": "%d particles, 40 per box" % a32.size}},
    }
    print(json.dumps(line))


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.workload == "boxes256":
        run_boxes_bench(args)
        return
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as g

    ph = g.load_package()
    pos, p = workload(args.nside, args.maxleaf or 16, seed_offset=rank, name=args.workload)
    n = pos.shape[0]
    torch.cuda.synchronize()
    free0, total_hbm = torch.cuda.mem_get_info()
    fp = ph.ForcePass(local)
    tuned = None
    tune = None
    # the autotuner's kernel choice (PHOTONS_F_ONE_WAY, or the mutual kernel's
    # build and staging), else the caller's
    pflags = args.pass_flags
    if not args.maxleaf:
        best, table, pflags = ph.autotune_leaf(fp, pos, p, error_bound=args.error_bound)
        best = broadcast_from_rank0(best, dist, "cuda")  # every replica runs rank 0's choice
        pflags = broadcast_from_rank0(pflags, dist, "cuda")
        p["maxleaf"] = best
        one_way = bool(pflags & ph.F_ONE_WAY) or best < 48
        tune = {"chosen_maxleaf": best,
                "chosen_kernel": "one-way" if one_way else "mutual shape %d%s" % (
                    (pflags >> 8) & 15, ", sources by TMA bulk copies" if pflags & ph.F_P2P_BULK else ""),
                "chosen_flags": pflags,
                "error_bound_median": args.error_bound, "candidates": table,
                "score": "fastest pass with median error vs the FP64 direct sum <= bound (2000-particle sample)"}
        # the candidates' smaller leaves grew the context's list pools: time the
        # chosen configuration in a fresh context sized for it alone.  The
        # tuning context stays allocated until the host-buffer leg has run:
        # on GB300 hosts, freeing its buffers was followed by seconds of
        # host-link copies slowed ten-fold for ~20 ms every ~0.5 s (device
        # work unaffected), which a serving process that keeps its context
        # never sees.
        tuned = fp
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        fp = ph.ForcePass(local)
    stream = torch.cuda.current_stream()
    fp.set_stream(stream.cuda_stream)
    dpos = torch.from_numpy(pos).to("cuda")
    dacc = torch.empty_like(dpos)
    torch.cuda.synchronize()

    def step():
        fp.run_device(dpos.data_ptr(), dacc.data_ptr(), n, p, precision=ph.FP32_SPLIT, flags=pflags)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    # end to end through the C ABI: pinned host buffers in, host buffers out.
    # Timed before the device-buffer loop: on GB300 hosts, host-link copies
    # timed after it ran ten-fold slower for ~20 ms every ~0.5 s in some
    # runs (device work unaffected), which this order did not show.
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    hp = ph.host_array(pos.shape)  # pinned by the library (cudaHostAlloc)
    hp[:] = pos
    ha = ph.host_array(pos.shape)
    for _ in range(3):  # the host-buffer pass is captured as its own graph on first use
        fp.run(hp, p, precision=ph.FP32_SPLIT, flags=pflags, out=ha)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    esteps = max(5, args.steps)
    e2e_parts = []
    e0.record(stream)
    t0 = time.perf_counter()
    for _ in range(esteps):
        t1 = time.perf_counter()
        fp.run(hp, p, precision=ph.FP32_SPLIT, flags=pflags, out=ha)
        wall_ms = (time.perf_counter() - t1) * 1e3
        t = fp.timings()  # CUDA events of this pass: copy in, device part, copy out
        e2e_parts.append((t["upload"], t["total"] - t["upload"] - t["download"], t["download"], t["total"], wall_ms))
    loop_ms = (time.perf_counter() - t0) * 1e3
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    # each call returns after its pass has finished, so the loop's wall time
    # is the whole job's time for esteps passes (max over ranks)
    e2e_ms = max_over_ranks(max(e0.elapsed_time(e1), loop_ms) / esteps, dist, "cuda")
    e2e_split = dict(zip(("h2d_ms", "device_ms", "d2h_ms", "events_total_ms", "host_call_ms"),
                         (float(np.median([q[i] for q in e2e_parts])) for i in range(5))))
    e2e_split["each"] = {"h2d_ms": [round(q[0], 3) for q in e2e_parts], "device_ms": [round(q[1], 3) for q in e2e_parts],
                         "d2h_ms": [round(q[2], 3) for q in e2e_parts], "host_call_ms": [round(q[4], 3) for q in e2e_parts]}
    hbm_used = free0 - torch.cuda.mem_get_info()[0]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    launches0 = ph.load_library().photons_launch_count()
    p2p_ms, phase = [], []
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
        t = fp.timings()
        p2p_ms.append(t["p2p"])
        phase.append(t)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = ph.load_library().photons_launch_count() - launches0
    clocks = sampler.stop() if sampler else None
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist, "cuda")
    counters = fp.counters()
    pairs = counters["pairs_local"] + counters["pairs_image"]
    value = n * world / (ms * 1e-3)

    acc32 = ha.copy()
    if tuned is not None:
        tuned.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # roofline of the dominant kernel (P2P, FP32 pipe).  From leaf 48 the
    # mutual kernel evaluates each symmetric leaf pair (local or image) once
    # for both leaves, so the pairs it evaluates are about half the
    # reference's pair set (self pairs, about 1 %, are counted at half here
    # although they are evaluated in full)
    mutual = p["maxleaf"] >= 48 and not (pflags & ph.F_ONE_WAY) and \
        os.environ.get("PHOTONS_P2P_KERNEL", "mutual") == "mutual"
    kernel = "k_p2p_mutual" if mutual else "k_p2p_split_packed"
    evaluated = pairs // 2 if mutual else pairs
    peak = ph.fp32_fma_peak(8192)
    t_p2p = float(np.mean(p2p_ms))
    achieved = FLOPS_PER_PAIR * pairs / (t_p2p * 1e-3) / 1e12
    traffic = TRAFFIC_PER_LAUNCH_256.get(kernel) if (args.nside == 256 and args.workload == "zeldovich256") else None
    extra = {}
    kdk = kdk_measure(ph, fp, torch, stream, dpos, dacc, n, p, args.steps, pflags) if args.kdk else None
    rng = np.random.default_rng(7)
    tgt = rng.choice(n, min(n, 10000), replace=False).astype(np.int32)
    ds = ph.direct_sum(pos, p, tgt)
    a32 = rel_err(acc32[tgt], ds)
    extra["errors"] = {"algorithmic_vs_direct_sum_10k": {
        "fp32_median": float(np.median(a32)), "fp32_p99": float(np.percentile(a32, 99)),
        "direct_sum": "FP64 GPU, untruncated erfc kernel, all sources within 2 rcut, minimum image"}}
    if not args.no_fp64:
        fp.run_device(dpos.data_ptr(), dacc.data_ptr(), n, p, precision=ph.FP64)
        torch.cuda.synchronize()
        t64 = fp.timings()
        acc64 = np.empty_like(pos)
        e0.record(stream)
        fp.run(pos, p, precision=ph.FP64, out=acc64, flags=ph.F_KEEP_LISTS)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        if not args.no_parity:
            extra["parity"] = parity_leg(fp, pos, p, tgt, acc64[tgt], acc32[tgt], os.cpu_count() or 1)
        e = rel_err(acc32, acc64)
        a64 = rel_err(acc64[tgt], ds)
        peak64 = ph.fp64_fma_peak()
        c64 = fp.counters()
        pairs64 = c64["pairs_local"] + c64["pairs_image"]
        ach64 = FLOPS_PER_PAIR * pairs64 / (t64["p2p"] * 1e-3) / 1e12
        # FP64 passes evaluate each symmetric leaf pair once (k_p2p_mutual64)
        # unless PHOTONS_F_ONE_WAY: about half the reference's pair set
        eval64 = pairs64 // 2
        ev_tf64 = FLOPS_PER_PAIR * eval64 / (t64["p2p"] * 1e-3) / 1e12
        extra["fp64_gpu"] = {"value": n / (ms64 * 1e-3), "ms_per_pass": ms64, "p2p_ms": t64["p2p"],
                             "speedup_fp32_over_fp64": ms64 / ms,
                             "roofline": {"bound": "fp64", "kernel": "k_p2p_mutual64", "achieved": ach64,
                                          "peak": peak64, "unit": "TFLOP/s", "frac": ach64 / peak64,
                                          "peak_source": "DFMA probe measured in this run",
                                          "work": "%d flops/pair x %d pairs (the reference's pair set, both "
                                                  "directions)" % (FLOPS_PER_PAIR, pairs64),
                                          "evaluated_pairs": eval64, "evaluated_tflops": ev_tf64,
                                          "evaluated_frac": ev_tf64 / peak64,
                                          "timed": "the whole P2P phase (list sort, pairing, slots, pair kernel, "
                                                   "reaction gather) between CUDA events"}}
        extra["errors"] = {
            "precision_fp32_vs_fp64gpu": {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)),
                                          "max": float(e.max())},
            "algorithmic_vs_direct_sum_10k": {
                "fp32_median": float(np.median(a32)), "fp32_p99": float(np.percentile(a32, 99)),
                "fp64_median": float(np.median(a64)), "fp64_p99": float(np.percentile(a64, 99)),
                "direct_sum": "FP64 GPU, untruncated erfc kernel, all sources within 2 rcut, minimum image"}}
    cpu = None if args.no_cpu else cpu_baseline(maxleaf=p["maxleaf"], name=args.workload)

    tmean = {k: float(np.mean([t[k] for t in phase])) for k in phase[0]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, p, n),
        "precision": "fp32-split (fp64 positions and centre differences)",
        "parallelism": "replicas" if world > 1 else "single GPU",
        "roofline": {"bound": "fp32", "kernel": kernel, "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "FFMA probe measured in this run (MEASURED_PEAKS.json holds no FP32 figure)",
                     "work": "%d flops/pair x %d pairs per launch (the reference's pair set, both directions)"
                             % (FLOPS_PER_PAIR, pairs),
                     "evaluated_pairs": evaluated, "evaluated_tflops": FLOPS_PER_PAIR * evaluated / (t_p2p * 1e-3) / 1e12,
                     "evaluated_frac": FLOPS_PER_PAIR * evaluated / (t_p2p * 1e-3) / 1e12 / peak,
                     "p2p_ms": t_p2p,
                     "timed": "the whole P2P phase between CUDA events on the pass stream (for the mutual kernel "
                              "also its list sort, pairing, slot assignment and reaction gather), so achieved "
                              "is a lower bound for the kernel alone"},
        "cpu_baseline": cpu,
        "e2e": {"value": n * world / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": n * 24 * world,
                "d2h_bytes_per_step": n * 24 * world, "ms_per_step": e2e_ms, "steps": esteps, "split_median": e2e_split,
                "path": "photons_force_pass with pinned host buffers (copies on the pass stream)"},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "phases_ms": tmean,
        "counters": {k: counters[k] for k in ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "nleaf",
                                              "nnode", "pairs_local", "pairs_image", "depth")},
        "pairs_per_particle": pairs / n,
        "hbm": {"device_bytes_used": int(hbm_used), "device_bytes_total": int(total_hbm),
                "what": "device memory taken by the pass context and the resident position/acceleration "
                        "buffers after warm-up (cudaMemGetInfo difference)"},
    }
    if kdk:
        line["kdk"] = kdk
    line.update(extra)
    if tune:
        line["autotune"] = tune
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
