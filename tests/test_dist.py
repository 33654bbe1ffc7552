"""The multi-rank path of bench.py on CPU: two gloo ranks on 127.0.0.1.

The force pass does not shard (each rank runs an independent box, weak
scaling, no collective on the data path), so what runs across ranks is the
bench's plumbing: the slowest rank's time, rank 0's leaf size on every
rank, a different box per rank, and the reference arm running on rank 0
alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _ranks(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    import numpy as np

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = {}
        # the slowest rank's step time, on every rank
        res["max_ms"] = bench.max_over_ranks(3.0 + 2.0 * rank, dist)
        # rank 0's autotuned leaf size reaches every replica
        res["leaf"] = bench.broadcast_from_rank0(32 if rank == 0 else 64, dist)
        # each replica's box differs (seed 3 + rank)
        pos, p = bench.workload(8, 16, seed_offset=rank)
        digest = torch.tensor([float(np.abs(pos).sum())], dtype=torch.float64)
        allv = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(allv, digest)
        res["distinct_boxes"] = len({float(v.item()) for v in allv}) == world
        res["n"] = int(pos.shape[0])
        with open(os.path.join(out, "rank%d.json" % rank), "w") as f:
            json.dump(res, f)
    finally:
        dist.destroy_process_group()


def test_bench_rank_plumbing_gloo(tmp_path):
    world = 2
    mp.start_processes(_ranks, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    got = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    for g in got:
        assert g["max_ms"] == 5.0
        assert g["leaf"] == 32
        assert g["distinct_boxes"]
        assert g["n"] == 8 ** 3


def test_reference_arm_runs_on_rank0_only(tmp_path):
    """Under torchrun only rank 0 times the reference's CPU path and prints
    its line; the other ranks exit 0 without work."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
