"""Multi-rank logic on CPU with gloo (world size 2).

Cloths are independent units, so the multi-GPU form of the batched solve is
a partition of the cloths over ranks with no data-path exchange; the only
collectives are the host-side ones bench.py uses (barrier, max of the timed
region over ranks, gather of per-rank statistics).  This test runs those on
two gloo ranks and checks the partition: disjoint, complete, balanced.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "cloth-cuda_gb300"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import scenes
    rng = np.random.default_rng(0)
    sizes = rng.integers(17, 130, 512) ** 2          # vertex counts of a 512-cloth batch
    mine = scenes.shard(sizes, rank, world)
    # per-rank "timed region": the max over ranks is what the bench reports
    t = torch.tensor([float(len(mine)) + rank * 0.25])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    counts = [None] * world
    dist.all_gather_object(counts, (mine, int(sizes[mine].sum())))
    dist.barrier()
    if rank == 0:
        np.save(os.path.join(out_dir, "shards.npy"), np.array([counts, float(t.item())], dtype=object),
                allow_pickle=True)
    dist.destroy_process_group()


def test_two_rank_partition_and_max_timing(tmp_path):
    world = 2
    port = _free_port()
    mp.start_processes(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    counts, tmax = np.load(tmp_path / "shards.npy", allow_pickle=True)
    idx = sorted(i for mine, _ in counts for i in mine)
    assert idx == list(range(512))                       # every cloth exactly once
    verts = [v for _, v in counts]
    assert abs(verts[0] - verts[1]) / sum(verts) < 0.05  # balanced by vertices
    assert tmax == max(len(mine) + r * 0.25 for r, (mine, _) in enumerate(counts))


def _leaving_worker(rank, world, port, out_dir):
    # rank 1 leaves between steps (after the first step's collective); rank 0
    # must learn of it at its next collective through the process-group
    # timeout instead of waiting forever
    import datetime
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=3))
    t = torch.tensor([1.0])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)          # step 1: both ranks
    if rank == 1:
        return                                      # leaves without a goodbye
    outcome = "completed"
    try:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)      # step 2: the peer is gone
    except Exception as e:                           # gloo raises on timeout / closed peer
        outcome = "error: " + type(e).__name__
    with open(os.path.join(out_dir, "outcome.txt"), "w") as f:
        f.write(outcome)


def test_departed_rank_is_reported_not_awaited(tmp_path):
    world = 2
    port = _free_port()
    ctx = mp.start_processes(_leaving_worker, args=(world, port, str(tmp_path)), nprocs=world, join=False,
                             start_method="spawn")
    while not ctx.join(timeout=30):
        pass
    outcome = (tmp_path / "outcome.txt").read_text()
    assert outcome.startswith("error"), outcome
