"""The multi-GPU (replica) path on CPU: world size 2 over gloo, 127.0.0.1.

Each rank takes its share of an ensemble's disks and reports its units and seconds; the job
rate is all units over the slowest rank's time, as bench.py computes it for N GPUs."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from redgb.replicas import job_rate, max_over_ranks, shard, sum_over_ranks


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard(range(65, 65 + 7), rank, world)
        units = float(len(mine))          # e.g. disk-years done by this rank
        secs = 1.0 + rank                  # the ranks' timed regions differ
        rate, total, slowest = job_rate(units, secs, dist)
        out.put((rank, mine, rate, total, slowest, max_over_ranks(rank, dist), sum_over_ranks(rank, dist)))
    finally:
        dist.destroy_process_group()


def test_shard_covers_everything_once():
    items = list(range(100))
    parts = [shard(items, r, 3) for r in range(3)]
    assert sum(parts, []) == items
    assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    assert shard(items, 0, 1) == items


def test_two_ranks_over_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, rate0, tot0, slow0, mx0, sm0), (r1, m1, rate1, tot1, slow1, mx1, sm1) = res
    assert m0 + m1 == list(range(65, 72)) and not set(m0) & set(m1)
    assert tot0 == tot1 == 7.0 and slow0 == slow1 == 2.0
    assert rate0 == rate1 == pytest.approx(3.5)
    assert mx0 == mx1 == 1.0 and sm0 == sm1 == 1.0


def test_single_process_needs_no_collective():
    rate, units, secs = job_rate(10.0, 4.0, None)
    assert (rate, units, secs) == (2.5, 10.0, 4.0)
