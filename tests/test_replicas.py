"""Replicas on several processes (the bench's N > 1 path), on CPU with gloo.

The path does not shard: each GPU runs its own replica and the only
cross-rank operations are a barrier around the timed region and the maximum
of the timed durations.  Two gloo ranks on the host check that plumbing, and
that the reference arm does its work on rank 0 alone.
"""

import os
import socket
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


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        bench.replica_barrier(world)
        mx = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
        ref = bench.reference_arm(None, rank, world) if rank != 0 else "rank0"
        out.put((rank, mx, ref))
        bench.replica_barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_share_only_the_max_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]  # every rank sees the slowest replica
    assert res[1][2] is None  # the reference arm runs on rank 0 only


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    bench.replica_barrier(1)
    assert bench.max_over_ranks(3.5, 1, torch.device("cpu")) == 3.5
