"""The multi-GPU form is replicas only: windows are independent units, so
`bench.py --gpus N` gives every rank its own block of the stream and takes the
slowest rank's time.  These tests run that host logic as two gloo ranks on the
CPU (no GPU, no collective on the data path)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # each rank's step time differs; the job's time is the slowest rank's
        ms = bench.max_over_ranks(torch, 1.5 + rank, world, device="cpu")
        first = bench.replica_first_tuple(rank, 8, 1 << 24)
        gathered = [None] * world
        dist.all_gather_object(gathered, first)
        out.put((rank, ms, first, gathered))
    finally:
        dist.destroy_process_group()


def test_replica_blocks_and_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = [out.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    # the slowest rank's time, on every rank
    assert [r[1] for r in res] == [2.5, 2.5]
    # every rank its own block of the stream: disjoint tuple ranges of 8 windows x 2^24
    firsts = res[0][3]
    assert firsts == [0, 8 << 24] and res[1][3] == firsts


def test_single_rank_needs_no_process_group():
    torch = pytest.importorskip("torch")
    import bench

    assert bench.max_over_ranks(torch, 3.25, 1) == 3.25
    assert bench.replica_first_tuple(0, 8, 1 << 24) == 0
