"""The multi-GPU path of bench.py is replicas: each rank aligns a disjoint shard of scans
against its own copy of the map, and the step time is the slowest rank's. Checked here with
two gloo ranks on the CPU (no GPU, no data-path collective)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        idx = bench.rank_scan_indices(8, rank, world)
        # each rank reports its own timings; the reduction gives every rank the maximum
        mx = bench.max_over_ranks([10.0 + rank, 100.0 - rank], "cpu")
        out[rank] = (idx, mx)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_replicas_shard_and_max_reduce():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    idx0, mx0 = res[0]
    idx1, mx1 = res[1]
    assert not set(idx0) & set(idx1)                       # disjoint shards
    assert sorted(idx0 + idx1) == list(range(2, 2 + 16))   # together: the whole job
    assert mx0 == mx1 == [11.0, 100.0]                     # slowest rank's time on every rank
