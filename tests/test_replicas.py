"""bench.py's multi-GPU form is replicas only (independent sources per rank, no data-path
collective): its timing is the slowest rank's, aggregated with one all-reduce.  Two gloo ranks
on the CPU check that aggregation and the whole-job value."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dev, wall = bench.max_over_ranks([1.0 + rank, 3.0 - rank], dist, "cpu")
        out[rank] = (dev, wall, bench.replica_gteps(1e9, 4, world, dev))
    finally:
        dist.destroy_process_group()


def test_two_rank_max_and_value():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of this (threaded) process
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        dev, wall, val = res[r]
        assert dev == 2.0 and wall == 3.0   # the slowest rank of each
        assert val == pytest.approx(1e9 * 4 * 2 / 2.0 / 1e9)


def test_single_process_identity():
    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
