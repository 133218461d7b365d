"""Multi-GPU form of the bench: independent replicas, one job per rank, no
collective in the data path; the timing is the max over ranks and the
throughput the sum of all ranks' paths.  Checked on CPU with two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist = bench.init_dist("gloo")
    assert bench.dist_info() == (rank, world, rank)
    local_time = 1.0 + rank  # rank 1 is the slow one
    t = bench.reduce_max(local_time, dist)
    paths = bench.reduce_sum(100.0 * (rank + 1), dist)
    seeds = [None] * world
    dist.all_gather_object(seeds, bench.replica_seed(rank))
    out[rank] = (t, paths, seeds)
    dist.destroy_process_group()


def test_two_rank_replicas_max_time_and_distinct_jobs():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0  # max over ranks
    assert res[0][1] == res[1][1] == 300.0
    assert len(set(res[0][2])) == world  # each rank runs its own job


def test_single_process_needs_no_group():
    import bench

    assert bench.init_dist("gloo") is None or os.environ.get("WORLD_SIZE", "1") != "1"
    assert bench.reduce_max(3.5, None) == 3.5
