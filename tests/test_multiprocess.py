"""The N-process host logic of bench.py on CPU with gloo (world size 2):
timings are the slowest rank's, replicas render their own frames (weak
scaling) and the whole-job value is per frame over all ranks.  Multi-GPU is
replicas only, so this is all the cross-rank logic there is."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        slowest = bench.max_over_ranks(10.0 + rank, world, torch.device("cpu"))
        bench.set_workload(1000, 64, 48)
        xyz = bench.make_scene(seed=rank)["xyz"]  # run_ours seeds each replica by its rank
        out[rank] = (slowest, bench.aggregate_ms_per_frame(slowest, world), float(xyz.sum()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_ranks_take_the_slowest_timing_and_aggregate_frames():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 11.0            # max over ranks
    assert res[0][1] == res[1][1] == 11.0 / world    # ms per frame over all replicas
    assert res[0][2] != res[1][2]                    # each replica renders its own scene


def test_single_process_is_the_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1, torch.device("cpu")) == 3.5
    assert bench.aggregate_ms_per_frame(3.5, 1) == 3.5
