"""The multi-rank host logic of bench.py on CPU, two gloo ranks: the path has
no exchange step, so N ranks run N independent replica chains (distinct
seeds), and the job's time is the slowest rank's (max over ranks), its rate
the trajectories of all ranks over that time."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms_local = [40.0, 55.0][rank]
        ms, rate = bench.job_time_and_rate(ms_local, 10, world, dist)
        out.put((rank, bench.replica_seed(rank), ms, rate))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replica_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    seeds = [r[1] for r in res]
    assert seeds[0] != seeds[1]
    for _, _, ms, rate in res:
        assert ms == 55.0
        assert rate == pytest.approx(2 * 10 / 0.055)


def test_single_rank_has_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.job_time_and_rate(20.0, 5, 1) == (20.0, pytest.approx(250.0))
