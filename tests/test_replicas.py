"""Multi-GPU form: replicas only.  Every rank runs its own frames and no
collective touches the data path; the bench reduces only its timing, taking
the slowest rank's time and the frames of all ranks.  This checks that
reduction with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    import torch
    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took 10 + 5 r ms for 8 + r frames
    ms, units = bench.whole_job(10.0 + 5.0 * rank, 8 + rank, world, torch.device("cpu"))
    out.put((rank, ms, units))
    dist.barrier()
    dist.destroy_process_group()


def test_whole_job_takes_slowest_rank_and_all_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 15.0, 17), (1, 15.0, 17)]


def test_whole_job_single_rank_has_no_collective():
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    assert bench.whole_job(12.5, 8, 1, None) == (12.5, 8)
