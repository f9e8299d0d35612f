"""The benchmark's multi-GPU path is replicas only: each rank advances its own system and the ranks
exchange two scalars (the largest timed-region duration and the atom-steps).  Checked here with
two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, atoms = bench.reduce_over_ranks(10.0 + rank, 9000.0 * 100)
    out[rank] = (ms, atoms)
    dist.destroy_process_group()


def test_two_ranks_take_max_time_and_sum_work():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            ms, atoms = out[r]
            assert ms == 11.0
            assert atoms == 2 * 9000.0 * 100


def test_single_process_is_local():
    import bench
    assert bench.reduce_over_ranks(5.0, 7.0) == (5.0, 7.0)
