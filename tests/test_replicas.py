"""Replica harness on CPU: two gloo ranks reduce their elapsed times to the maximum and
aggregate the job rate (the path bench.py takes under torchrun with one rank per GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from hexed_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = replicas.max_over_ranks(times[rank])
        dist.barrier()
        out[rank] = (ms, replicas.job_rate(1000., world, ms))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_max_over_ranks_and_rate_with_gloo(world):
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    times = [12.5, 20.0, 7.0][:world]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, times, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(world):
        ms, rate = out[r]
        assert ms == max(times)
        assert rate == pytest.approx(1000. * world / (max(times) / 1e3))


def test_single_process_is_identity():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_rate(10., 1, 1000.) == 10.
