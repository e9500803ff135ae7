"""Replica timing on CPU with world_size 2 over gloo (the N>1 path of the
bench: independent replicas, job time = max over ranks, throughput = all
ranks' units over it)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    from axia_gpu import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, lr, w = replicas.world()
        assert (r, lr, w) == (rank, rank, world)
        seconds = 2.0 if rank == 0 else 5.0  # the slow rank sets the job time
        thr, job_s = replicas.job_throughput(1000.0, seconds, dist)
        out[rank] = (thr, job_s)
    finally:
        dist.destroy_process_group()


def test_job_throughput_two_ranks_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        thr, job_s = out[r]
        assert job_s == pytest.approx(5.0)
        assert thr == pytest.approx(2 * 1000.0 / 5.0)


def test_job_throughput_single_process():
    from axia_gpu import replicas
    thr, job_s = replicas.job_throughput(300.0, 1.5)
    assert job_s == 1.5 and thr == pytest.approx(200.0)
