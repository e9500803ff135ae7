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


def _cube_work():
    from axia_gpu import meshgen, replicas
    cubes = meshgen.cube_family(count=64, lo=10, hi=40)
    # node blocks of a structured C3D8 grid with m = n + 1 nodes per edge: (3m - 2)^3
    return [replicas.mesh_work(c.n_nodes, (3 * (c.shape[0] + 1) - 2) ** 3) for c in cubes]


def _partition_rank(rank, world, port, out):
    import torch.distributed as dist

    from axia_gpu import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        work = _cube_work()
        mine = replicas.partition_meshes(work, world)[rank]
        got = [None] * world
        dist.all_gather_object(got, mine)  # what every rank will solve
        out[rank] = (got, sum(work[k] for k in mine))
    finally:
        dist.destroy_process_group()


def test_mesh_partition_two_ranks_gloo():
    """The 64 independent cubes split over two ranks (gloo on CPU): every rank
    derives the same split, every mesh is solved by exactly one rank, and the
    ranks' estimated work is within 10 % of each other."""
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_partition_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got0, got1 = out[0][0], out[1][0]
    assert got0 == got1
    flat = sorted(k for part in got0 for k in part)
    assert flat == list(range(64))
    loads = [out[r][1] for r in range(world)]
    assert max(loads) <= 1.10 * min(loads), loads


@pytest.mark.parametrize("world", [1, 3, 4, 8])
def test_mesh_partition_covers_and_balances(world):
    from axia_gpu import replicas
    work = _cube_work()
    parts = replicas.partition_meshes(work, world)
    assert sorted(k for p in parts for k in p) == list(range(64))
    loads = [sum(work[k] for k in p) for p in parts]
    assert max(loads) <= 1.10 * (sum(loads) / world) + max(work), loads
