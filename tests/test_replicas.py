"""The multi-GPU form is replicas: each rank meshes its own seeded world and the benchmark reduces
timing (max over ranks) and work (sum over ranks) with one collective at the end, none on the data
path. This runs that host logic as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    from hypercraft_gb300 import worldgen
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each replica's own world (the seed offset bench.make_world uses)
        seed = worldgen.WORLD_SEED + 7919 * rank
        w = worldgen.generate(3, 3, 3, (-1, -1, -1), seed=seed, caves=True, air_ring=False)
        chunks = len(w.meshable())
        t = 1.0 + rank  # this rank's timed region
        out[rank] = (bench.max_over_ranks(t, world), bench.sum_over_ranks(chunks * 5, world), int(w.blocks.sum()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_time_and_work():
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    world, port = 2, _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (t0, n0, s0), (t1, n1, s1) = out[0], out[1]
    assert t0 == t1 == 2.0, "the job's time is the slowest rank's"
    assert n0 == n1 and n0 > 0, "the job's work is the sum over ranks"
    assert s0 != s1, "each replica meshes its own seeded world"
