"""Full-size parity of the batched form: the whole scale world (32 x 8 x 32 = 8,192 chunks) and the
whole mixture world (32 x 16 x 32 = 16,384 chunks) are meshed in one batch, and a seeded random
sample of 512 chunks of each is compared byte for byte with the CPU oracle (the restatement of
client/src/ChunkMeshTask.cpp:41-127). The mixture sample is drawn so that it holds every kind of
chunk, its checkerboard and random-fill chunks included."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SAMPLE = 512


def _world(kind):
    from hypercraft_gb300 import worldgen
    return worldgen.scale_world(32, 8, 32) if kind == "scale" else worldgen.mixture_world(32, 16, 32)


@pytest.mark.parametrize("kind", ["scale", "mixture"])
def test_full_size_batch_matches_oracle_on_a_sample(ctx, oracle, kind):
    from hypercraft_gb300 import batch, worldgen
    from oracle import bind
    w = _world(kind)
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    assert n == (8192 if kind == "scale" else 16384)
    # arena sized by a counting run, then the autotuned plan (the bench's form)
    probe = batch.Arena(1, 1, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, probe, batch.PERSISTENT)
    plan.launch()
    need_q, need_m, _ = plan.result(check=False)
    plan.close()
    arena = batch.Arena(need_q + 1024, need_m + 64, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.AUTO)
    plan.launch()
    q, m, f = plan.result()
    assert (q, m, f) == (need_q, need_m, 0)

    pick = bind.sample_positions(n, SAMPLE, seed=2024)
    kinds = w.kinds[rw.chunks[pick]]
    if kind == "mixture":
        for k in (worldgen.KIND_AIR, worldgen.KIND_STONE, worldgen.KIND_TERRAIN, worldgen.KIND_RANDOM,
                  worldgen.KIND_CHECKER):
            assert (kinds == k).any(), f"sample holds no chunk of kind {k}"
    got = arena.sample_meshes(pick)
    want = bind.mesh_rows(oracle, w.blocks, w.heights, rw.neighbours[pick], os.cpu_count() or 1)
    quads = 0
    for i, ref in zip(pick, want):
        g = got[int(i)]
        assert len(g) == len(ref), (int(i), int(rw.chunks[i]))
        assert all(a == b for a, b in zip(g, ref)), (int(i), int(rw.chunks[i]))
        quads += sum(len(x.vertices) for x in g) // 4
    assert quads > 0
    plan.close()
    rw.pool.close()
