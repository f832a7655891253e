"""Batched forms (persistent work-stealing kernel in a CUDA graph, and one launch per chunk) give
each chunk exactly the meshes of the single-chunk call and of the CPU oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_world(kind):
    from hypercraft_gb300 import worldgen
    return worldgen.scale_world(4, 3, 4) if kind == "scale" else worldgen.mixture_world(4, 4, 4)


@pytest.mark.parametrize("kind", ["scale", "mixture"])
@pytest.mark.parametrize("mode", [0, 1, 2, 17, 18, 19, 20, 21, 22])
def test_batch_matches_oracle(ctx, oracle, kind, mode):
    """Persistent plan, per-chunk plan, the autotuned plan (whichever variant it keeps) and each
    other persistent variant pinned (window relight on one, two and four CTAs per chunk; 2 and 4
    chunks per claim; no global record scratch)."""
    from hypercraft_gb300 import batch
    w = _small_world(kind)
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    arena = batch.Arena(3_000_000, 4096, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, mode)
    if mode >= 16:
        assert plan.variant()[0] == mode - 16
    for _ in range(2):  # replay: cursors and work counter reset each launch
        plan.launch()
        q, m, f = plan.result()
    assert f == 0
    host = arena.host()
    total = 0
    for i, c in enumerate(rw.chunks):
        got = arena.chunk_meshes(i, host)
        nb = rw.neighbours[i]
        want = oracle.mesh_chunk([w.blocks[k] for k in nb], [w.heights[k] for k in nb])
        assert len(got) == len(want), (i, int(c))
        assert all(a == b for a, b in zip(got, want)), (i, int(c))
        total += sum(len(x.vertices) for x in got) // 4
    assert total == q


@pytest.mark.parametrize("mode", [0, 17, 18, 19, 20, 21, 22])
def test_batch_most_quads_match_oracle(ctx, oracle, mode):
    """The 196,608-quad chunk through each persistent variant (records past the shared buffer and
    the global scratch: the emission merges again in windows)."""
    import cases
    from hypercraft_gb300 import batch
    b, h = cases.transparent_checker()
    pool = batch.Pool(ctx, 27)
    pool.upload(0, np.stack(b), np.stack(h))
    arena = batch.Arena(400_000, 64, 1)
    plan = batch.BatchPlan(ctx, pool, np.arange(27, dtype=np.int32)[None, :], arena, mode)
    plan.launch()
    q, m, f = plan.result()
    assert f == 0 and q == 196608
    got, want = arena.chunk_meshes(0, arena.host()), oracle.mesh_chunk(b, h)
    assert len(got) == len(want) and all(a == c for a, c in zip(got, want))
    plan.close()
    pool.close()


def test_stage_times_and_blank_chunks(ctx):
    """The plan's in-graph stage events time every stage of the light-pass variant, and chunks the
    blank test skips get the empty result (no quad, status ok)."""
    from hypercraft_gb300 import batch
    w = _small_world("mixture")
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    arena = batch.Arena(3_000_000, 4096, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.PERSISTENT)
    plan.launch()
    planes_ms, light_ms, mesh_ms = plan.stage_ms()
    assert planes_ms > 0 and light_ms > 0 and mesh_ms > 0
    res = arena.results_host(n).reshape(n, 5)
    blank = [i for i in range(n) if not (w.blocks[rw.chunks[i]] != 0).any()]  # all-air chunks
    assert blank, "the mixture holds all-air chunks"
    assert (res[blank] == 0).all()


def test_async_download_matches_download(ctx):
    """hc_batch_plan_download_async on a stream gives the words hc_batch_plan_download gives."""
    import torch
    from hypercraft_gb300 import batch
    w = _small_world("scale")
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    arena = batch.Arena(3_000_000, 4096, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.PERSISTENT)
    plan.launch()
    q, m, f = plan.result()
    bufs = [(np.zeros(q * 8, np.uint32), np.zeros(q * 6, np.uint16), np.zeros(m * 12, np.uint32),
             np.zeros(n * 5, np.uint32)) for _ in range(2)]
    lib = rw.pool.lib
    ctx.check(lib.hc_batch_plan_download(plan.handle, q, m, *(b.ctypes.data for b in bufs[0])), "download")
    st = torch.cuda.Stream()
    ctx.check(lib.hc_batch_plan_download_async(plan.handle, q, m, *(b.ctypes.data for b in bufs[1]), st.cuda_stream),
              "download_async")
    st.synchronize()
    assert all(np.array_equal(a, b) for a, b in zip(*bufs))


def test_batch_matches_single_chunk_call(ctx):
    from hypercraft_gb300 import batch
    w = _small_world("mixture")
    rw = batch.upload_world(ctx, w)
    arena = batch.Arena(3_000_000, 4096, len(rw.chunks))
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.PERSISTENT, ctas_per_sm=1)
    plan.launch()
    plan.result()
    host = arena.host()
    for i in range(0, len(rw.chunks), 5):
        nb = rw.neighbours[i]
        single = ctx.mesh_chunk([w.blocks[k] for k in nb], [w.heights[k] for k in nb])
        got = arena.chunk_meshes(i, host)
        assert len(got) == len(single) and all(a == b for a, b in zip(got, single))


def test_bad_neighbour_slot_is_reported(ctx):
    from hypercraft_gb300 import batch
    w = _small_world("scale")
    rw = batch.upload_world(ctx, w)
    nbr = rw.neighbours.copy()
    nbr[1, 3] = -1
    nbr[2, 26] = w.n_chunks + 5
    arena = batch.Arena(3_000_000, 4096, len(nbr))
    plan = batch.BatchPlan(ctx, rw.pool, nbr, arena, batch.PERSISTENT)
    plan.launch()
    q, m, f = plan.result()
    assert f == 2
    res = arena.host()["results"].reshape(-1, 5)
    assert res[1, 4] == batch.RESULT_BAD_SLOT and res[2, 4] == batch.RESULT_BAD_SLOT
    assert (res[[0] + list(range(3, len(nbr))), 4] == 0).all()


def test_small_arena_reports_capacity(ctx):
    from hypercraft_gb300 import batch
    from hypercraft_gb300.mesher import HcError, HC_ERR_CAPACITY
    w = _small_world("mixture")
    rw = batch.upload_world(ctx, w)
    arena = batch.Arena(1000, 8, len(rw.chunks))
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.PERSISTENT)
    plan.launch()
    with pytest.raises(HcError) as e:
        plan.result()
    assert e.value.status == HC_ERR_CAPACITY
    q, m, f = plan.result(check=False)
    assert q > 1000 and f > 0  # required sizes are reported; chunks that did not fit are flagged
    res = arena.host()["results"].reshape(-1, 5)
    assert ((res[:, 4] == 0) | (res[:, 4] == batch.RESULT_ARENA_FULL)).all()
