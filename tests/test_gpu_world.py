"""Edit pipeline on the device against the CPU restatement of the reference's task chain
(SetBlock -> FloodSunlight -> SetSunlight -> kMesh): final blocks and heights, the set of remeshed
chunks, and byte-exact meshes of every remeshed chunk."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _meshes_of_chunk(oracle, w, cell):
    nb = w.neighbours(*w.coords(int(cell)))
    return oracle.mesh_chunk([w.blocks[k] for k in nb], [w.heights[k] for k in nb])


def _run(ctx, oracle, edits, world_factory, cluster=None):
    from hypercraft_gb300 import batch, world as hw
    from oracle import edits as oe
    w_gpu = world_factory()
    w_ref = world_factory()
    before = {int(c): _meshes_of_chunk(oracle, w_ref, c) for c in w_ref.meshable()}
    dirty_ref = oe.apply_edits(w_ref, edits)

    rw = hw.ResidentWorld(ctx, w_gpu)
    if cluster:
        rw.set_cluster(cluster)
    rw.apply_edits(edits)
    arena = batch.Arena(4_000_000, 8192, w_gpu.n_chunks)
    cells, q, m = rw.remesh(arena)
    b, h = rw.download()
    assert np.array_equal(b, w_ref.blocks), "final blocks differ"
    assert np.array_equal(h, w_ref.heights), "final sunlight heights differ"

    meshable = set(int(c) for c in w_ref.meshable())
    got = set(int(c) for c in cells)
    assert list(cells) == sorted(cells), "remesh order is grid order"
    assert got <= dirty_ref & meshable
    for c in (dirty_ref & meshable) - got:  # the reference would remesh these too, to the same meshes
        assert all(a == b for a, b in zip(before[c], _meshes_of_chunk(oracle, w_ref, c)))
    host = arena.host()
    for i, c in enumerate(cells):
        want = _meshes_of_chunk(oracle, w_ref, c)
        got_m = arena.chunk_meshes(i, host)
        assert len(got_m) == len(want) and all(a == b for a, b in zip(got_m, want)), int(c)
    # every chunk whose mesh changed was remeshed
    for c in meshable - got:
        assert all(a == b for a, b in zip(before[c], _meshes_of_chunk(oracle, w_ref, c))), c
    # a second remesh with no new edits has nothing to do
    cells2, _, _ = rw.remesh(arena)
    assert len(cells2) == 0
    return len(cells)


@pytest.mark.parametrize("cluster", [1, 2, 4, 8])
def test_seeded_edits_match_reference_chain(ctx, oracle, cluster):
    """Every cluster size (CTAs meshing one chunk together) gives the reference's meshes."""
    from hypercraft_gb300 import world as hw
    n = _run(ctx, oracle, hw.seeded_edits(4096, seed=7), hw.edit_world, cluster)
    assert n > 10


def test_repeated_and_reverted_edits(ctx, oracle):
    from hypercraft_gb300 import world as hw
    w = hw.edit_world()
    e = hw.seeded_edits(600, seed=11)
    # the same voxels edited again: some reverted to their original block, some changed twice
    again = e[:300].copy()
    orig = np.array([w.blocks[((x >> 5) + 3) + 7 * (((z >> 5) + 3) + 7 * ((y >> 5) + 2)),
                              (x & 31) + ((y & 31) * 32 + (z & 31)) * 32] for x, y, z in
                     zip(again["x"], again["y"], again["z"])], np.uint32)
    again["block"][:150] = orig[:150]
    again["block"][150:] = 9  # glass
    edits = np.concatenate([e, again, e[:50]])
    _run(ctx, oracle, edits, hw.edit_world)


def test_edits_outside_the_world_are_ignored(ctx, oracle):
    from hypercraft_gb300 import world as hw
    e = hw.seeded_edits(64, seed=3)
    far = e.copy()
    far["y"] += 10_000
    _run(ctx, oracle, np.concatenate([e, far]), hw.edit_world)


def test_loads_wait_for_neighbours_and_unloads_drop(ctx, oracle):
    """A loaded chunk is remeshed once its 26 neighbours are resident (kGenerate queues kMesh for
    itself; kMesh waits for the neighbours); a marked neighbour that waited is remeshed when the
    missing chunk arrives; an unloaded chunk's pending remesh is dropped."""
    from hypercraft_gb300 import batch, world as hw
    w = hw.edit_world()
    m = w.index(3, 2, 3)    # missing at first
    a = w.index(4, 2, 3)    # loaded first: waits for m
    b = w.index(5, 2, 5)    # loaded, then unloaded before the remesh (no neighbour of m or a)
    resident = np.ones(w.n_chunks, bool)
    resident[[m, a, b]] = False
    rw = hw.ResidentWorld(ctx, w, resident=resident)
    arena = batch.Arena(4_000_000, 8192, w.n_chunks)

    rw.load([a])
    cells, _, _ = rw.remesh(arena)
    assert len(cells) == 0, "a waits for m"

    rw.load([m])
    cells, _, _ = rw.remesh(arena)
    assert list(cells) == sorted([m, a])
    host = arena.host()
    for i, c in enumerate(cells):
        want = _meshes_of_chunk(oracle, w, c)
        got = arena.chunk_meshes(i, host)
        assert len(got) == len(want) and all(x == y for x, y in zip(got, want)), int(c)

    rw.load([b])
    rw.unload([b])
    cells, _, _ = rw.remesh(arena)
    assert len(cells) == 0, "b's pending remesh was dropped with it"

    rw.load([b])
    rw.unload([a])
    rw.load([a])  # the same cell leaves and returns between two remeshes: remeshed once
    cells, _, _ = rw.remesh(arena)
    assert list(cells) == sorted([a, b])
    host = arena.host()
    for i, c in enumerate(cells):
        want = _meshes_of_chunk(oracle, w, c)
        got = arena.chunk_meshes(i, host)
        assert len(got) == len(want) and all(x == y for x, y in zip(got, want)), int(c)


def test_full_arena_requeues_only_what_did_not_fit(ctx, oracle):
    """Chunks that do not fit the arena stay marked and are remeshed by the next call; the ones
    that fit are the reference's meshes."""
    from hypercraft_gb300 import batch, world as hw
    w = hw.edit_world()
    resident = np.ones(w.n_chunks, bool)
    inner = [w.index(x, y, z) for x in (2, 3, 4) for y in (1, 2, 3) for z in (2, 3, 4)]
    resident[inner] = False
    rw = hw.ResidentWorld(ctx, w, resident=resident)
    rw.load(inner)
    want_quads = sum(len(m.vertices) // 4 for c in inner for m in _meshes_of_chunk(oracle, w, c))
    small = batch.Arena(want_quads // 2, 8192, w.n_chunks)
    cells, _, _, status = rw.remesh(small, partial=True)
    assert sorted(int(c) for c in cells) == sorted(inner)
    assert 0 < int((status != 0).sum()) < len(cells)
    host = small.host()
    for i, c in enumerate(cells):
        if status[i] == 0:
            want = _meshes_of_chunk(oracle, w, c)
            got = small.chunk_meshes(i, host)
            assert len(got) == len(want) and all(x == y for x, y in zip(got, want)), int(c)
    big = batch.Arena(4_000_000, 8192, w.n_chunks)
    again, _, _ = rw.remesh(big)
    assert sorted(int(c) for c in again) == sorted(int(c) for i, c in enumerate(cells) if status[i] != 0)
    host = big.host()
    for i, c in enumerate(again):
        want = _meshes_of_chunk(oracle, w, c)
        got = big.chunk_meshes(i, host)
        assert len(got) == len(want) and all(x == y for x, y in zip(got, want)), int(c)
    assert len(rw.remesh(big)[0]) == 0


def test_loads_apply_stored_edits(ctx, oracle):
    """A loaded chunk's stored edits (the reference's packed block and sunlight entries) are applied
    in order after its generated data, and the chunk is meshed from the result."""
    from hypercraft_gb300 import batch, world as hw
    w = hw.edit_world()
    rng = np.random.default_rng(21)
    cells = [w.index(3, 2, 3), w.index(4, 2, 3)]
    resident = np.ones(w.n_chunks, bool)
    resident[cells] = False
    rw = hw.ResidentWorld(ctx, w, resident=resident)
    entries, want_b, want_h = [], [], []
    for c in cells:
        idx = rng.integers(0, 32768, 3000)
        idx[-100:] = idx[:100]  # the same cell edited twice: the later entry wins
        blk = rng.choice([0, 1, 9, 14, 16, 24], size=len(idx))
        cols = rng.integers(0, 1024, 200)
        hts = rng.integers(0, 33, 200)
        be, se = hw.pack_block_entries(idx, blk), hw.pack_sunlight_entries(cols, hts)
        entries.append((be, se))
        b, h = hw.apply_entries(w.blocks[c], w.heights[c], be, se)
        want_b.append(b)
        want_h.append(h)
    rw.load(cells, entries=entries)
    got_b, got_h = rw.download()
    for k, c in enumerate(cells):
        assert np.array_equal(got_b[c], want_b[k]) and np.array_equal(got_h[c], want_h[k])
    arena = batch.Arena(4_000_000, 8192, w.n_chunks)
    remeshed, _, _ = rw.remesh(arena)
    assert sorted(int(c) for c in remeshed) == sorted(cells)
    w.blocks[cells] = np.stack(want_b)
    w.heights[cells] = np.stack(want_h)
    host = arena.host()
    for i, c in enumerate(remeshed):
        want = _meshes_of_chunk(oracle, w, c)
        got = arena.chunk_meshes(i, host)
        assert len(got) == len(want) and all(x == y for x, y in zip(got, want)), int(c)
