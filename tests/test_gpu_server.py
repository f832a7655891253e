"""Request server on the device: a seeded serving trace (edits, 16^3 fills, loads and unloads
along a player walk) replayed in real time, many requests per tick, against the same trace run one
request per tick and against each tick's requests run alone; and the meshes the one-at-a-time run
produces against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID, ORIGIN, RADIUS = (16, 8, 16), (-8, -4, -8), 4


@pytest.fixture(scope="module")
def library():
    from hypercraft_gb300 import server as hs
    return hs.ChunkLibrary(6, 4, 6, seed=77)


def _trace(library, seed=3, rate=20000.0, duration=0.05):
    from hypercraft_gb300 import server as hs
    wl = hs.ServingWorkload(library, GRID, ORIGIN, RADIUS, seed=seed)
    init = wl.initial_loads()
    reqs, times = wl.trace(rate, duration)
    return init, reqs, times


def _neighbourhood_moves(srv, reqs):
    """Grid cells whose 27-neighbourhood saw a load or unload in `reqs`."""
    from hypercraft_gb300 import server as hs
    out = set()
    for r in reqs:
        if r["kind"] in (hs.REQ_LOAD, hs.REQ_UNLOAD):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        p = (int(r["x"]) + dx, int(r["y"]) + dy, int(r["z"]) + dz)
                        if all(ORIGIN[a] <= p[a] < ORIGIN[a] + GRID[a] for a in range(3)):
                            out.add(srv.cell(*p))
    return out


def _server(ctx, **kw):
    from hypercraft_gb300 import server as hs
    return hs.Server(ctx, GRID, ORIGIN, pool_capacity=1024, max_loads_per_tick=64, arena_quads=2 << 20,
                     arena_meshes=8192, **kw)


def _meshes_equal(a, b):
    return a is not None and b is not None and len(a) == len(b) and all(x == y for x, y in zip(a, b))


def test_same_result_alone_and_in_the_mix(ctx, oracle, library):
    init, reqs, times = _trace(library)
    assert len(reqs) > 500

    # alone: one request per tick, each pass finished before the next request is submitted; the
    # sink checks the first chunks of every pass against the oracle on the pool as it is then
    alone = _server(ctx)
    latest_alone, checked, errors = {}, [0], []

    def sink_alone(tick, cells, meshes, status):
        # runs inside a ctypes callback, where an exception would be swallowed: record it instead
        try:
            for i, c in enumerate(cells):
                if status[i] != 0:
                    errors.append(f"tick {tick}: chunk {int(c)} status {int(status[i])}")
                latest_alone[int(c)] = meshes[i]
            for i, c in enumerate(cells[:2]):
                if checked[0] >= 120:
                    break
                ix, iy, iz = (int(v) - o for v, o in zip(alone.cell_pos(int(c)), ORIGIN))
                nb = _neighbours(ix, iy, iz)
                b, h = alone.download(nb)
                want = oracle.mesh_chunk(list(b), list(h))
                if not _meshes_equal(meshes[i], want):
                    errors.append(f"tick {tick}: chunk {int(c)} differs from the oracle")
                checked[0] += 1
        except Exception as e:  # noqa: BLE001
            errors.append(repr(e))

    alone.set_sink(sink_alone)
    alone.submit(init)
    alone.drain()
    for r in reqs:
        alone.submit(r[None])
        alone.drain()
    assert not errors, errors[:5]
    assert checked[0] >= 60
    st_alone = alone.stats()

    # mix: real-time replay at 20k requests/s, 1 ms ticks, three passes in flight
    mix = _server(ctx)
    latest_mix = {}

    def sink_mix(tick, cells, meshes, status):
        for i, c in enumerate(cells):
            if status[i] == 0:
                latest_mix[int(c)] = meshes[i]

    mix.set_sink(sink_mix)
    mix.submit(init)
    mix.drain()
    mix.start()
    lat, elapsed = mix.replay(reqs, times)
    mix.stop()
    st_mix = mix.stats()
    assert st_mix["ticks"] < st_alone["ticks"], "requests were batched"
    assert (lat > 0).all()

    # same final world: resident set, blocks and heights of every resident chunk
    ra, rm = alone.resident(), mix.resident()
    assert np.array_equal(ra >= 0, rm >= 0)
    cells = np.nonzero(ra >= 0)[0]
    ba, ha = alone.download(cells)
    bm, hm = mix.download(cells)
    assert np.array_equal(ba, bm) and np.array_equal(ha, hm)

    # same latest meshes of every chunk whose neighbourhood no load or unload touched
    moved = _neighbourhood_moves(alone, reqs)
    steady = [c for c in latest_alone if c not in moved]
    assert len(steady) >= 10
    for c in steady:
        assert _meshes_equal(latest_alone[c], latest_mix.get(c)), c
    alone.close()
    mix.close()


def test_every_pass_same_alone_and_in_the_mix(ctx, library):
    """Every pass of the real-time mix, run again alone: the requests that one tick of the mix
    admitted are submitted together to a fresh server and run as one pass, with nothing else in
    flight. Each pass remeshes the same chunks, in the same order, with the same meshes."""
    init, reqs, times = _trace(library, seed=5)
    mix = _server(ctx)
    passes_mix = {}

    def sink_mix(tick, cells, meshes, status):
        passes_mix[int(tick)] = ([int(c) for c in cells], list(meshes), [int(x) for x in status])

    mix.set_sink(sink_mix)
    mix.submit(init)
    mix.drain()
    passes_mix.clear()
    mix.start()
    _, _, ticks = mix.replay(reqs, times, with_ticks=True)
    mix.stop()
    groups = sorted(set(int(t) for t in ticks))
    assert len(groups) < len(reqs), "requests were batched"
    assert set(t for t, p in passes_mix.items() if p[0]) <= set(groups), "a pass without admitted requests"

    alone = _server(ctx)
    last = {}

    def sink_alone(tick, cells, meshes, status):
        last["pass"] = ([int(c) for c in cells], list(meshes), [int(x) for x in status])

    alone.set_sink(sink_alone)
    alone.submit(init)
    alone.drain()
    remeshed = 0
    for t in groups:
        group = reqs[ticks == t]
        last.clear()
        alone.submit(group)
        assert alone.step() == len(group), t
        got = last.get("pass", ([], [], []))
        want = passes_mix.get(t, ([], [], []))
        assert got[0] == want[0], t
        assert got[2] == want[2], t
        for i, c in enumerate(got[0]):
            if got[2][i] == 0:
                assert _meshes_equal(got[1][i], want[1][i]), (t, c)
        remeshed += len(got[0])
    assert remeshed >= 20
    alone.close()
    mix.close()


def _neighbours(ix, iy, iz):
    """Grid cells of the 27 chunks around (ix, iy, iz), in the reference's neighbour order."""
    rev = (1, -1, 0)
    out = []
    for i in range(27):
        dx, dy, dz = rev[i // 9], rev[(i // 3) % 3], rev[i % 3]
        out.append((ix + dx) + GRID[0] * ((iz + dz) + GRID[2] * (iy + dy)))
    return out


def test_rejects_and_slot_reuse(ctx, library):
    """Requests outside the grid are rejected; unloaded slots are reused by later loads."""
    from hypercraft_gb300 import server as hs
    srv = hs.Server(ctx, GRID, ORIGIN, pool_capacity=8, max_loads_per_tick=4, arena_quads=1 << 20,
                    arena_meshes=4096)
    r = np.zeros(12, hs.REQUEST_DTYPE)
    k = library.index(0, 0, 0)
    for i in range(8):
        r[i]["kind"], r[i]["x"], r[i]["y"], r[i]["z"] = hs.REQ_LOAD, i - 4, 0, 0
        r[i]["blocks"], r[i]["heights"] = library.blocks[k].ctypes.data, library.heights[k].ctypes.data
    r[8]["kind"], r[8]["x"] = hs.REQ_LOAD, 1000  # outside the grid
    r[8]["blocks"], r[8]["heights"] = library.blocks[k].ctypes.data, library.heights[k].ctypes.data
    r[9]["kind"], r[9]["x"], r[9]["y"], r[9]["z"] = hs.REQ_UNLOAD, -4, 0, 0
    r[10]["kind"], r[10]["x"], r[10]["y"], r[10]["z"] = hs.REQ_LOAD, 0, 1, 0  # needs the freed slot
    r[10]["blocks"], r[10]["heights"] = library.blocks[k].ctypes.data, library.heights[k].ctypes.data
    r[11]["kind"], r[11]["size"] = hs.REQ_FILL, 40  # bad fill size
    r["tag"] = np.arange(12)
    srv.submit(r)
    srv.drain()
    done = srv.poll()
    assert sorted(done["tag"].tolist()) == list(range(12))
    status = dict(zip(done["tag"].tolist(), done["status"].tolist()))
    assert status[8] == 1 and status[11] == 1
    assert all(status[i] == 0 for i in (0, 1, 2, 3, 4, 5, 6, 7, 9, 10))
    res = srv.resident()
    assert res[srv.cell(-4, 0, 0)] == -1 and res[srv.cell(0, 1, 0)] >= 0
    assert srv.stats()["resident"] == 8
    srv.close()


def test_loads_with_stored_edits(ctx, library):
    """A LOAD request's stored edits are applied after its data, before it is meshed."""
    from hypercraft_gb300 import server as hs, world as hw
    srv = hs.Server(ctx, GRID, ORIGIN, pool_capacity=64, max_loads_per_tick=8, arena_quads=1 << 20,
                    arena_meshes=4096)
    rng = np.random.default_rng(5)
    k = library.index(0, 0, 0)
    be = hw.pack_block_entries(rng.integers(0, 32768, 500), rng.choice([0, 1, 24], 500))
    se = hw.pack_sunlight_entries(rng.integers(0, 1024, 50), rng.integers(0, 33, 50))
    r = np.zeros(2, hs.REQUEST_DTYPE)
    for i, (x, with_entries) in enumerate(((0, True), (1, False))):
        r[i]["kind"], r[i]["x"], r[i]["y"], r[i]["z"] = hs.REQ_LOAD, x, 0, 0
        r[i]["blocks"], r[i]["heights"] = library.blocks[k].ctypes.data, library.heights[k].ctypes.data
        if with_entries:
            r[i]["block_entries"], r[i]["n_block_entries"] = be.ctypes.data, len(be)
            r[i]["sunlight_entries"], r[i]["n_sunlight_entries"] = se.ctypes.data, len(se)
    srv.submit(r)
    srv.drain()
    b, h = srv.download([srv.cell(0, 0, 0), srv.cell(1, 0, 0)])
    wb, wh = hw.apply_entries(library.blocks[k], library.heights[k], be, se)
    assert np.array_equal(b[0], wb) and np.array_equal(h[0], wh)
    assert np.array_equal(b[1], library.blocks[k]) and np.array_equal(h[1], library.heights[k])
    srv.close()


def test_draw_records_match_the_renderer_rule(ctx, library):
    """Every pass's MeshInfo<ChunkMeshInfo> records equal WorldRenderer::PushChunkMesh's: the arena
    offsets and counts, and the float AABB = u32 AABB / 16 + chunk base (bit for bit)."""
    from hypercraft_gb300 import server as hs
    srv = _server(ctx)
    init, _, _ = _trace(library)
    errors, seen = [], [0]

    def sink(tick, cells, meshes, status, md, mi):
        try:
            for j in range(len(md)):
                c = int(cells[int(md[j]["chunk"])])
                want = hs.mesh_info_of(md[j], srv.cell_pos(c))
                if want.tobytes() != mi[j].tobytes():
                    errors.append((tick, j, want, mi[j]))
                seen[0] += 1
        except Exception as e:  # noqa: BLE001
            errors.append(repr(e))

    sink.wants_infos = True
    srv.set_sink(sink)
    srv.submit(init)
    srv.drain()
    assert not errors, errors[:3]
    assert seen[0] > 50
    srv.close()
