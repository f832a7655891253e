"""The batched form lights a whole batch of chunks at once instead of relighting a 62^3 window per
chunk; this pins, on the CPU, that the two agree on every meshed chunk's [-1, 33)^3 box.

The batch form's rule (no window, no border bound, missing chunks dark) is restated here over a
whole world grid with numpy; each inner chunk's box is compared with the oracle's window relight
(the reference's BFS, client/src/ChunkMeshTask.cpp:48-111)."""
import numpy as np
import pytest

import cases


def _world_light(w, reg):
    """Sun and torch light of every cell of a worldgen.World by the level recurrence
    S_15 = seeds, S_t = S_{t+1} | seeds_t | (pass & dilate6(S_{t+1}))."""
    n = 32
    X, Y, Z = w.nx * n, w.ny * n, w.nz * n
    blocks = np.zeros((Y, Z, X), np.uint16)
    sun15 = np.zeros((Y, Z, X), bool)
    for c in range(w.n_chunks):
        ix, iy, iz = w.coords(c)
        b = w.blocks[c].reshape(n, n, n)  # (y, z, x)
        blocks[iy * n:(iy + 1) * n, iz * n:(iz + 1) * n, ix * n:(ix + 1) * n] = b
        h = w.heights[c].reshape(n, n).astype(np.int64)  # (z, x)
        y = np.arange(n)[:, None, None]
        sun15[iy * n:(iy + 1) * n, iz * n:(iz + 1) * n, ix * n:(ix + 1) * n] = \
            (y.astype(np.uint32) >= (h[None] & 0xFFFFFFFF).astype(np.uint32))
    passes = reg["transparency"][blocks] != 0
    emit = reg["light"][blocks].astype(np.int64)

    def cascade(seed_level):
        light = np.zeros(blocks.shape, np.uint8)
        s = seed_level >= 15
        light[s] = 15
        for t in range(14, 0, -1):
            d = np.zeros_like(s)
            d[1:] |= s[:-1]
            d[:-1] |= s[1:]
            d[:, 1:] |= s[:, :-1]
            d[:, :-1] |= s[:, 1:]
            d[:, :, 1:] |= s[:, :, :-1]
            d[:, :, :-1] |= s[:, :, 1:]
            s = s | (seed_level >= t) | (passes & d)
            light[s & (light == 0)] = t
        return light

    sun = cascade(np.where(sun15, 15, 0))
    torch = cascade(emit)
    return sun, torch


@pytest.mark.parametrize("seed", [1, 2])
def test_batch_light_equals_window_relight(oracle, seed):
    from hypercraft_gb300 import worldgen
    from oracle import bind
    reg = bind.oracle_registry()
    w = worldgen.generate(4, 4, 4, (-2, -2, -2), seed=worldgen.WORLD_SEED + seed, caves=True, air_ring=False)
    # denser light: scatter glowstone and a few low-light blocks through the caves
    rng = np.random.default_rng(seed)
    for c in range(w.n_chunks):
        air = np.nonzero(w.blocks[c] == 0)[0]
        pick = rng.choice(air, size=min(len(air), 40), replace=False)
        w.blocks[c, pick] = 24
    w.recompute_heights()
    sun, torch = _world_light(w, reg)
    checked = 0
    for c in w.meshable():
        ix, iy, iz = w.coords(int(c))
        nb = w.neighbours(ix, iy, iz)
        win = oracle.relight_window([w.blocks[k] for k in nb], [w.heights[k] for k in nb]).reshape(62, 62, 62)
        box = win[14:48, 14:48, 14:48]  # window index v + 15 for v in [-1, 33), (y, z, x)
        y0, z0, x0 = iy * 32 - 1, iz * 32 - 1, ix * 32 - 1
        s = sun[y0:y0 + 34, z0:z0 + 34, x0:x0 + 34]
        t = torch[y0:y0 + 34, z0:z0 + 34, x0:x0 + 34]
        assert np.array_equal(box & 15, s), f"sun differs in chunk {int(c)}"
        assert np.array_equal(box >> 4, t), f"torch differs in chunk {int(c)}"
        checked += 1
    assert checked == 8


def test_light_cases_have_light(oracle):
    """The golden glow case holds torch light (the comparison above is not vacuous)."""
    b, h = cases.glow(3)
    assert (oracle.relight_window(b, h) >> 4).max() >= 14
