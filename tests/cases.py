"""Seeded input cases for the parity tests: each case is 27 chunks (blocks, heights) in the
reference's neighbour order (centre = 26). numpy's PCG64 and the integer world generator give
identical bytes on x86 and aarch64, so the committed golden digests apply on every host.
"""
from __future__ import annotations

import hashlib

import numpy as np

N = 32768
IDX = np.arange(N)
X, Z, Y = IDX % 32, (IDX // 32) % 32, IDX // 1024


def _blank(fill=0, height=0):
    return [np.full(N, fill, np.uint16) for _ in range(27)], [np.full(1024, height, np.int8) for _ in range(27)]


def _from_world(world, ix, iy, iz):
    nb = world.neighbours(ix, iy, iz)
    return [world.blocks[i].copy() for i in nb], [world.heights[i].copy() for i in nb]


def plain():
    from hypercraft_gb300 import worldgen
    return _from_world(worldgen.plain_world(), 1, 1, 1)


def random_all(seed):
    """Every id 0..27 (3 unregistered) with random metas, 50% air, random heights in [-2, 34]."""
    rng = np.random.default_rng(seed)
    b, h = [], []
    for _ in range(27):
        ids = rng.integers(0, 28, N)
        metas = rng.integers(0, 256, N)
        raw = np.where(rng.random(N) < 0.5, 0, ids | (metas << 8)).astype(np.uint16)
        b.append(raw)
        h.append(rng.integers(-2, 35, 1024).astype(np.int8))
    return b, h


def liquids(seed):
    """Water, flowing water of every level, plants, vines, cactus, glass, ice, leaves."""
    rng = np.random.default_rng(seed)
    choices = np.array([0, 0, 14, 15, 15, 15, 1, 5, 21, 20, 9, 12, 16, 19, 22, 23, 7], np.int64)
    b, h = [], []
    for _ in range(27):
        ids = rng.choice(choices, N)
        metas = rng.integers(0, 20, N)
        b.append((ids | (metas << 8)).astype(np.uint16))
        h.append(rng.integers(0, 33, 1024).astype(np.int8))
    return b, h


def checker():
    """3D stone/air checkerboard: 98,304 quads in the centre chunk, seven opaque meshes."""
    b, h = _blank()
    for i in range(27):
        b[i] = np.where((X + Y + Z) % 2 == 0, 1, 0).astype(np.uint16)
    return b, h


def transparent_checker():
    """3D glass/ice checkerboard: every cell face shows from both sides, 196,608 quads in the centre
    chunk (more than the mesher keeps records for, so its emission merges planes again)."""
    b, h = _blank()
    for i in range(27):
        b[i] = np.where((X + Y + Z) % 2 == 0, 9, 12).astype(np.uint16)
    return b, h


def glow(seed):
    """5% glowstone in half-filled stone: torch light across chunk borders; sun from random heights."""
    rng = np.random.default_rng(seed)
    b, h = [], []
    for _ in range(27):
        r = rng.random(N)
        b.append(np.where(r < 0.05, 24, np.where(r < 0.55, 1, 0)).astype(np.uint16))
        h.append(rng.integers(0, 33, 1024).astype(np.int8))
    return b, h


def single_block(block=1):
    b, h = _blank()
    b[26][5 + (7 * 32 + 9) * 32] = block
    return b, h


def two_blocks_merge():
    b, h = _blank()
    b[26][3 + (4 * 32 + 5) * 32] = 1
    b[26][4 + (4 * 32 + 5) * 32] = 1
    return b, h


def l_shape():
    b, h = _blank()
    for x, y, z in [(3, 4, 5), (4, 4, 5), (5, 4, 5), (3, 4, 6), (3, 4, 7), (3, 5, 5)]:
        b[26][x + (y * 32 + z) * 32] = 3
    return b, h


def border_faces():
    """Solid centre chunk against varied neighbours: faces only on the chunk's boundary layers."""
    rng = np.random.default_rng(7)
    b, h = _blank(1)
    for i in range(26):
        b[i] = np.where(rng.random(N) < 0.5, 0, rng.choice([1, 9, 12, 14, 16, 24], N)).astype(np.uint16)
    return b, h


def all_air():
    return _blank(0)


def all_stone():
    return _blank(1, 32)


def vines_and_plants():
    b, h = _blank()
    vals = [21 | (t << 8) for t in range(8)] + [5 | (v << 8) for v in range(4)] + [7, 19, 20, 22, 23]
    for k in range(0, N, 3):
        b[26][k] = vals[(k // 3) % len(vals)]
    for i in range(26):
        b[i][::5] = 1
    return b, h


def _slab(centre_top):
    """27 chunks of flat ground: the centre layer of chunks is stone below y = 10 with `centre_top`
    (a function of the cell arrays giving the raw block at y = 10) on top, sunlit above; the layer
    above is air, the one below stone."""
    b, h = [], []
    for i in range(27):
        cy = (i // 3) % 3  # 0: the layer above, 1: below, 2: the centre's
        if cy == 0:
            b.append(np.zeros(N, np.uint16)), h.append(np.zeros(1024, np.int8))
        elif cy == 1:
            b.append(np.ones(N, np.uint16)), h.append(np.full(1024, 32, np.int8))
        else:
            b.append(np.where(Y < 10, 1, np.where(Y == 10, 4, 0)).astype(np.uint16))
            h.append(np.full(1024, 11, np.int8))
    b[26] = np.where(Y < 10, 1, np.where(Y == 10, centre_top(X, Z), 0)).astype(np.uint16)
    return b, h


def flat_ground(leaves: bool):
    """A flat grass top: its face plane holds 1,024 faces (keyed in two halves) that merge into one
    quad across the split row; with leaves on the rows around the split (z = 14..16), the row above
    the second half holds complex faces."""
    b, h = _slab(lambda x, z: np.full(x.shape, 4))
    if leaves:
        for x, z in [(3, 15), (4, 15), (9, 15), (20, 15), (31, 15), (0, 16), (12, 16), (7, 14), (25, 14)]:
            b[26][x + (11 * 32 + z) * 32] = 16
    return b, h


def stripes():
    """Grass and dirt tops in z rows: pairs of equal rows (rows linked by equal-below cells) for
    z < 16, single rows alternating for z >= 16 (isolated rows), and a glass strip."""
    b, h = _slab(lambda x, z: np.where(z < 16, np.where((z // 2) % 2 == 0, 4, 3), np.where(z % 2 == 0, 4, 3)))
    b[26][np.flatnonzero((Y == 11) & (X == 5))] = 9
    return b, h


def terrain_sample(kind: str, k: int):
    """Chunk k of a small seeded scale (caves + glowstone) or mixture world."""
    from hypercraft_gb300 import worldgen
    w = (worldgen.scale_world(4, 4, 4) if kind == "scale" else worldgen.mixture_world(4, 4, 4))
    inner = w.meshable()
    c = int(inner[(k * 7919) % len(inner)])
    return _from_world(w, *w.coords(c))


CASES = {
    "plain": plain,
    "random_all_1": lambda: random_all(1),
    "random_all_2": lambda: random_all(2),
    "liquids_1": lambda: liquids(11),
    "liquids_2": lambda: liquids(12),
    "checker": checker,
    "glow_1": lambda: glow(21),
    "single_stone": lambda: single_block(1),
    "single_glass": lambda: single_block(9),
    "single_glowstone": lambda: single_block(24),
    "two_blocks_merge": two_blocks_merge,
    "l_shape": l_shape,
    "border_faces": border_faces,
    "all_air": all_air,
    "all_stone": all_stone,
    "vines_and_plants": vines_and_plants,
    "scale_0": lambda: terrain_sample("scale", 0),
    "scale_1": lambda: terrain_sample("scale", 1),
    "mixture_0": lambda: terrain_sample("mixture", 0),
    "mixture_1": lambda: terrain_sample("mixture", 1),
    "mixture_2": lambda: terrain_sample("mixture", 2),
}


def input_digest(blocks27, heights27) -> str:
    h = hashlib.sha256()
    for b in blocks27:
        h.update(np.ascontiguousarray(b, np.uint16).astype("<u2").tobytes())
    for x in heights27:
        h.update(np.ascontiguousarray(x, np.int8).tobytes())
    return h.hexdigest()


def mesh_digest(meshes) -> str:
    """sha256 of the meshes in order: header (vertex count, index count, AABB, flag), vertices, indices."""
    h = hashlib.sha256()
    for m in meshes:
        hdr = np.array([len(m.vertices), len(m.indices), *m.aabb, int(m.transparent)], "<u4")
        h.update(hdr.tobytes())
        h.update(np.ascontiguousarray(m.vertices).astype("<u4").tobytes())
        h.update(np.ascontiguousarray(m.indices).astype("<u2").tobytes())
    return h.hexdigest()


def light34_from_window(light62: np.ndarray) -> np.ndarray:
    """[-1, 32]^3 of a 62^3 window (x fastest, then z, then y), x fastest again."""
    w = light62.reshape(62, 62, 62)  # [y][z][x]
    return np.ascontiguousarray(w[14:48, 14:48, 14:48]).reshape(-1)
