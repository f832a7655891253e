"""CPU restatement of the reference's edit task chain, for the edit pipeline's parity tests.

TEST INFRASTRUCTURE (like the rest of oracle/).

Follows, edit by edit in order:
  * ChunkTaskRunner<kSetBlock>::Run (client/src/ChunkSetBlockTask.cpp:37-131): a block that differs
    from the stored one is written; every neighbour chunk i with
    ChunkShouldRemesh(block_pos - 32 * offset_i) (client/include/client/ChunkMeshTask.inl:9-15) is
    marked for remeshing; the block's column is flooded;
  * ChunkTaskRunner<kFloodSunlight>::Run (client/src/ChunkFloodSunlightTask.cpp:33-66): a flooded
    column's height becomes 32 if the chunk above has a positive height there, else one above its
    highest block that stops vertical light;
  * ChunkTaskRunner<kSetSunlight>::Run (client/src/ChunkSetSunlightTask.cpp:28-90): a changed height
    is stored, the 27 chunks around are marked (its ChunkShouldRemesh test does not depend on the
    neighbour and always holds for heights 0..32), and the chunk below is flooded at that column.
The chunk above the top grid layer, or a missing one, counts as lit from above.
"""
from __future__ import annotations

import numpy as np

from . import bind

_VERTICAL = None


def _vertical_table():
    global _VERTICAL
    if _VERTICAL is None:
        reg = bind.oracle_registry()
        _VERTICAL = reg["transparency"] == 2
    return _VERTICAL


def _should_remesh(x, y, z):
    def d(v):
        return -1 - v if v < -1 else (v - 33 if v >= 33 else 0)
    return 15 > d(x) + d(y) + d(z)


def apply_edits(world, edits) -> set:
    """Applies edits to world (a worldgen.World, modified in place); returns the chunk indices the
    reference's tasks would remesh."""
    vertical = _vertical_table()
    nx, ny, nz = world.nx, world.ny, world.nz
    cx0, cy0, cz0 = world.origin
    dirty, floods = set(), {}
    for e in edits:
        x, y, z, b = int(e["x"]), int(e["y"]), int(e["z"]), int(e["block"]) & 0xFFFF
        ix, iy, iz = (x >> 5) - cx0, (y >> 5) - cy0, (z >> 5) - cz0
        if not (0 <= ix < nx and 0 <= iy < ny and 0 <= iz < nz):
            continue
        cell = ix + nx * (iz + nz * iy)
        lx, ly, lz = x & 31, y & 31, z & 31
        idx = lx + (ly * 32 + lz) * 32
        if world.blocks[cell, idx] == b:
            continue
        world.blocks[cell, idx] = b
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    jx, jy, jz = ix + dx, iy + dy, iz + dz
                    if 0 <= jx < nx and 0 <= jy < ny and 0 <= jz < nz and _should_remesh(lx - 32 * dx, ly - 32 * dy,
                                                                                          lz - 32 * dz):
                        dirty.add(jx + nx * (jz + nz * jy))
        floods.setdefault((ix, iz, lx, lz), set()).add(iy)
    changed = set()
    for (ix, iz, lx, lz), layers in floods.items():
        cascade = False
        for iy in range(max(layers), -1, -1):
            if not cascade and iy not in layers:
                continue
            cell = ix + nx * (iz + nz * iy)
            col = lx + 32 * lz
            if iy + 1 < ny and world.heights[ix + nx * (iz + nz * (iy + 1)), col] > 0:
                nh = 32
            else:
                ys = world.blocks[cell, col::1024]  # y = 0..31
                stop = np.nonzero(~vertical[ys])[0]
                nh = int(stop[-1]) + 1 if len(stop) else 0
            cascade = int(world.heights[cell, col]) != nh
            if cascade:
                world.heights[cell, col] = nh
                changed.add((ix, iy, iz))
    for ix, iy, iz in changed:
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    jx, jy, jz = ix + dx, iy + dy, iz + dz
                    if 0 <= jx < nx and 0 <= jy < ny and 0 <= jz < nz:
                        dirty.add(jx + nx * (jz + nz * jy))
    return dirty
