"""Block edits on a resident world, then relight + remesh of the chunks they touch.

Python side of include/hc_gb300.h's hc_world_* entry points, which replace the reference's edit task
chain (client/src/ChunkSetBlockTask.cpp:37-131 -> ChunkFloodSunlightTask.cpp:33-66 ->
ChunkSetSunlightTask.cpp:28-90 -> kMesh).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import batch
from .mesher import Context, library

EDIT_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("block", "<u4")])


class _Desc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("nx", "ny", "nz", "cx0", "cy0", "cz0")]


class ChunkLoad(ctypes.Structure):
    _fields_ = [("cx", ctypes.c_int32), ("cy", ctypes.c_int32), ("cz", ctypes.c_int32), ("slot", ctypes.c_int32),
                ("blocks", ctypes.c_void_p), ("heights", ctypes.c_void_p), ("block_entries", ctypes.c_void_p),
                ("sunlight_entries", ctypes.c_void_p), ("n_block_entries", ctypes.c_uint32),
                ("n_sunlight_entries", ctypes.c_uint32)]


def pack_block_entries(cells, blocks) -> np.ndarray:
    """PackedChunkBlockEntry (common/include/common/Data.hpp:36-58): cell index << 16 | raw block."""
    return (np.asarray(cells, np.uint32) << 16) | (np.asarray(blocks, np.uint32) & 0xFFFF)


def pack_sunlight_entries(columns, heights) -> np.ndarray:
    """PackedChunkSunlightEntry (common/include/common/Data.hpp:60-81): column index << 6 | height."""
    return ((np.asarray(columns, np.uint32) << 6) | (np.asarray(heights, np.uint32) & 63)).astype(np.uint16)


def apply_entries(blocks, heights, block_entries=None, sunlight_entries=None):
    """Host restatement of loading a chunk's stored edits (ChunkGenerateTask.cpp:33-36), in order."""
    blocks, heights = blocks.copy(), heights.copy()
    for e in (block_entries if block_entries is not None else []):
        e = int(e)
        if (e >> 16) < 32768:
            blocks[e >> 16] = e & 0xFFFF
    for e in (sunlight_entries if sunlight_entries is not None else []):
        e = int(e)
        heights[e >> 6] = np.int8(e & 63)
    return blocks, heights


def _bind(lib):
    if getattr(lib, "_world_bound", False):
        return lib
    vp, P = ctypes.c_void_p, ctypes.POINTER
    lib.hc_world_create.argtypes = [vp, vp, P(_Desc), vp, P(vp)]
    lib.hc_world_destroy.argtypes = [vp]
    lib.hc_world_destroy.restype = None
    lib.hc_world_apply_edits.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_int, vp]
    lib.hc_world_remesh.argtypes = [vp, P(batch._Arena), vp, ctypes.c_uint32, P(ctypes.c_uint32),
                                    P(ctypes.c_uint64), P(ctypes.c_uint32), vp]
    lib.hc_world_load.argtypes = [vp, P(ChunkLoad), ctypes.c_uint32, vp]
    lib.hc_world_unload.argtypes = [vp, vp, ctypes.c_uint32, vp]
    lib.hc_world_touch.argtypes = [vp, vp]
    lib.hc_world_set_cluster.argtypes = [vp, ctypes.c_int]
    lib._world_bound = True
    return lib


class ResidentWorld:
    """A generated world (worldgen.World) resident in a device pool, slot = chunk index."""

    def __init__(self, ctx: Context, world, resident=None, capacity=None):
        """resident: optional bool mask of the chunks loaded at creation (default all); chunk i
        uses pool slot i."""
        self.ctx, self.world = ctx, world
        self.lib = _bind(batch._bind(library()))
        self.pool = batch.Pool(ctx, capacity or world.n_chunks)
        self.pool.upload(0, world.blocks, world.heights)
        slots = np.arange(world.n_chunks, dtype=np.int32)
        if resident is not None:
            slots[~np.asarray(resident, bool)] = -1
        h = ctypes.c_void_p()
        desc = _Desc(world.nx, world.ny, world.nz, *world.origin)
        ctx.check(self.lib.hc_world_create(ctx.handle, self.pool.handle, ctypes.byref(desc), slots.ctypes.data,
                                           ctypes.byref(h)), "hc_world_create")
        self.handle = h

    def apply_edits(self, edits: np.ndarray, stream=None):
        """edits: structured array of EDIT_DTYPE (host) or a torch int32 (n, 4) cuda tensor."""
        if hasattr(edits, "data_ptr"):
            self.ctx.check(self.lib.hc_world_apply_edits(self.handle, edits.data_ptr(), edits.shape[0], 1, stream),
                           "hc_world_apply_edits")
        else:
            e = np.ascontiguousarray(edits, EDIT_DTYPE)
            self.ctx.check(self.lib.hc_world_apply_edits(self.handle, e.ctypes.data, len(e), 0, stream),
                           "hc_world_apply_edits")

    def load(self, cells, blocks=None, heights=None, stream=None, entries=None):
        """Loads grid cells (chunk i into pool slot i) from the world's arrays, or from the given
        (n, 32768) blocks and (n, 1024) heights; entries: optional per-chunk (block_entries,
        sunlight_entries) of stored edits, applied on the device after the copy."""
        cells = np.asarray(cells, np.int64)
        b = np.ascontiguousarray(self.world.blocks[cells] if blocks is None else blocks, np.uint16)
        h = np.ascontiguousarray(self.world.heights[cells] if heights is None else heights, np.int8)
        loads = (ChunkLoad * len(cells))()
        keep = []
        for i, c in enumerate(cells):
            ix, iy, iz = self.world.coords(int(c))
            ox, oy, oz = self.world.origin
            be, se = (entries[i] if entries is not None else (None, None))
            be = np.ascontiguousarray(be if be is not None else np.zeros(0), np.uint32)
            se = np.ascontiguousarray(se if se is not None else np.zeros(0), np.uint16)
            keep += [be, se]
            loads[i] = ChunkLoad(ox + ix, oy + iy, oz + iz, int(c), b[i].ctypes.data, h[i].ctypes.data,
                                 be.ctypes.data if len(be) else None, se.ctypes.data if len(se) else None,
                                 len(be), len(se))
        self.ctx.check(self.lib.hc_world_load(self.handle, loads, len(cells), stream), "hc_world_load")

    def unload(self, cells, stream=None):
        pos = np.array([[o + c for o, c in zip(self.world.origin, self.world.coords(int(i)))] for i in cells],
                       np.int32).reshape(-1, 3)
        self.ctx.check(self.lib.hc_world_unload(self.handle, pos.ctypes.data, len(pos), stream), "hc_world_unload")

    def set_cluster(self, ctas_per_chunk: int):
        """CTAs (SMs) that mesh one chunk together in remesh: 1, 2, 4 or 8."""
        self.ctx.check(self.lib.hc_world_set_cluster(self.handle, ctas_per_chunk), "hc_world_set_cluster")

    def touch(self, stream=None):
        """Rebuilds every resident chunk's light planes (after writing the pool directly)."""
        self.ctx.check(self.lib.hc_world_touch(self.handle, stream), "hc_world_touch")

    def remesh(self, arena: batch.Arena, stream=None, partial: bool = False):
        """Relights + meshes the marked chunks into arena; returns (cells, quads, meshes). With
        partial=True a full arena is not an error: returns (cells, quads, meshes, status) where
        status[i] != 0 marks a chunk that did not fit (it stays marked for the next call)."""
        from .mesher import HcError, HC_ERR_CAPACITY
        cells = np.empty(self.world.n_chunks, np.int32)
        n, q, m = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint32()
        a = arena.c()
        st = self.lib.hc_world_remesh(self.handle, ctypes.byref(a), cells.ctypes.data, len(cells), ctypes.byref(n),
                                      ctypes.byref(q), ctypes.byref(m), stream)
        if not (partial and st == HC_ERR_CAPACITY):
            self.ctx.check(st, "hc_world_remesh")
        cells = cells[:n.value].copy()
        if not partial:
            return cells, q.value, m.value
        status = arena.results_host(len(cells))[:, 4].copy()
        return cells, q.value, m.value, status

    def download(self):
        return batch.pool_download(self.pool, 0, self.world.n_chunks)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hc_world_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def edit_world(seed: int = 12314524):
    """Edit workload: 7 x 5 x 7 chunks of the single-chunk terrain (chunk y -2..2) so every edited
    chunk has its neighbours."""
    from . import worldgen
    return worldgen.generate(7, 5, 7, (-3, -2, -3), seed=seed, caves=False, leaves_permille=50)


def seeded_edits(n: int = 4096, seed: int = 7, centre=(16, 16, 16), radius: int = 48) -> np.ndarray:
    """n edits uniform in the ball of `radius` voxels around `centre`: half place stone (1), half set
    air (0), and 10% of all edits place glowstone (24) instead."""
    rng = np.random.default_rng(seed)
    pts = []
    while sum(len(p) for p in pts) < n:
        c = rng.integers(-radius, radius + 1, size=(4 * n, 3))
        pts.append(c[(c ** 2).sum(1) <= radius * radius])
    p = np.concatenate(pts)[:n] + np.asarray(centre)
    kind = rng.random(n)
    block = np.where(kind < 0.5, 1, 0).astype(np.uint32)
    block[rng.random(n) < 0.1] = 24
    out = np.empty(n, EDIT_DTYPE)
    out["x"], out["y"], out["z"], out["block"] = p[:, 0], p[:, 1], p[:, 2], block
    return out
