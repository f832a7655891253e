"""Device chunk pool and batched meshing (Python side of include/hc_gb300.h's pool/plan entry points).

The reference meshes chunks one task at a time on worker threads (client/src/ChunkTaskPool.cpp:87-130,
client/src/WorldWorker.cpp:18-27). Here the chunks live in a device pool and a batch plan meshes a
list of them in one persistent work-stealing kernel replayed as a CUDA graph (or, for comparison,
with one kernel launch per chunk). torch provides device memory only.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from .mesher import HC_OK, HcError, MESH_DESC_DTYPE, BlockMesh, Context, library

PERSISTENT, PER_CHUNK, AUTO = 0, 1, 2


def variant_mode(v: int) -> int:
    """Mode that builds persistent variant v alone (HC_BATCH_VARIANT)."""
    return 16 + v


VARIANTS = ("light pass, one CTA per chunk", "window relight, one CTA per chunk", "window relight, 2-CTA clusters",
            "window relight, 4-CTA clusters", "light pass, 2 chunks per claim", "light pass, 4 chunks per claim",
            "light pass, no global record scratch (windowed emission)")
LIGHT_PASS_VARIANTS = (0, 4, 5, 6)


def launches_per_run(v: int) -> int:
    """Kernels one run of persistent variant v launches: plane refresh, blank test (one CTA per
    chunk), 15 light levels (light-pass variants) and the mesher."""
    return 18 if v in LIGHT_PASS_VARIANTS else (3 if v == 1 else 2)


RESULT_OK, RESULT_ARENA_FULL, RESULT_BAD_SLOT = 0, 1, 2


class _Arena(ctypes.Structure):
    _fields_ = [("quad_capacity", ctypes.c_uint64), ("mesh_capacity", ctypes.c_uint32),
                ("vertices", ctypes.c_void_p), ("indices", ctypes.c_void_p), ("meshes", ctypes.c_void_p),
                ("results", ctypes.c_void_p)]


def _bind(lib):
    if getattr(lib, "_batch_bound", False):
        return lib
    vp, P = ctypes.c_void_p, ctypes.POINTER
    lib.hc_pool_create.argtypes = [vp, ctypes.c_uint32, P(vp)]
    lib.hc_pool_download.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, ctypes.c_int, vp]
    lib.hc_pool_destroy.argtypes = [vp]
    lib.hc_pool_destroy.restype = None
    lib.hc_pool_capacity.argtypes = [vp]
    lib.hc_pool_capacity.restype = ctypes.c_uint32
    lib.hc_pool_buffers.argtypes = [vp, P(vp), P(vp)]
    lib.hc_pool_upload.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, ctypes.c_int, vp]
    lib.hc_batch_plan_create.argtypes = [vp, vp, vp, ctypes.c_uint32, P(_Arena), ctypes.c_int, ctypes.c_int, P(vp)]
    lib.hc_batch_plan_destroy.argtypes = [vp]
    lib.hc_batch_plan_destroy.restype = None
    lib.hc_batch_plan_launch.argtypes = [vp, vp]
    lib.hc_batch_plan_result.argtypes = [vp, P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint32)]
    lib.hc_batch_plan_download.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint32, vp, vp, vp, vp]
    lib.hc_batch_plan_download_async.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint32, vp, vp, vp, vp, vp]
    lib.hc_batch_plan_variant.argtypes = [vp, P(ctypes.c_int), vp]
    lib.hc_batch_plan_stage_ms.argtypes = [vp, vp]
    lib._batch_bound = True
    return lib


class Pool:
    """`capacity` resident chunk slots on the context's device."""

    def __init__(self, ctx: Context, capacity: int):
        self.ctx, self.lib = ctx, _bind(library())
        h = ctypes.c_void_p()
        ctx.check(self.lib.hc_pool_create(ctx.handle, capacity, ctypes.byref(h)), "hc_pool_create")
        self.handle, self.capacity = h, capacity
        b, hh = ctypes.c_void_p(), ctypes.c_void_p()
        ctx.check(self.lib.hc_pool_buffers(h, ctypes.byref(b), ctypes.byref(hh)), "hc_pool_buffers")
        self.blocks_ptr, self.heights_ptr = b.value, hh.value

    def upload(self, first: int, blocks, heights, stream=None):
        """blocks (n, 32768) uint16 and heights (n, 1024) int8: numpy (host) or torch cuda tensors."""
        on_dev = hasattr(blocks, "data_ptr")
        if on_dev:
            bp, hp, n = blocks.data_ptr(), heights.data_ptr(), blocks.shape[0]
        else:
            blocks = np.ascontiguousarray(blocks, np.uint16)
            heights = np.ascontiguousarray(heights, np.int8)
            bp, hp, n = blocks.ctypes.data, heights.ctypes.data, blocks.shape[0]
        self.ctx.check(self.lib.hc_pool_upload(self.handle, first, n, bp, hp, int(on_dev), stream), "hc_pool_upload")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hc_pool_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


class Arena:
    """Device buffers (torch) receiving a batch's meshes."""

    def __init__(self, quad_capacity: int, mesh_capacity: int, n_chunks: int, device: int = 0):
        import torch
        dev = torch.device("cuda", device)
        self.quad_capacity, self.mesh_capacity, self.n = int(quad_capacity), int(mesh_capacity), int(n_chunks)
        self.vertices = torch.empty(self.quad_capacity * 8, dtype=torch.int32, device=dev)
        self.indices = torch.empty(self.quad_capacity * 6 + 2, dtype=torch.int16, device=dev)
        self.meshes = torch.empty(self.mesh_capacity * 12, dtype=torch.int32, device=dev)
        self.results = torch.empty(self.n * 5, dtype=torch.int32, device=dev)

    def c(self) -> _Arena:
        return _Arena(self.quad_capacity, self.mesh_capacity, self.vertices.data_ptr(), self.indices.data_ptr(),
                      self.meshes.data_ptr(), self.results.data_ptr())

    def chunk_meshes(self, i: int, host=None) -> list:
        """The meshes of batch position i, in reference order (reads the arena back)."""
        res = (host or self.host())
        r = res["results"][5 * i:5 * i + 5]
        if r[4] != RESULT_OK:
            raise HcError(int(r[4]), f"chunk {i} status {int(r[4])}")
        descs = res["meshes"][int(r[2]):int(r[2]) + int(r[3])]
        out = []
        for d in descs:
            vo, vc, io, ic = (int(d[k]) for k in ("vertex_offset", "vertex_count", "index_offset", "index_count"))
            out.append(BlockMesh(res["vertices"][vo:vo + vc].copy(), res["indices"][io:io + ic].copy(),
                                 tuple(int(x) for x in d["aabb_min"]) + tuple(int(x) for x in d["aabb_max"]),
                                 bool(d["transparent"])))
        return out

    def sample_meshes(self, positions) -> dict:
        """{batch position: its meshes} for the given positions, reading back only their descriptor
        and vertex/index ranges (a full-size arena holds gigabytes)."""
        n = self.n
        res = self.results[:5 * n].cpu().numpy().view(np.uint32).reshape(-1, 5)
        out = {}
        for i in positions:
            r = res[int(i)]
            if r[4] != RESULT_OK:
                raise HcError(int(r[4]), f"chunk {int(i)} status {int(r[4])}")
            d0, dn = int(r[2]), int(r[3])
            descs = self.meshes[12 * d0:12 * (d0 + dn)].cpu().numpy().view(MESH_DESC_DTYPE)
            meshes = []
            for d in descs:
                vo, vc, io, ic = (int(d[k]) for k in ("vertex_offset", "vertex_count", "index_offset", "index_count"))
                v = self.vertices[2 * vo:2 * (vo + vc)].cpu().numpy().view(np.uint32).reshape(-1, 2)
                ix = self.indices[io:io + ic].cpu().numpy().view(np.uint16)
                meshes.append(BlockMesh(v, ix, tuple(int(x) for x in d["aabb_min"]) + tuple(int(x) for x in d["aabb_max"]),
                                        bool(d["transparent"])))
            out[int(i)] = meshes
        return out

    def results_host(self, n: int) -> np.ndarray:
        """The first n chunks' result words, (n, 5) uint32."""
        return self.results[:5 * n].cpu().numpy().view(np.uint32).reshape(-1, 5)

    def host(self) -> dict:
        return {"vertices": self.vertices.cpu().numpy().view(np.uint32).reshape(-1, 2),
                "indices": self.indices.cpu().numpy().view(np.uint16),
                "meshes": self.meshes.cpu().numpy().view(MESH_DESC_DTYPE),
                "results": self.results.cpu().numpy().view(np.uint32)}


class BatchPlan:
    """Meshes the chunks named by a (n, 27) neighbour slot table into an Arena."""

    def __init__(self, ctx: Context, pool: Pool, neighbours, arena: Arena, mode: int = PERSISTENT, ctas_per_sm: int = 0):
        import torch
        self.ctx, self.lib, self.pool, self.arena = ctx, _bind(library()), pool, arena
        self.neighbours = torch.as_tensor(np.ascontiguousarray(neighbours, np.int32)).to(
            torch.device("cuda", ctx.device)) if not hasattr(neighbours, "data_ptr") else neighbours
        self.n = int(self.neighbours.shape[0])
        assert self.n == arena.n
        self._arena_c = arena.c()
        h = ctypes.c_void_p()
        ctx.check(self.lib.hc_batch_plan_create(ctx.handle, pool.handle, self.neighbours.data_ptr(), self.n,
                                                ctypes.byref(self._arena_c), mode, ctas_per_sm, ctypes.byref(h)),
                  "hc_batch_plan_create")
        self.handle = h

    def launch(self, stream=None):
        self.ctx.check(self.lib.hc_batch_plan_launch(self.handle, stream), "hc_batch_plan_launch")

    def variant(self):
        """(variant index, its description, ms per variant as timed by the autotuner)."""
        v = ctypes.c_int()
        ms = np.zeros(len(VARIANTS), np.float32)
        self.lib.hc_batch_plan_variant(self.handle, ctypes.byref(v), ms.ctypes.data)
        return v.value, VARIANTS[v.value], [float(x) for x in ms]

    def stage_ms(self):
        """Device time of the last launch's stages (waits for it): plane refresh, light pass, meshing."""
        ms = np.zeros(3, np.float32)
        self.ctx.check(self.lib.hc_batch_plan_stage_ms(self.handle, ms.ctypes.data), "hc_batch_plan_stage_ms")
        return [float(x) for x in ms]

    def result(self, check: bool = True):
        """(quads, meshes, failed chunks) of the last launch (waits for it)."""
        q, m, f = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        st = self.lib.hc_batch_plan_result(self.handle, ctypes.byref(q), ctypes.byref(m), ctypes.byref(f))
        if check and st != HC_OK:
            self.ctx.check(st, "hc_batch_plan_result")
        return q.value, m.value, f.value

    def download(self, quads: int, meshes: int, vertices: np.ndarray, indices: np.ndarray, descs: np.ndarray,
                 results: np.ndarray):
        self.ctx.check(self.lib.hc_batch_plan_download(
            self.handle, quads, meshes, vertices.ctypes.data if vertices is not None else None,
            indices.ctypes.data if indices is not None else None, descs.ctypes.data if descs is not None else None,
            results.ctypes.data if results is not None else None), "hc_batch_plan_download")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hc_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


@dataclass
class ResidentWorld:
    """A generated world uploaded to a device pool (slot = chunk index)."""
    world: object
    pool: Pool
    chunks: np.ndarray       # batch order -> chunk index
    neighbours: np.ndarray   # (n, 27) slots


def upload_world(ctx: Context, world, chunks=None) -> ResidentWorld:
    pool = Pool(ctx, world.n_chunks)
    pool.upload(0, world.blocks, world.heights)
    chunks = world.meshable() if chunks is None else np.asarray(chunks, np.int32)
    return ResidentWorld(world, pool, chunks, world.neighbour_table(chunks))


def pool_download(pool: Pool, first: int, count: int):
    """Blocks (count, 32768) uint16 and heights (count, 1024) int8 of slots [first, first+count)."""
    lib = _bind(library())
    b = np.empty((count, 32768), np.uint16)
    h = np.empty((count, 1024), np.int8)
    pool.ctx.check(lib.hc_pool_download(pool.handle, first, count, b.ctypes.data, h.ctypes.data, 0, None),
                   "hc_pool_download")
    return b, h
