"""Request server over a device-resident world, and the seeded serving workload.

Python side of include/hc_gb300.h's hc_server_* entry points, which replace the reference's chunk
task scheduling (client/src/ChunkTaskPool.cpp:16-130, client/src/WorldWorker.cpp:18-27) and its
chunk loader (client/src/LocalClient.cpp:14-27): edits, 16^3 region fills, chunk loads and
unloads are batched into fixed ticks, each one device pass of unloads -> loads -> edits ->
sunlight heights -> relight + remesh.

The workload (``serving_trace``): Poisson arrivals; 70% single-block edits within 48 voxels of a
player, 25% loads of the chunks entering a view sphere of radius 16 chunks as the player takes a
seeded random walk (the chunks leaving it are unloaded first), 5% fills of a 16^3 region near the
player. Chunk contents come from a seeded library of the 30/20/35/10/5 mixture of air, stone,
terrain, random-fill and checkerboard chunks.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import batch
from .mesher import BlockMesh, Context, HcError, MESH_DESC_DTYPE, library

REQ_EDIT, REQ_FILL, REQ_LOAD, REQ_UNLOAD = 0, 1, 2, 3

REQUEST_DTYPE = np.dtype({"names": ["kind", "block", "x", "y", "z", "size", "blocks", "heights", "tag", "block_entries",
                                    "sunlight_entries", "n_block_entries", "n_sunlight_entries"],
                          "formats": ["<u4", "<u4", "<i4", "<i4", "<i4", "<u4", "<u8", "<u8", "<u8", "<u8", "<u8", "<u4",
                                      "<u4"],
                          "offsets": [0, 4, 8, 12, 16, 20, 24, 32, 40, 48, 56, 64, 68], "itemsize": 72})
COMPLETION_DTYPE = np.dtype({"names": ["tag", "kind", "status", "tick", "submit_ns", "done_ns"],
                             "formats": ["<u8", "<u4", "<u4", "<u8", "<u8", "<u8"],
                             "offsets": [0, 8, 12, 16, 24, 32], "itemsize": 40})


class _Desc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("nx", "ny", "nz", "cx0", "cy0", "cz0")]


class ServerConfig(ctypes.Structure):
    _fields_ = [("tick_us", ctypes.c_uint32), ("depth", ctypes.c_uint32), ("max_edits_per_tick", ctypes.c_uint32),
                ("max_loads_per_tick", ctypes.c_uint32), ("arena_quads", ctypes.c_uint64),
                ("arena_meshes", ctypes.c_uint32), ("ctas_per_chunk", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("ticks", "requests_done", "requests_rejected", "chunks_remeshed",
                                               "chunks_requeued", "quads", "edits", "loads", "unloads",
                                               "gpu_ns_total", "gpu_ns_max")] + \
               [(n, ctypes.c_uint32) for n in ("pool_capacity", "resident", "free_slots", "queued")]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


SINK = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                        ctypes.c_uint32)

# MeshInfo<ChunkMeshInfo> (client/include/client/mesh/MeshInfo.hpp:9-12, ChunkMesh.hpp:12-18)
MESH_INFO_DTYPE = np.dtype([("index_count", "<u4"), ("first_index", "<u4"), ("vertex_offset", "<u4"),
                            ("aabb_min", "<f4", 3), ("aabb_max", "<f4", 3), ("base_position", "<i4", 3),
                            ("transparent", "<u4")])


def mesh_info_of(desc, chunk_pos) -> np.void:
    """Host restatement of WorldRenderer::PushChunkMesh's record (WorldRenderer.hpp:69-87):
    (fAABB)aabb / 16 + base, in float32."""
    out = np.zeros(1, MESH_INFO_DTYPE)[0]
    base = np.asarray(chunk_pos, np.int32) * 32
    out["index_count"], out["first_index"], out["vertex_offset"] = desc["index_count"], desc["index_offset"], \
        desc["vertex_offset"]
    out["aabb_min"] = np.asarray(desc["aabb_min"], np.uint32).astype(np.float32) / np.float32(16) + base.astype(np.float32)
    out["aabb_max"] = np.asarray(desc["aabb_max"], np.uint32).astype(np.float32) / np.float32(16) + base.astype(np.float32)
    out["base_position"] = base
    out["transparent"] = desc["transparent"]
    return out


def _bind(lib):
    if getattr(lib, "_server_bound", False):
        return lib
    vp, P, u32, u64 = ctypes.c_void_p, ctypes.POINTER, ctypes.c_uint32, ctypes.c_uint64
    lib.hc_server_create.argtypes = [vp, P(_Desc), u32, P(ServerConfig), P(vp)]
    lib.hc_server_destroy.argtypes = [vp]
    lib.hc_server_destroy.restype = None
    lib.hc_server_submit.argtypes = [vp, vp, u32]
    lib.hc_server_start.argtypes = [vp]
    lib.hc_server_stop.argtypes = [vp]
    lib.hc_server_step.argtypes = [vp, P(u32)]
    lib.hc_server_poll.argtypes = [vp, vp, u32, P(u32)]
    lib.hc_server_get_stats.argtypes = [vp, P(ServerStats)]
    lib.hc_server_set_sink.argtypes = [vp, SINK, vp]
    lib.hc_server_resident.argtypes = [vp, vp]
    lib.hc_server_pool.argtypes = [vp]
    lib.hc_server_pool.restype = vp
    lib.hc_server_replay.argtypes = [vp, vp, vp, u32, vp, vp, P(u64)]
    lib._server_bound = True
    return lib


class Server:
    """A request server over an empty nx x ny x nz chunk grid whose cell (0, 0, 0) is chunk origin."""

    def __init__(self, ctx: Context, grid, origin, *, pool_capacity: int = 0, tick_us: int = 1000, depth: int = 3,
                 max_edits_per_tick: int = 16384, max_loads_per_tick: int = 256, arena_quads: int = 4 << 20,
                 arena_meshes: int = 1 << 15, ctas_per_chunk: int = 0):
        self.ctx = ctx
        self.lib = _bind(batch._bind(library()))
        self.grid, self.origin = tuple(grid), tuple(origin)
        self.cfg = ServerConfig(tick_us, depth, max_edits_per_tick, max_loads_per_tick, arena_quads, arena_meshes,
                                ctas_per_chunk)
        h = ctypes.c_void_p()
        ctx.check(self.lib.hc_server_create(ctx.handle, ctypes.byref(_Desc(*self.grid, *self.origin)), pool_capacity,
                                            ctypes.byref(self.cfg), ctypes.byref(h)), "hc_server_create")
        self.handle = h
        self._sink = None
        self._keep = []  # load data referenced by queued requests

    @property
    def n_cells(self) -> int:
        return self.grid[0] * self.grid[1] * self.grid[2]

    def cell(self, cx, cy, cz) -> int:
        ix, iy, iz = cx - self.origin[0], cy - self.origin[1], cz - self.origin[2]
        return ix + self.grid[0] * (iz + self.grid[2] * iy)

    def cell_pos(self, cell: int) -> tuple:
        nx, nz = self.grid[0], self.grid[2]
        return (self.origin[0] + cell % nx, self.origin[1] + cell // (nx * nz), self.origin[2] + (cell // nx) % nz)

    def submit(self, reqs: np.ndarray):
        r = np.ascontiguousarray(reqs, REQUEST_DTYPE)
        self.ctx.check(self.lib.hc_server_submit(self.handle, r.ctypes.data, len(r)), "hc_server_submit")

    def start(self):
        self.ctx.check(self.lib.hc_server_start(self.handle), "hc_server_start")

    def stop(self):
        self.ctx.check(self.lib.hc_server_stop(self.handle), "hc_server_stop")

    def step(self) -> int:
        n = ctypes.c_uint32()
        self.ctx.check(self.lib.hc_server_step(self.handle, ctypes.byref(n)), "hc_server_step")
        return n.value

    def drain(self, max_steps: int = 100000) -> int:
        """Steps (threads stopped) until nothing is queued and no chunk is marked."""
        steps = 0
        while steps < max_steps:
            st = self.stats()
            if self.step() == 0 and st["queued"] == 0 and self.stats()["ticks"] == st["ticks"]:
                return steps
            steps += 1
        raise RuntimeError("server did not drain")

    def poll(self, cap: int = 1 << 16) -> np.ndarray:
        out = np.empty(cap, COMPLETION_DTYPE)
        n = ctypes.c_uint32()
        self.ctx.check(self.lib.hc_server_poll(self.handle, out.ctypes.data, cap, ctypes.byref(n)), "hc_server_poll")
        return out[:n.value].copy()

    def stats(self) -> dict:
        s = ServerStats()
        self.ctx.check(self.lib.hc_server_get_stats(self.handle, ctypes.byref(s)), "hc_server_get_stats")
        return s.as_dict()

    def resident(self) -> np.ndarray:
        out = np.empty(self.n_cells, np.int32)
        self.ctx.check(self.lib.hc_server_resident(self.handle, out.ctypes.data), "hc_server_resident")
        return out

    def download(self, cells):
        """(blocks, heights) of the given resident grid cells (server idle)."""
        slots = self.resident()[np.asarray(cells, np.int64)]
        if (slots < 0).any():
            raise ValueError("cell not resident")
        lib = self.lib
        pool = lib.hc_server_pool(self.handle)
        b = np.empty((len(slots), 32768), np.uint16)
        h = np.empty((len(slots), 1024), np.int8)
        for i, s in enumerate(slots):
            self.ctx.check(lib.hc_pool_download(pool, int(s), 1, b[i].ctypes.data, h[i].ctypes.data, 0, None),
                           "hc_pool_download")
        return b, h

    def set_sink(self, fn):
        """fn(tick, cells (n,) int32, meshes_by_position list of lists of BlockMesh, status (n,)) on
        the completion thread after every pass; None removes it."""
        if fn is None:
            self._sink = None
            self.ctx.check(self.lib.hc_server_set_sink(self.handle, SINK(), None), "hc_server_set_sink")
            return

        def cb(_user, tick, n, cells_p, results_p, verts_p, idx_p, meshes_p, infos_p, quads, mesh_count):
            cells = np.ctypeslib.as_array(ctypes.cast(cells_p, ctypes.POINTER(ctypes.c_int32)), (n,)).copy() if n else \
                np.empty(0, np.int32)
            res = np.ctypeslib.as_array(ctypes.cast(results_p, ctypes.POINTER(ctypes.c_uint32)), (n * 5,)).reshape(-1, 5) \
                if n else np.empty((0, 5), np.uint32)
            verts = np.ctypeslib.as_array(ctypes.cast(verts_p, ctypes.POINTER(ctypes.c_uint32)),
                                          (quads * 8,)).reshape(-1, 2) if quads else np.empty((0, 2), np.uint32)
            idx = np.ctypeslib.as_array(ctypes.cast(idx_p, ctypes.POINTER(ctypes.c_uint16)), (quads * 6,)) if quads \
                else np.empty(0, np.uint16)
            md = np.frombuffer(ctypes.string_at(meshes_p, mesh_count * MESH_DESC_DTYPE.itemsize), MESH_DESC_DTYPE) \
                if mesh_count else np.empty(0, MESH_DESC_DTYPE)
            mi = np.frombuffer(ctypes.string_at(infos_p, mesh_count * MESH_INFO_DTYPE.itemsize), MESH_INFO_DTYPE) \
                if mesh_count else np.empty(0, MESH_INFO_DTYPE)
            per_chunk = []
            for i in range(n):
                r = res[i]
                if r[4] != 0:
                    per_chunk.append(None)
                    continue
                ms = []
                for d in md[int(r[2]):int(r[2]) + int(r[3])]:
                    vo, vc, io, ic = (int(d[k]) for k in ("vertex_offset", "vertex_count", "index_offset", "index_count"))
                    ms.append(BlockMesh(verts[vo:vo + vc].copy(), idx[io:io + ic].copy(),
                                        tuple(int(x) for x in d["aabb_min"]) + tuple(int(x) for x in d["aabb_max"]),
                                        bool(d["transparent"])))
                per_chunk.append(ms)
            if getattr(fn, "wants_infos", False):
                fn(int(tick), cells, per_chunk, res[:, 4].copy(), md.copy(), mi.copy())
            else:
                fn(int(tick), cells, per_chunk, res[:, 4].copy())

        self._sink = SINK(cb)
        self.ctx.check(self.lib.hc_server_set_sink(self.handle, self._sink, None), "hc_server_set_sink")

    def replay(self, reqs: np.ndarray, arrival_ns: np.ndarray, with_ticks: bool = False):
        """Real-time replay of a timed trace on a started server: (latency_ns per request, elapsed_ns),
        plus the tick that admitted each request when with_ticks."""
        r = np.ascontiguousarray(reqs, REQUEST_DTYPE)
        a = np.ascontiguousarray(arrival_ns, np.uint64)
        lat = np.zeros(len(r), np.uint64)
        ticks = np.zeros(len(r), np.uint64) if with_ticks else None
        el = ctypes.c_uint64()
        self.ctx.check(self.lib.hc_server_replay(self.handle, r.ctypes.data, a.ctypes.data, len(r), lat.ctypes.data,
                                                 ticks.ctypes.data if with_ticks else None, ctypes.byref(el)),
                       "hc_server_replay")
        return (lat, el.value, ticks) if with_ticks else (lat, el.value)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


# ------------------------------------------------------------------------------------------------
# Seeded serving workload
# ------------------------------------------------------------------------------------------------

class ChunkLibrary:
    """Chunk contents for any position: a seeded library of mixture chunks, chunk (x, y, z) taking
    entry hash(x, y, z) mod size."""

    def __init__(self, nx: int = 16, ny: int = 8, nz: int = 16, seed: int = 0x5E7E):
        from . import worldgen
        w = worldgen.mixture_world(nx, ny, nz, seed=seed)
        inner = np.nonzero(~_ring_mask(w))[0]
        self.blocks = np.ascontiguousarray(w.blocks[inner])
        self.heights = np.ascontiguousarray(w.heights[inner])
        self.kinds = w.kinds[inner].copy()
        self.seed = seed

    def __len__(self):
        return len(self.blocks)

    def index(self, x: int, y: int, z: int) -> int:
        h = (x * 0x9E3779B1 + y * 0x85EBCA77 + z * 0xC2B2AE3D + self.seed) & 0xFFFFFFFF
        h ^= h >> 15
        h = (h * 0x2C1B3C6D) & 0xFFFFFFFF
        h ^= h >> 12
        return h % len(self.blocks)


def _ring_mask(w) -> np.ndarray:
    i = np.arange(w.n_chunks)
    ix, iz, iy = i % w.nx, (i // w.nx) % w.nz, i // (w.nx * w.nz)
    return (ix == 0) | (iy == 0) | (iz == 0) | (ix == w.nx - 1) | (iy == w.ny - 1) | (iz == w.nz - 1)


def sphere_offsets(radius: int) -> np.ndarray:
    r = np.arange(-radius, radius + 1)
    d = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    d2 = (d ** 2).sum(1)
    keep = d2 <= radius * radius
    d, d2 = d[keep], d2[keep]
    return d[np.argsort(d2, kind="stable")]  # nearest first, like the reference's loading list


def _load_req(lib: ChunkLibrary, pos, tag=0):
    r = np.zeros(1, REQUEST_DTYPE)
    k = lib.index(*pos)
    r["kind"], r["x"], r["y"], r["z"] = REQ_LOAD, pos[0], pos[1], pos[2]
    r["blocks"], r["heights"] = lib.blocks[k].ctypes.data, lib.heights[k].ctypes.data
    r["tag"] = tag
    return r[0]


class ServingWorkload:
    """Player walk, view sphere and request mixture over a grid of chunks.

    The grid is nx x ny x nz chunks from origin; the player walks in x/z (one chunk per move,
    seeded direction, kept `radius + 2` chunks from the grid's x/z edges) at a fixed chunk height.
    """

    def __init__(self, lib: ChunkLibrary, grid=(96, 32, 96), origin=(-48, -16, -48), radius: int = 16, seed: int = 1):
        self.lib, self.grid, self.origin, self.radius = lib, tuple(grid), tuple(origin), radius
        self.rng = np.random.default_rng(seed)
        self.player = np.array([origin[0] + grid[0] // 2, origin[1] + grid[1] // 2, origin[2] + grid[2] // 2])
        self.sphere = sphere_offsets(radius)
        self.resident = set()
        self.load_queue = []

    def in_grid(self, p) -> bool:
        return all(self.origin[a] <= p[a] < self.origin[a] + self.grid[a] for a in range(3))

    def view(self, centre) -> list:
        return [tuple(int(v) for v in centre + d) for d in self.sphere if self.in_grid(centre + d)]

    def initial_loads(self) -> np.ndarray:
        """Loads of the whole view sphere at the start position."""
        pos = self.view(self.player)
        self.resident = set(pos)
        return np.array([_load_req(self.lib, p) for p in pos], REQUEST_DTYPE)

    def _move(self) -> list:
        """Moves the player one chunk; returns the unload requests and queues the new loads."""
        lo = [self.origin[a] + self.radius + 2 for a in (0, 2)]
        hi = [self.origin[a] + self.grid[a] - self.radius - 3 for a in (0, 2)]
        for _ in range(8):
            d = [(1, 0), (-1, 0), (0, 1), (0, -1)][int(self.rng.integers(4))]
            nxp, nzp = self.player[0] + d[0], self.player[2] + d[1]
            if lo[0] <= nxp <= hi[0] and lo[1] <= nzp <= hi[1]:
                break
        else:
            nxp, nzp = self.player[0], self.player[2]
        self.player = np.array([nxp, self.player[1], nzp])
        view = set(self.view(self.player))
        gone = sorted(self.resident - view)
        new = [p for p in self.view(self.player) if p not in self.resident]
        self.resident = view
        self.load_queue.extend(new)
        out = []
        for p in gone:
            r = np.zeros(1, REQUEST_DTYPE)[0]
            r["kind"], r["x"], r["y"], r["z"] = REQ_UNLOAD, p[0], p[1], p[2]
            out.append(r)
        return out

    def _near_voxel(self, reach: int = 48):
        while True:
            d = self.rng.integers(-reach, reach + 1, size=3)
            if (d ** 2).sum() <= reach * reach:
                break
        return self.player * 32 + 16 + d

    def trace(self, rate: float, duration_s: float, edit_frac=0.70, load_frac=0.25):
        """(requests, arrival_ns): Poisson arrivals at `rate` per second for `duration_s`. Unloads
        of the chunks the player leaves go in just before the loads that follow the move (they
        are extra requests, outside the mixture)."""
        gaps = self.rng.exponential(1.0 / rate, size=int(rate * duration_s * 1.2) + 16)
        t = np.cumsum(gaps)
        t = t[t < duration_s]
        reqs, times = [], []
        for ti in t:
            u = self.rng.random()
            ns = int(ti * 1e9)
            if u < edit_frac:
                v = self._near_voxel()
                r = np.zeros(1, REQUEST_DTYPE)[0]
                b = self.rng.random()
                r["kind"], r["x"], r["y"], r["z"] = REQ_EDIT, v[0], v[1], v[2]
                r["block"] = 24 if b < 0.1 else (1 if b < 0.55 else 0)
                reqs.append(r)
                times.append(ns)
            elif u < edit_frac + load_frac:
                while not self.load_queue:
                    for r in self._move():
                        reqs.append(r)
                        times.append(ns)
                reqs.append(_load_req(self.lib, self.load_queue.pop(0)))
                times.append(ns)
            else:
                v = self._near_voxel() - 8
                r = np.zeros(1, REQUEST_DTYPE)[0]
                r["kind"], r["x"], r["y"], r["z"], r["size"] = REQ_FILL, v[0], v[1], v[2], 16
                r["block"] = [1, 0, 9][int(self.rng.integers(3))]
                reqs.append(r)
                times.append(ns)
        out = np.array(reqs, REQUEST_DTYPE)
        out["tag"] = np.arange(len(out))
        return out, np.array(times, np.uint64)
