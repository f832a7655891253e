"""Python mirror of the reference's chunk mesh task, backed by the CUDA library.

The reference runs ``ChunkTaskRunner<ChunkTaskType::kMesh>::Run`` (client/src/ChunkMeshTask.cpp:41-127)
on a ``ChunkTaskRunnerData<kMesh>`` holding the 27 neighbour chunks (client/include/client/
ChunkMeshTask.inl:17-29) and pushes the resulting ``std::vector<BlockMesh>`` to the renderer.
``MeshTaskRunner.run`` takes the same 27 chunks and returns the same list of ``BlockMesh``.

Every computation goes through ``libhc_gb300.so`` (include/hc_gb300.h); there is no CPU path. If
the library or a usable GPU is missing, construction raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from ._paths import lib_path

HC_OK, HC_ERR_INVALID_ARG, HC_ERR_OUT_OF_MEMORY, HC_ERR_CAPACITY, HC_ERR_DEVICE_TIMEOUT, HC_ERR_CUDA, HC_ERR_NO_DEVICE = range(7)
CHUNK_MAX_QUADS = 720896
CHUNK_MAX_MESHES = 96

MESH_DESC_DTYPE = np.dtype([("vertex_offset", "<u4"), ("vertex_count", "<u4"), ("index_offset", "<u4"),
                            ("index_count", "<u4"), ("aabb_min", "<u4", 3), ("aabb_max", "<u4", 3),
                            ("transparent", "<u4"), ("chunk", "<u4")])
assert MESH_DESC_DTYPE.itemsize == 48


class HcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hc status {status}: {message}")
        self.status = status


class _ChunkMesh(ctypes.Structure):
    _fields_ = [("mesh_capacity", ctypes.c_uint32), ("vertex_capacity", ctypes.c_uint32),
                ("index_capacity", ctypes.c_uint32), ("mesh_count", ctypes.c_uint32),
                ("vertex_count", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("meshes", ctypes.c_void_p), ("vertices", ctypes.c_void_p), ("indices", ctypes.c_void_p)]


_lib = None


def library() -> ctypes.CDLL:
    """Loads the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        path = lib_path("libhc_gb300.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        lib.hc_status_string.restype = ctypes.c_char_p
        lib.hc_status_string.argtypes = [ctypes.c_int]
        lib.hc_last_error.restype = ctypes.c_char_p
        lib.hc_last_error.argtypes = [vp]
        lib.hc_ctx_create.argtypes = [ctypes.c_int, P(vp)]
        lib.hc_ctx_destroy.argtypes = [vp]
        lib.hc_ctx_destroy.restype = None
        for name in ("hc_mesh_chunk", "hc_mesh_chunk_device"):
            f = getattr(lib, name)
            f.argtypes = [vp, vp, vp, P(_ChunkMesh), vp]
        lib.hc_relight_chunk_device.argtypes = [vp, vp, vp, vp, vp]
        _lib = lib
    return _lib


@dataclass
class BlockMesh:
    """client/include/client/BlockVertex.hpp:20-25: packed vertices (n, 2) uint32, uint16 indices,
    uint32 AABB in 1/16-voxel units (min xyz, max xyz) and the transparent flag."""
    vertices: np.ndarray
    indices: np.ndarray
    aabb: tuple
    transparent: bool

    def __eq__(self, o) -> bool:
        return (bool(self.transparent) == bool(o.transparent) and tuple(self.aabb) == tuple(o.aabb)
                and np.array_equal(self.vertices, o.vertices) and np.array_equal(self.indices, o.indices))


def meshes_from_descs(descs: np.ndarray, vertices: np.ndarray, indices: np.ndarray) -> list:
    out = []
    for d in descs:
        vo, vc, io, ic = int(d["vertex_offset"]), int(d["vertex_count"]), int(d["index_offset"]), int(d["index_count"])
        out.append(BlockMesh(vertices[vo:vo + vc].copy(), indices[io:io + ic].copy(),
                             tuple(int(x) for x in d["aabb_min"]) + tuple(int(x) for x in d["aabb_max"]),
                             bool(d["transparent"])))
    return out


class Context:
    """A device context (block tables + single-chunk buffers) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = library()
        h = ctypes.c_void_p()
        st = self.lib.hc_ctx_create(device, ctypes.byref(h))
        if st != HC_OK:
            raise HcError(st, f"hc_ctx_create({device}) failed: {self.lib.hc_status_string(st).decode()}")
        self.handle = h
        self.device = device
        self._verts = np.empty((CHUNK_MAX_QUADS * 4, 2), np.uint32)
        self._idx = np.empty(CHUNK_MAX_QUADS * 6, np.uint16)
        self._descs = np.empty(CHUNK_MAX_MESHES, MESH_DESC_DTYPE)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hc_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def check(self, st: int, what: str):
        if st != HC_OK:
            msg = self.lib.hc_last_error(self.handle).decode()
            raise HcError(st, f"{what}: {self.lib.hc_status_string(st).decode()}: {msg}")

    @staticmethod
    def _ptr_arrays(blocks27, heights27):
        b = (ctypes.c_void_p * 27)(*[int(x) for x in blocks27])
        h = (ctypes.c_void_p * 27)(*[int(x) for x in heights27])
        return b, h

    def mesh_chunk(self, blocks27, heights27) -> list:
        """Host arrays in, list of BlockMesh out (reference order)."""
        blocks27 = [np.ascontiguousarray(x, np.uint16) for x in blocks27]
        heights27 = [np.ascontiguousarray(x, np.int8) for x in heights27]
        assert len(blocks27) == 27 and len(heights27) == 27
        b, h = self._ptr_arrays([x.ctypes.data for x in blocks27], [x.ctypes.data for x in heights27])
        out = _ChunkMesh(CHUNK_MAX_MESHES, CHUNK_MAX_QUADS * 4, CHUNK_MAX_QUADS * 6, 0, 0, 0,
                         self._descs.ctypes.data, self._verts.ctypes.data, self._idx.ctypes.data)
        self.check(self.lib.hc_mesh_chunk(self.handle, b, h, ctypes.byref(out), None), "hc_mesh_chunk")
        return meshes_from_descs(self._descs[:out.mesh_count], self._verts, self._idx)

    def mesh_chunk_device(self, block_ptrs, height_ptrs, verts_ptr, vcap, idx_ptr, icap, desc_ptr, mcap, stream=None):
        """Device pointers in and out; returns (mesh_count, vertex_count, index_count)."""
        b, h = self._ptr_arrays(block_ptrs, height_ptrs)
        out = _ChunkMesh(mcap, vcap, icap, 0, 0, 0, desc_ptr, verts_ptr, idx_ptr)
        st = self.lib.hc_mesh_chunk_device(self.handle, b, h, ctypes.byref(out), stream)
        self.check(st, "hc_mesh_chunk_device")
        return out.mesh_count, out.vertex_count, out.index_count

    def relight_chunk_device(self, block_ptrs, height_ptrs, light_ptr, stream=None):
        b, h = self._ptr_arrays(block_ptrs, height_ptrs)
        self.check(self.lib.hc_relight_chunk_device(self.handle, b, h, light_ptr, stream), "hc_relight_chunk_device")


@dataclass
class MeshTaskData:
    """ChunkTaskRunnerData<kMesh>: the 27 chunks (blocks, sunlight heights) in neighbour order."""
    blocks: list
    heights: list

    @classmethod
    def from_world(cls, world, ix: int, iy: int, iz: int) -> "MeshTaskData":
        nb = world.neighbours(ix, iy, iz)
        if (nb < 0).any():
            raise ValueError("a mesh task needs all 26 neighbours")
        return cls([world.blocks[i] for i in nb], [world.heights[i] for i in nb])


class MeshTaskRunner:
    """ChunkTaskRunner<kMesh>: relights the centre chunk's window and meshes it on the GPU."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or Context()

    def run(self, data: MeshTaskData) -> list:
        return self.ctx.mesh_chunk(data.blocks, data.heights)
