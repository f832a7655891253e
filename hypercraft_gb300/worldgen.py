"""Seeded synthetic chunk grids for the relight + mesh path (host-side, no GPU).

Thin ctypes wrapper over ``csrc/hc_worldgen.cpp``. A grid holds ``nx * ny * nz`` chunks; chunk
``(ix, iy, iz)`` is stored at index ``ix + nx * (iz + nz * iy)`` with the reference's own chunk
layout: 32^3 uint16 blocks indexed ``x + (y*32 + z)*32`` and 32^2 int8 sunlight heights indexed
``x + z*32`` (client/include/client/Chunk.hpp:95-96).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from ._paths import lib_path

KIND_AIR, KIND_STONE, KIND_TERRAIN, KIND_RANDOM, KIND_CHECKER = range(5)
WORLD_SEED = 12314524  # the reference client's terrain seed (client/src/LocalClient.cpp:37)


class _Grid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("nx", "ny", "nz", "cx0", "cy0", "cz0")]


class _Params(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("caves", ctypes.c_int32), ("leaves_permille", ctypes.c_int32),
                ("air_ring", ctypes.c_int32), ("mixture", ctypes.c_int32), ("default_kind", ctypes.c_int32)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = lib_path("libhc_worldgen.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        P = ctypes.POINTER
        lib.hcw_assign_kinds.argtypes = [P(_Grid), P(_Params), ctypes.c_void_p]
        lib.hcw_generate.argtypes = [P(_Grid), P(_Params), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.hcw_recompute_heights.argtypes = [P(_Grid), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_int]
        lib.hcw_neighbours.argtypes = [P(_Grid), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        _lib = lib
    return _lib


@dataclass
class World:
    """A chunk grid: blocks (n, 32768) uint16, heights (n, 1024) int8, kinds (n,) uint8."""
    nx: int
    ny: int
    nz: int
    origin: tuple
    blocks: np.ndarray
    heights: np.ndarray
    kinds: np.ndarray
    air_ring: bool

    @property
    def n_chunks(self) -> int:
        return self.nx * self.ny * self.nz

    def index(self, ix: int, iy: int, iz: int) -> int:
        return ix + self.nx * (iz + self.nz * iy)

    def coords(self, i: int) -> tuple:
        return i % self.nx, i // (self.nx * self.nz), (i // self.nx) % self.nz

    def neighbours(self, ix: int, iy: int, iz: int) -> np.ndarray:
        """27 chunk indices in the reference's neighbour order (centre = 26); -1 outside."""
        out = np.empty(27, np.int32)
        _load().hcw_neighbours(ctypes.byref(self._grid()), ix, iy, iz, out.ctypes.data)
        return out

    def meshable(self) -> np.ndarray:
        """Indices of chunks whose 26 neighbours all lie inside the grid."""
        ix = np.arange(self.n_chunks) % self.nx
        iz = (np.arange(self.n_chunks) // self.nx) % self.nz
        iy = np.arange(self.n_chunks) // (self.nx * self.nz)
        ok = (ix > 0) & (ix < self.nx - 1) & (iy > 0) & (iy < self.ny - 1) & (iz > 0) & (iz < self.nz - 1)
        return np.nonzero(ok)[0].astype(np.int32)

    def neighbour_table(self, chunks) -> np.ndarray:
        """(len(chunks), 27) int32 neighbour table for the given chunk indices (-1 outside the grid);
        the same order as ``neighbours`` (common/include/common/Position.hpp:146-152)."""
        c = np.asarray(chunks, np.int64)
        ix, iz, iy = c % self.nx, (c // self.nx) % self.nz, c // (self.nx * self.nz)
        rev = np.array([1, -1, 0])
        i = np.arange(27)
        dx, dy, dz = rev[i // 9], rev[(i // 3) % 3], rev[i % 3]
        x, y, z = ix[:, None] + dx, iy[:, None] + dy, iz[:, None] + dz
        ok = (x >= 0) & (y >= 0) & (z >= 0) & (x < self.nx) & (y < self.ny) & (z < self.nz)
        return np.where(ok, x + self.nx * (z + self.nz * y), -1).astype(np.int32)

    def recompute_heights(self, threads: int = 0) -> None:
        _load().hcw_recompute_heights(ctypes.byref(self._grid()), self.kinds.ctypes.data, int(self.air_ring),
                                      self.blocks.ctypes.data, self.heights.ctypes.data, threads or os.cpu_count())

    def _grid(self) -> _Grid:
        return _Grid(self.nx, self.ny, self.nz, *self.origin)


def generate(nx: int, ny: int, nz: int, origin=(0, 0, 0), *, seed: int = WORLD_SEED, caves: bool = False,
             leaves_permille: int = 50, air_ring: bool = False, mixture: bool = False,
             default_kind: int = KIND_TERRAIN, threads: int = 0) -> World:
    lib = _load()
    g = _Grid(nx, ny, nz, *origin)
    p = _Params(seed, int(caves), leaves_permille, int(air_ring), int(mixture), default_kind)
    n = nx * ny * nz
    kinds = np.empty(n, np.uint8)
    blocks = np.empty((n, 32768), np.uint16)
    heights = np.empty((n, 1024), np.int8)
    lib.hcw_assign_kinds(ctypes.byref(g), ctypes.byref(p), kinds.ctypes.data)
    rc = lib.hcw_generate(ctypes.byref(g), ctypes.byref(p), kinds.ctypes.data, blocks.ctypes.data,
                          heights.ctypes.data, threads or os.cpu_count())
    if rc != 0:
        raise RuntimeError(f"hcw_generate failed ({rc})")
    return World(nx, ny, nz, tuple(origin), blocks, heights, kinds, air_ring)


def plain_world(seed: int = WORLD_SEED) -> World:
    """Single-chunk workload: 3x3x3 chunks of noise terrain (chunk y -1..1), 5% leaves, no caves."""
    return generate(3, 3, 3, (-1, -1, -1), seed=seed, caves=False, leaves_permille=50)


def scale_world(nx: int = 32, ny: int = 8, nz: int = 32, seed: int = WORLD_SEED) -> World:
    """Terrain with caves and glowstone, padded by a ring of lit all-air chunks (chunk y from -ny/2)."""
    return generate(nx + 2, ny + 2, nz + 2, (-(nx // 2) - 1, -(ny // 2) - 1, -(nz // 2) - 1), seed=seed, caves=True,
                    leaves_permille=50, air_ring=True)


def mixture_world(nx: int = 32, ny: int = 16, nz: int = 32, seed: int = WORLD_SEED) -> World:
    """Seeded 30/20/35/10/5 mixture of air, stone, terrain, random fill and checkerboard chunks."""
    return generate(nx + 2, ny + 2, nz + 2, (-(nx // 2) - 1, -(ny // 2) - 1, -(nz // 2) - 1), seed=seed, caves=True,
                    leaves_permille=50, air_ring=True, mixture=True)
