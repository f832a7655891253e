"""ctypes bindings of the CPU oracle (``hc_oracle.cpp``) and the reference harness (``oracle/_ref``).

TEST INFRASTRUCTURE: imported only by tests/, the smoke check and bench.py's CPU-baseline leg,
always as the checker or the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from dataclasses import dataclass

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(ORACLE_DIR)
BUILD_DIR = os.path.join(ORACLE_DIR, "_build")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
ORACLE_LIB = os.path.join(BUILD_DIR, "libhc_oracle.so")
REF_LIB = os.path.join(REF_DIR, "libhcref.so")
# the reference headers and generated block table, copied out of a checkout for hosts without one
BUNDLE_DIR = os.path.join(REF_DIR, "src")

FLAT_WORDS = 9


def build_oracle(force: bool = False) -> str:
    """Compiles the oracle restatement with g++ (any host, x86 or aarch64)."""
    srcs = [os.path.join(ORACLE_DIR, "hc_oracle.cpp"), os.path.join(REPO_DIR, "hypercraft_gb300", "csrc", "hc_registry.cpp")]
    if not force and os.path.exists(ORACLE_LIB) and all(os.path.getmtime(s) <= os.path.getmtime(ORACLE_LIB) for s in srcs):
        return ORACLE_LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-pthread", "-o", ORACLE_LIB] + srcs, check=True)
    return ORACLE_LIB


def reference_source() -> str | None:
    """The reference checkout: $HC_REFERENCE_SRC, else a checkout named ``reference`` beside the
    repository; None where neither holds the reference's mesher header."""
    for p in (os.environ.get("HC_REFERENCE_SRC"), os.path.join(os.path.dirname(REPO_DIR), "reference")):
        if p and os.path.isfile(os.path.join(p, "client", "include", "client", "BlockMeshAlgo.hpp")):
            return p
    return None


def _make(*args: str) -> None:
    jobs = str(min(8, os.cpu_count() or 1))
    subprocess.run(["make", "-s", "-f", "Makefile.ref", f"-j{jobs}", *args], cwd=ORACLE_DIR, check=True)


def _bundle(src: str) -> None:
    """Copies what the harness build reads from the checkout into ``_ref/src``, unmodified and at the
    same relative paths: the headers the two translation units include (``make deps``), the whole glm
    tree (it includes other headers on aarch64 than on x86) and the generated Block.cpp. The bundle
    is git-ignored; it lets a host without the checkout build the same library."""
    stamp = os.path.join(BUNDLE_DIR, ".complete")
    if os.path.exists(stamp):
        return
    out = subprocess.run(["make", "-s", "-f", "Makefile.ref", f"REF={src}", "deps"], cwd=ORACLE_DIR, check=True,
                         capture_output=True, text=True).stdout
    root = os.path.realpath(src)
    for line in out.split():
        f = os.path.realpath(os.path.join(ORACLE_DIR, line))
        if not f.startswith(root + os.sep):
            continue  # the harness's own files and system headers
        dst = os.path.join(BUNDLE_DIR, os.path.relpath(f, root))
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(f, dst)
    shutil.copytree(os.path.join(root, "dep", "glm"), os.path.join(BUNDLE_DIR, "dep", "glm"), dirs_exist_ok=True)
    shutil.copyfile(os.path.join(REF_DIR, "Block.cpp"), os.path.join(BUNDLE_DIR, "Block.cpp"))
    open(stamp, "w").close()


def build_reference() -> str | None:
    """Builds the reference harness (``_ref/libhcref.so``): from the checkout where there is one (and
    then also writes the bundle), else from the bundle; None where neither is present."""
    src = reference_source()
    if src is not None:
        _make(f"REF={src}")
        _bundle(src)
        return REF_LIB
    if os.path.isfile(os.path.join(BUNDLE_DIR, "Block.cpp")):
        args = (f"REF={BUNDLE_DIR}", f"BLOCK_CPP={os.path.join(BUNDLE_DIR, 'Block.cpp')}")
        _make(*args)
        if not _loadable(REF_LIB):  # a library built for another host came along with the bundle
            _make("-B", *args)
        return REF_LIB
    return REF_LIB if os.path.exists(REF_LIB) and _loadable(REF_LIB) else None


def _loadable(path: str) -> bool:
    try:
        ctypes.CDLL(path)
        return True
    except OSError:
        return False


class FlatMeshes(ctypes.Structure):
    _fields_ = [("mesh_cap", ctypes.c_uint32), ("vertex_cap", ctypes.c_uint32), ("index_cap", ctypes.c_uint32),
                ("mesh_count", ctypes.c_uint32), ("vertex_count", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("meshes", ctypes.c_void_p), ("vertices", ctypes.c_void_p), ("indices", ctypes.c_void_p)]


@dataclass
class Mesh:
    """One reference BlockMesh: (n, 2) uint32 packed vertices, uint16 indices, u32 AABB, flag."""
    vertices: np.ndarray
    indices: np.ndarray
    aabb: tuple
    transparent: bool

    def __eq__(self, o) -> bool:
        return (self.transparent == o.transparent and tuple(self.aabb) == tuple(o.aabb)
                and np.array_equal(self.vertices, o.vertices) and np.array_equal(self.indices, o.indices))


def meshes_from_flat(meshes: np.ndarray, vertices: np.ndarray, indices: np.ndarray, count: int) -> list:
    out, vo, io = [], 0, 0
    for i in range(count):
        w = meshes[i * FLAT_WORDS:(i + 1) * FLAT_WORDS]
        nv, ni = int(w[0]), int(w[1])
        out.append(Mesh(vertices[vo:vo + nv].copy(), indices[io:io + ni].copy(),
                        tuple(int(x) for x in w[2:8]), bool(w[8])))
        vo += nv
        io += ni
    return out


class _Runner:
    def __init__(self, path: str, prefix: str):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        f = getattr(self.lib, prefix + "_mesh_chunk")
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(FlatMeshes)]
        f.restype = ctypes.c_int
        g = getattr(self.lib, prefix + "_relight_window")
        g.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        self._mesh, self._relight = f, g
        self.cap = (64, 1 << 20, 3 << 19)

    @staticmethod
    def _ptrs(blocks27, heights27):
        b = (ctypes.c_void_p * 27)(*[np.ascontiguousarray(x).ctypes.data for x in blocks27])
        h = (ctypes.c_void_p * 27)(*[np.ascontiguousarray(x).ctypes.data for x in heights27])
        return b, h

    def relight_window(self, blocks27, heights27) -> np.ndarray:
        """62^3 light window (x fastest, then z, then y)."""
        blocks27 = [np.ascontiguousarray(x, np.uint16) for x in blocks27]
        heights27 = [np.ascontiguousarray(x, np.int8) for x in heights27]
        b, h = self._ptrs(blocks27, heights27)
        out = np.empty(62 ** 3, np.uint8)
        self._relight(b, h, out.ctypes.data)
        return out

    def mesh_chunk(self, blocks27, heights27) -> list:
        blocks27 = [np.ascontiguousarray(x, np.uint16) for x in blocks27]
        heights27 = [np.ascontiguousarray(x, np.int8) for x in heights27]
        b, h = self._ptrs(blocks27, heights27)
        while True:
            mc, vc, ic = self.cap
            meshes = np.zeros(mc * FLAT_WORDS, np.uint32)
            verts = np.zeros((vc, 2), np.uint32)
            idx = np.zeros(ic, np.uint16)
            fm = FlatMeshes(mc, vc, ic, 0, 0, 0, meshes.ctypes.data, verts.ctypes.data, idx.ctypes.data)
            rc = self._mesh(b, h, ctypes.byref(fm))
            if rc == 0:
                return meshes_from_flat(meshes, verts, idx, fm.mesh_count)
            self.cap = (max(mc, fm.mesh_count), max(vc, fm.vertex_count), max(ic, fm.index_count))


_oracle = None
_reference = None


def oracle() -> _Runner:
    """The CPU restatement (builds it on first use)."""
    global _oracle
    if _oracle is None:
        _oracle = _Runner(build_oracle(), "hco")
        _bind_oracle_extras(_oracle.lib)
    return _oracle


def reference() -> _Runner | None:
    """The reference's own templates, where they could be built here; else None."""
    global _reference
    if _reference is None:
        path = build_reference()
        if path is None:
            return None
        _reference = _Runner(path, "hcref")
        _bind_reference_extras(_reference.lib)
    return _reference


def _bind_many(lib, name):
    f = getattr(lib, name)
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_uint64


def mesh_many(runner, blocks: np.ndarray, heights: np.ndarray, nbr: np.ndarray, threads: int):
    """Relights + meshes every row of the (n, 27) chunk-index table `nbr` on `threads` threads;
    returns (quads, meshes)."""
    nbr = np.ascontiguousarray(nbr, np.int32)
    m = ctypes.c_uint64()
    fn = getattr(runner.lib, runner.prefix + "_mesh_many")
    q = fn(blocks.ctypes.data, heights.ctypes.data, nbr.ctypes.data, nbr.shape[0], threads, ctypes.byref(m))
    return int(q), int(m.value)


def mesh_rows(runner, blocks: np.ndarray, heights: np.ndarray, nbr: np.ndarray, threads: int) -> list:
    """The meshes of every row of the (n, 27) chunk-index table `nbr`, one list per row, computed on
    `threads` threads (the foreign calls release the interpreter lock)."""
    from concurrent.futures import ThreadPoolExecutor

    def one(row):
        # each call sizes its own buffers (the runner's shared capacity hint only ever grows)
        return runner.mesh_chunk([blocks[k] for k in row], [heights[k] for k in row])

    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        return list(ex.map(one, np.asarray(nbr)))


def sample_positions(n: int, size: int, seed: int) -> np.ndarray:
    """A seeded random sample of `size` of `n` batch positions, sorted; both bench arms and the
    full-size parity test draw their samples this way."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, min(n, size), replace=False))


def _bind_oracle_extras(lib):
    _bind_many(lib, "hco_mesh_many")
    lib.hco_mesh_chunk_lit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(FlatMeshes)]
    lib.hco_dump_registry.argtypes = [ctypes.c_void_p] * 9
    lib.hco_flow_mesh.argtypes = [ctypes.c_void_p, ctypes.c_uint8, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hco_chunk_should_remesh.argtypes = [ctypes.c_int] * 3


def _bind_reference_extras(lib):
    _bind_many(lib, "hcref_mesh_many")
    lib.hcref_dump_registry.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32, ctypes.c_void_p]
    lib.hcref_flow_mesh.argtypes = [ctypes.c_uint16, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hcref_flow_fetch_offsets.argtypes = [ctypes.c_uint16, ctypes.c_void_p, ctypes.c_void_p]
    lib.hcref_chunk_should_remesh.argtypes = [ctypes.c_int] * 3


def oracle_registry() -> dict:
    """The registry restatement as numpy arrays (per raw value), plus the static face table."""
    lib = oracle().lib
    tex = np.zeros((65536, 6), np.uint16)
    tr, li, co, mk, mf, mc = (np.zeros(65536, np.uint8) for _ in range(6))
    faces = np.zeros(256 * 24, np.uint8)
    nf = ctypes.c_uint32(0)
    lib.hco_dump_registry(tex.ctypes.data, tr.ctypes.data, li.ctypes.data, co.ctypes.data, mk.ctypes.data,
                          mf.ctypes.data, mc.ctypes.data, faces.ctypes.data, ctypes.byref(nf))
    return dict(tex=tex, transparency=tr, light=li, collision=co, mesh_kind=mk, mesh_first=mf, mesh_count=mc,
                faces=faces[:nf.value * 24].reshape(-1, 24))


def reference_registry() -> dict | None:
    ref = reference()
    if ref is None:
        return None
    tex = np.zeros((65536, 6), np.uint16)
    tr, li, co = (np.zeros(65536, np.uint8) for _ in range(3))
    key = np.zeros(65536, np.uint16)
    cap = 256 * (1 + 16 * 24)
    faces = np.zeros(cap, np.uint8)
    nm = ctypes.c_uint32(0)
    rc = ref.lib.hcref_dump_registry(tex.ctypes.data, tr.ctypes.data, li.ctypes.data, co.ctypes.data, key.ctypes.data,
                                     faces.ctypes.data, cap, ctypes.byref(nm))
    assert rc == 0
    meshes = []
    for k in range(nm.value):
        rec = faces[k * (1 + 16 * 24):(k + 1) * (1 + 16 * 24)]
        meshes.append(rec[1:1 + 24 * int(rec[0])].reshape(-1, 24).copy())
    return dict(tex=tex, transparency=tr, light=li, collision=co, mesh_key=key, meshes=meshes)
