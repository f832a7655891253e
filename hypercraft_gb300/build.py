"""Builds the in-tree shared libraries (nvcc for sm_103a, g++ for host code).

``build()`` compiles, in parallel:
  * ``_lib/libhc_gb300.so``   the CUDA relighter + mesher, world stages and request server behind
    include/hc_gb300.h;
  * ``_lib/libhc_worldgen.so`` the seeded synthetic world generator (host only).
Each library is rebuilt only when one of its sources is newer than it.
"""
from __future__ import annotations

import glob
import os
import subprocess

from ._paths import CSRC_DIR, INCLUDE_DIR, LIB_DIR

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources(*patterns):
    out = []
    for p in patterns:
        out += sorted(glob.glob(os.path.join(CSRC_DIR, p)))
    return out


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _jobs(force: bool):
    jobs = []
    gpu = os.path.join(LIB_DIR, "libhc_gb300.so")
    gpu_deps = _sources("*.cu", "*.cuh", "*.h", "hc_registry.cpp", "hc_server.cpp") + [os.path.join(INCLUDE_DIR,
                                                                                              "hc_gb300.h")]
    if force or _stale(gpu, gpu_deps):
        jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                     "-o", gpu, os.path.join(CSRC_DIR, "hc_gb300.cu"), os.path.join(CSRC_DIR, "hc_registry.cpp"),
                     os.path.join(CSRC_DIR, "hc_server.cpp")])
    wg = os.path.join(LIB_DIR, "libhc_worldgen.so")
    wg_deps = _sources("hc_worldgen.*", "hc_registry.*", "hc_flow.h")
    if force or _stale(wg, wg_deps):
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-o", wg,
                     os.path.join(CSRC_DIR, "hc_worldgen.cpp"), os.path.join(CSRC_DIR, "hc_registry.cpp")])
    return jobs


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(LIB_DIR, exist_ok=True)
    procs = []
    for cmd in _jobs(force):
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"{' '.join(cmd)}\n{out.decode(errors='replace')}")
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))


if __name__ == "__main__":
    build(verbose=True)
