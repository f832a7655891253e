"""The C-ABI library loads without a GPU and exports every entry point include/*.h declares."""
import ctypes
import glob
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for hdr in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(hc_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = _declared()
    for n in ("hc_ctx_create", "hc_ctx_destroy", "hc_mesh_chunk", "hc_mesh_chunk_device", "hc_relight_chunk_device",
              "hc_status_string", "hc_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    from hypercraft_gb300.mesher import library
    lib = library()
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(built):
    from hypercraft_gb300.mesher import library
    lib = library()
    for s in range(7):
        assert lib.hc_status_string(s)


def test_context_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from hypercraft_gb300.mesher import library, HC_ERR_NO_DEVICE
    lib = library()
    h = ctypes.c_void_p()
    assert lib.hc_ctx_create(0, ctypes.byref(h)) == HC_ERR_NO_DEVICE
    assert not h.value


def test_variant_tables_match_the_header():
    """The Python mirror names every persistent variant the header enumerates, in its order, and
    counts the light-pass variants' extra launches (15 light levels) in the launch claim."""
    from hypercraft_gb300 import batch
    text = open(os.path.join(REPO, "include", "hc_gb300.h")).read()
    enum = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"\bHC_VARIANT_(\w+)\s*=\s*(\d+)", text))
    count = enum.pop("COUNT")
    assert count == len(batch.VARIANTS) == len(enum)
    assert sorted(enum.values()) == list(range(count))
    light = {v for k, v in enum.items() if k in ("LIGHT_PASS", "CLAIM2", "CLAIM4", "NO_SCRATCH")}
    assert light == set(batch.LIGHT_PASS_VARIANTS)
    for v in range(count):
        assert ("light pass" in batch.VARIANTS[v]) == (v in light)
        assert batch.launches_per_run(v) == (18 if v in light else (3 if v == enum["WINDOW"] else 2))
