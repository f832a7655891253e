"""CPU oracle and registry pinned against the reference: the committed golden digests (made by
running the reference's own templates, tests/golden/make_golden.py) everywhere, and the live
reference harness where the reference sources are present."""
import hashlib
import json
import os

import numpy as np
import pytest

import cases

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _oracle_registry_digest():
    from oracle import bind
    reg = bind.oracle_registry()
    out = {k: hashlib.sha256(np.ascontiguousarray(reg[k]).tobytes()).hexdigest()
           for k in ("tex", "transparency", "light", "collision")}
    h = hashlib.sha256()
    faces = reg["faces"]
    for raw in range(65536):
        kind = int(reg["mesh_kind"][raw])
        if kind == 0:
            h.update(b"-")
        elif kind == 2:
            h.update(b"flow")
        else:
            f0, n = int(reg["mesh_first"][raw]), int(reg["mesh_count"][raw])
            h.update(faces[f0:f0 + n].tobytes())
    out["custom_meshes"] = h.hexdigest()
    return out


def test_registry_matches_reference_table(built):
    assert _oracle_registry_digest() == GOLDEN["registry"]


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_oracle_matches_golden(oracle, name):
    b, h = cases.CASES[name]()
    g = GOLDEN["cases"][name]
    assert cases.input_digest(b, h) == g["input"], "seeded input generation changed"
    light = oracle.relight_window(b, h)
    assert hashlib.sha256(light.tobytes()).hexdigest() == g["light62"]
    meshes = oracle.mesh_chunk(b, h)
    assert len(meshes) == g["mesh_count"]
    assert sum(len(m.vertices) for m in meshes) // 4 == g["quads"]
    assert cases.mesh_digest(meshes) == g["meshes"]


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_oracle_matches_live_reference(oracle, reference, seed):
    for make in (cases.random_all, cases.liquids, cases.glow):
        b, h = make(seed)
        assert np.array_equal(oracle.relight_window(b, h), reference.relight_window(b, h))
        mo, mr = oracle.mesh_chunk(b, h), reference.mesh_chunk(b, h)
        assert len(mo) == len(mr) and all(a == c for a, c in zip(mo, mr))


def test_flow_mesh_matches_live_reference(oracle, reference):
    import ctypes
    rng = np.random.default_rng(5)
    for _ in range(3000):
        meta = int(rng.integers(0, 256))
        nei = np.array([int(rng.choice([0, 14, 15, 1, 5, 9])) | (int(rng.integers(0, 256)) << 8) for _ in range(8)],
                       np.uint16)
        f1, f2 = np.zeros(384, np.uint8), np.zeros(384, np.uint8)
        n1, n2 = ctypes.c_uint32(), ctypes.c_uint32()
        t1, t2 = np.zeros(6, np.uint16), np.zeros(6, np.uint16)
        reference.lib.hcref_flow_mesh(15 | (meta << 8), nei.ctypes.data, f1.ctypes.data, ctypes.byref(n1), t1.ctypes.data)
        oracle.lib.hco_flow_mesh(nei.ctypes.data, min(meta & 15, 8), f2.ctypes.data, ctypes.byref(n2), t2.ctypes.data)
        assert n1.value == n2.value and np.array_equal(f1[:24 * n1.value], f2[:24 * n2.value])
        assert np.array_equal(t1, t2)


def test_chunk_should_remesh_matches_live_reference(oracle, reference):
    for x in range(-20, 53, 3):
        for y in range(-20, 53, 5):
            for z in range(-20, 53, 7):
                assert oracle.lib.hco_chunk_should_remesh(x, y, z) == reference.lib.hcref_chunk_should_remesh(x, y, z)


def test_light_window_shape_and_range(oracle):
    b, h = cases.glow(3)
    light = oracle.relight_window(b, h)
    assert light.shape == (62 ** 3,)
    assert (light & 15).max() <= 15 and (light >> 4).max() <= 15


def test_edit_chain_marks_every_changed_mesh(oracle):
    """The restated SetBlock -> FloodSunlight -> SetSunlight rules mark every chunk whose mesh
    changes (checked by meshing every chunk before and after)."""
    from hypercraft_gb300 import world as hw
    from oracle import edits as oe
    w = hw.edit_world()
    def mesh(c):
        nb = w.neighbours(*w.coords(int(c)))
        return oracle.mesh_chunk([w.blocks[k] for k in nb], [w.heights[k] for k in nb])
    meshable = [int(c) for c in w.meshable()]
    before = {c: mesh(c) for c in meshable}
    dirty = oe.apply_edits(w, hw.seeded_edits(1024, seed=5))
    changed = {c for c in meshable if not (len(before[c]) == len(after := mesh(c)) and
                                           all(a == b for a, b in zip(before[c], after)))}
    assert changed, "the edits change some meshes"
    assert changed <= dirty


def test_seeded_edits_are_deterministic():
    from hypercraft_gb300 import world as hw
    a, b = hw.seeded_edits(4096, seed=7), hw.seeded_edits(4096, seed=7)
    assert np.array_equal(a, b)
    d = np.sqrt((a["x"] - 16.0) ** 2 + (a["y"] - 16.0) ** 2 + (a["z"] - 16.0) ** 2)
    assert d.max() <= 48 and 0.05 < np.mean(a["block"] == 24) < 0.15


def test_stored_edit_entries_pack_like_the_reference():
    """PackedChunkBlockEntry / PackedChunkSunlightEntry bit layouts (common/include/common/Data.hpp:36-86)."""
    from hypercraft_gb300 import world as hw
    be = hw.pack_block_entries([0, 32767, 1234], [0x0201, 0xffff, 9])
    assert list(be) == [0x0201, (32767 << 16) | 0xffff, (1234 << 16) | 9]
    se = hw.pack_sunlight_entries([0, 1023, 77], [0, 32, 5])
    assert se.dtype == np.uint16 and list(se) == [0, (1023 << 6) | 32, (77 << 6) | 5]
    b, h = hw.apply_entries(np.zeros(32768, np.uint16), np.zeros(1024, np.int8),
                            hw.pack_block_entries([5, 5], [1, 2]), hw.pack_sunlight_entries([3], [17]))
    assert b[5] == 2 and h[3] == 17
