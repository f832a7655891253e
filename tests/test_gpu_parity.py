"""GPU parity: the CUDA path through the C ABI against the reference's digests and the CPU oracle.
Bit-exact throughout (integer and byte work)."""
import hashlib
import json
import os

import numpy as np
import pytest

import cases

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
pytestmark = pytest.mark.gpu


def _device_chunks(b, h):
    import torch
    bt = [torch.from_numpy(np.ascontiguousarray(x).view(np.int16)).cuda() for x in b]
    ht = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in h]
    return bt, ht


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_mesh_chunk_matches_reference_digest(ctx, name):
    b, h = cases.CASES[name]()
    g = GOLDEN["cases"][name]
    meshes = ctx.mesh_chunk(b, h)
    assert len(meshes) == g["mesh_count"]
    assert sum(len(m.vertices) for m in meshes) // 4 == g["quads"]
    assert cases.mesh_digest(meshes) == g["meshes"]


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_relight_matches_reference_digest(ctx, name):
    import torch
    b, h = cases.CASES[name]()
    bt, ht = _device_chunks(b, h)
    out = torch.zeros(34 ** 3, dtype=torch.uint8, device="cuda")
    ctx.relight_chunk_device([x.data_ptr() for x in bt], [x.data_ptr() for x in ht], out.data_ptr())
    torch.cuda.synchronize()
    light = out.cpu().numpy()
    assert hashlib.sha256(light.tobytes()).hexdigest() == GOLDEN["cases"][name]["light34"]


@pytest.mark.parametrize("seed", [201, 202, 203, 204])
def test_mesh_chunk_matches_oracle_random(ctx, oracle, seed):
    for make in (cases.random_all, cases.liquids, cases.glow):
        b, h = make(seed)
        mg, mo = ctx.mesh_chunk(b, h), oracle.mesh_chunk(b, h)
        assert len(mg) == len(mo)
        for a, c in zip(mg, mo):
            assert a == c


@pytest.mark.parametrize("make", [lambda: cases.flat_ground(False), lambda: cases.flat_ground(True), cases.stripes],
                         ids=["flat_ground", "flat_ground_leaves", "stripes"])
def test_split_planes_and_isolated_rows_match_oracle(ctx, oracle, make):
    """A 1,024-face plane keyed in two halves (one quad across the split row; complex faces on the
    row above the second half) and planes mixing isolated rows with rows linked by equal-below cells."""
    b, h = make()
    mg, mo = ctx.mesh_chunk(b, h), oracle.mesh_chunk(b, h)
    assert len(mg) == len(mo) and all(a == c for a, c in zip(mg, mo))


def test_most_quads_match_oracle(ctx, oracle):
    """196,608 quads: past the shared and global record buffers, so the emission merges planes again
    in windows; the result still equals the oracle's."""
    b, h = cases.transparent_checker()
    mg, mo = ctx.mesh_chunk(b, h), oracle.mesh_chunk(b, h)
    assert sum(len(m.vertices) for m in mo) // 4 == 196608
    assert len(mg) == len(mo) and all(a == c for a, c in zip(mg, mo))


def test_device_entry_point_matches_host_entry_point(ctx):
    import torch
    from hypercraft_gb300.mesher import MESH_DESC_DTYPE, meshes_from_descs
    b, h = cases.liquids(31)
    bt, ht = _device_chunks(b, h)
    cap_q = 400000
    verts = torch.zeros(cap_q * 8, dtype=torch.int32, device="cuda")
    idx = torch.zeros(cap_q * 6, dtype=torch.int16, device="cuda")
    descs = torch.zeros(96 * 12, dtype=torch.int32, device="cuda")
    mc, vc, ic = ctx.mesh_chunk_device([x.data_ptr() for x in bt], [x.data_ptr() for x in ht], verts.data_ptr(),
                                       cap_q * 4, idx.data_ptr(), cap_q * 6, descs.data_ptr(), 96)
    d = descs.cpu().numpy().view(MESH_DESC_DTYPE)[:mc]
    v = verts.cpu().numpy().view(np.uint32).reshape(-1, 2)
    i = idx.cpu().numpy().view(np.uint16)
    dev = meshes_from_descs(d, v, i)
    host = ctx.mesh_chunk(b, h)
    assert len(dev) == len(host) and all(a == c for a, c in zip(dev, host))
    assert vc == sum(len(m.vertices) for m in host) and ic == sum(len(m.indices) for m in host)


def test_device_entry_point_reports_capacity(ctx):
    import torch
    from hypercraft_gb300.mesher import HcError, HC_ERR_CAPACITY
    b, h = cases.checker()
    bt, ht = _device_chunks(b, h)
    verts = torch.zeros(1000 * 8, dtype=torch.int32, device="cuda")
    idx = torch.zeros(1000 * 6, dtype=torch.int16, device="cuda")
    descs = torch.zeros(96 * 12, dtype=torch.int32, device="cuda")
    with pytest.raises(HcError) as e:
        ctx.mesh_chunk_device([x.data_ptr() for x in bt], [x.data_ptr() for x in ht], verts.data_ptr(), 4000,
                              idx.data_ptr(), 6000, descs.data_ptr(), 96)
    assert e.value.status == HC_ERR_CAPACITY
