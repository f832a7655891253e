"""The entry point that allocates nothing (hc_mesh_batch_noalloc), called through the C ABI, gives
each chunk exactly the meshes of the regular batched entry point, on two calls in a row.

It exists for callers that cannot allocate device memory, such as code running in a host
application's frame loop under a fixed memory budget or a plugin whose host owns all device
allocations. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    vp = ctypes.c_void_p
    f = lib.hc_mesh_batch_noalloc
    f.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint32, vp, vp, vp, ctypes.c_uint64, ctypes.c_uint32, vp,
                  ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32), vp,
                  ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def _meshes_of(chunk, results, descs, verts, idx):
    from hypercraft_gb300.mesher import BlockMesh
    r = results[5 * chunk:5 * chunk + 5]
    assert r[4] == 0
    out = []
    for d in descs[int(r[2]):int(r[2]) + int(r[3])]:
        vo, vc, io, ic = (int(d[k]) for k in ("vertex_offset", "vertex_count", "index_offset", "index_count"))
        assert int(d["chunk"]) == chunk
        out.append(BlockMesh(verts[vo:vo + vc].copy(), idx[io:io + ic].copy(),
                             tuple(int(x) for x in d["aabb_min"]) + tuple(int(x) for x in d["aabb_max"]),
                             bool(d["transparent"])))
    return out


def test_noalloc_matches_batched_entry_point_twice():
    import torch
    from hypercraft_gb300 import batch, mesher, worldgen
    from hypercraft_gb300.build import build
    build()
    ctx = mesher.Context(0)
    w = worldgen.mixture_world(4, 4, 4)
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)

    # the existing entry point
    arena = batch.Arena(3_000_000, 4096, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.PERSISTENT)
    plan.launch()
    q_ref, m_ref, f_ref = plan.result()
    assert f_ref == 0
    ref = arena.host()
    expected = [arena.chunk_meshes(i, ref) for i in range(n)]

    # the no-alloc entry point: the caller passes every buffer
    f = _bind(mesher.library())
    blocks = torch.from_numpy(w.blocks.view(np.int16)).cuda()
    heights = torch.from_numpy(w.heights).cuda()
    nbr = torch.from_numpy(rw.neighbours).cuda()
    qcap, mcap = 3_000_000, 4096
    verts = torch.zeros(qcap * 8, dtype=torch.int32, device="cuda")
    idx = torch.zeros(qcap * 6, dtype=torch.int16, device="cuda")
    descs = torch.zeros(mcap * 12, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        verts.fill_(-1)
        results = np.zeros(n * 5, np.uint32)
        q, m, fc = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        err = ctypes.create_string_buffer(256)
        st = f(blocks.data_ptr(), heights.data_ptr(), w.n_chunks, nbr.data_ptr(), n, verts.data_ptr(), idx.data_ptr(),
               descs.data_ptr(), qcap, mcap, results.ctypes.data, ctypes.byref(q), ctypes.byref(m), ctypes.byref(fc),
               None, err, len(err))
        assert st == 0, err.value.decode()
        assert (q.value, m.value, fc.value) == (q_ref, m_ref, 0), call
        d = descs.cpu().numpy().view(mesher.MESH_DESC_DTYPE)
        v = verts.cpu().numpy().view(np.uint32).reshape(-1, 2)
        ii = idx.cpu().numpy().view(np.uint16)
        for i in range(n):
            got = _meshes_of(i, results, d, v, ii)
            assert len(got) == len(expected[i]), (call, i)
            assert all(a == b for a, b in zip(got, expected[i])), (call, i)  # bit-exact


def test_noalloc_rejects_oversized_batch():
    import torch
    from hypercraft_gb300 import mesher
    from hypercraft_gb300.build import build
    build()
    f = _bind(mesher.library())
    dummy = torch.zeros(1024, dtype=torch.int32, device="cuda")
    err = ctypes.create_string_buffer(256)
    q, m, fc = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
    st = f(dummy.data_ptr(), dummy.data_ptr(), 1, dummy.data_ptr(), 16385, dummy.data_ptr(), dummy.data_ptr(),
           dummy.data_ptr(), 1, 1, None, ctypes.byref(q), ctypes.byref(m), ctypes.byref(fc), None, err, len(err))
    assert st == mesher.HC_ERR_CAPACITY
    assert b"16384" in err.value
