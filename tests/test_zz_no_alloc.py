"""The entry point that allocates nothing (hc_mesh_batch_noalloc), called through the C ABI, gives
each chunk exactly the meshes of the regular batched entry point, on two calls in a row; it reports
short output buffers with the required sizes.

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


def _world(kind):
    from hypercraft_gb300 import worldgen
    if kind == "mixture":
        return worldgen.mixture_world(4, 4, 4)
    # 2 x 2 x 2 checkerboard chunks (98,304 quads each, far past the 4,096 quad records a CTA keeps
    # in shared memory: the no-alloc path has no record scratch, so it merges again in windows)
    return worldgen.generate(4, 4, 4, (-2, -2, -2), caves=False, air_ring=True, default_kind=worldgen.KIND_CHECKER)


def _reference_run(ctx, w):
    from hypercraft_gb300 import batch
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    arena = batch.Arena(3_000_000, 4096, n)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, batch.PERSISTENT)
    plan.launch()
    q_ref, m_ref, f_ref = plan.result()
    assert f_ref == 0
    ref = arena.host()
    expected = [arena.chunk_meshes(i, ref) for i in range(n)]
    return rw, n, q_ref, m_ref, expected


def _call(f, blocks, heights, w, nbr, n, verts, idx, descs, qcap, mcap, results):
    q, m, fc = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
    err = ctypes.create_string_buffer(256)
    st = f(blocks.data_ptr(), heights.data_ptr(), w.n_chunks, nbr.data_ptr(), n, verts.data_ptr(), idx.data_ptr(),
           descs.data_ptr(), qcap, mcap, results.ctypes.data, ctypes.byref(q), ctypes.byref(m), ctypes.byref(fc),
           None, err, len(err))
    return st, q.value, m.value, fc.value, err.value.decode()


@pytest.mark.parametrize("kind", ["mixture", "checker"])
def test_noalloc_matches_batched_entry_point_twice(kind):
    import torch
    from hypercraft_gb300 import mesher
    from hypercraft_gb300.build import build
    build()
    ctx = mesher.Context(0)
    w = _world(kind)
    rw, n, q_ref, m_ref, expected = _reference_run(ctx, w)  # the existing entry point
    if kind == "checker":
        assert all(sum(len(x.vertices) for x in e) // 4 > 4096 for e in expected)

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
        st, q, m, fc, err = _call(f, blocks, heights, w, nbr, n, verts, idx, descs, qcap, mcap, results)
        assert st == 0, err
        assert (q, m, fc) == (q_ref, m_ref, 0), call
        d = descs.cpu().numpy().view(mesher.MESH_DESC_DTYPE)
        v = verts.cpu().numpy().view(np.uint32).reshape(-1, 2)
        ii = idx.cpu().numpy().view(np.uint16)
        for i in range(n):
            got = _meshes_of(i, results, d, v, ii)
            assert len(got) == len(expected[i]), (call, i)
            assert all(a == b for a, b in zip(got, expected[i])), (call, i)  # bit-exact


def test_noalloc_short_buffers_report_required_sizes():
    """Output buffers too small for the batch: HC_ERR_CAPACITY with the required quad and mesh counts
    written back; the chunks that fit are complete and the others have status 1 and no output. The
    next call with large enough buffers matches the batched entry point again."""
    import torch
    from hypercraft_gb300 import mesher
    from hypercraft_gb300.build import build
    build()
    ctx = mesher.Context(0)
    w = _world("mixture")
    rw, n, q_ref, m_ref, expected = _reference_run(ctx, w)
    f = _bind(mesher.library())
    blocks = torch.from_numpy(w.blocks.view(np.int16)).cuda()
    heights = torch.from_numpy(w.heights).cuda()
    nbr = torch.from_numpy(rw.neighbours).cuda()
    for qcap, mcap in ((q_ref // 2, 4096), (3_000_000, max(1, m_ref // 2))):
        verts = torch.zeros(qcap * 8, dtype=torch.int32, device="cuda")
        idx = torch.zeros(qcap * 6, dtype=torch.int16, device="cuda")
        descs = torch.zeros(mcap * 12, dtype=torch.int32, device="cuda")
        results = np.zeros(n * 5, np.uint32)
        st, q, m, fc, err = _call(f, blocks, heights, w, nbr, n, verts, idx, descs, qcap, mcap, results)
        assert st == mesher.HC_ERR_CAPACITY, err
        assert (q, m) == (q_ref, m_ref) and fc > 0
        r = results.reshape(-1, 5)
        assert set(np.unique(r[:, 4]).tolist()) <= {0, 1} and int((r[:, 4] == 1).sum()) == fc
        d = descs.cpu().numpy().view(mesher.MESH_DESC_DTYPE)
        v = verts.cpu().numpy().view(np.uint32).reshape(-1, 2)
        ii = idx.cpu().numpy().view(np.uint16)
        for i in np.nonzero(r[:, 4] == 0)[0]:
            got = _meshes_of(int(i), results, d, v, ii)
            assert len(got) == len(expected[i]) and all(a == b for a, b in zip(got, expected[i])), i
    qcap, mcap = 3_000_000, 4096
    verts = torch.zeros(qcap * 8, dtype=torch.int32, device="cuda")
    idx = torch.zeros(qcap * 6, dtype=torch.int16, device="cuda")
    descs = torch.zeros(mcap * 12, dtype=torch.int32, device="cuda")
    results = np.zeros(n * 5, np.uint32)
    st, q, m, fc, err = _call(f, blocks, heights, w, nbr, n, verts, idx, descs, qcap, mcap, results)
    assert st == 0 and (q, m, fc) == (q_ref, m_ref, 0), err


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
