"""The seeded serving workload (host side): Poisson arrivals, the 70 / 25 / 5 request mix, loads of
chunks entering the view sphere after the unloads of those leaving it, all positions in the grid."""
import numpy as np


_FIELDS = ["kind", "block", "x", "y", "z", "size"]  # the rest are host pointers into the library


def _workload(seed=4):
    from hypercraft_gb300 import server as hs
    lib = hs.ChunkLibrary(4, 2, 4, seed=9)
    return hs, hs.ServingWorkload(lib, grid=(24, 10, 24), origin=(-12, -5, -12), radius=4, seed=seed)


def test_trace_is_deterministic_and_mixed():
    hs, a = _workload()
    _, b = _workload()
    ia, ib = a.initial_loads(), b.initial_loads()
    ra, ta = a.trace(20000.0, 0.2)
    rb, tb = b.trace(20000.0, 0.2)
    for f in _FIELDS:
        assert np.array_equal(ia[f], ib[f]) and np.array_equal(ra[f], rb[f]), f
    assert np.array_equal(ta, tb)
    assert (np.diff(ta.astype(np.int64)) >= 0).all(), "arrivals in time order"
    mix = ra[ra["kind"] != hs.REQ_UNLOAD]["kind"]
    frac = np.bincount(mix, minlength=4)[:3] / len(mix)
    assert abs(frac[hs.REQ_EDIT] - 0.70) < 0.05 and abs(frac[hs.REQ_LOAD] - 0.25) < 0.05
    assert abs(frac[hs.REQ_FILL] - 0.05) < 0.03
    assert (ra[ra["kind"] == hs.REQ_FILL]["size"] == 16).all()
    assert abs(len(mix) / 0.2 - 20000.0) < 2000.0, "the requested rate"


def test_view_is_kept_resident_in_order():
    hs, w = _workload(seed=7)
    resident = {tuple(int(v) for v in (r["x"], r["y"], r["z"])) for r in w.initial_loads()}
    reqs, _ = w.trace(20000.0, 0.3)
    for r in reqs:
        p = (int(r["x"]), int(r["y"]), int(r["z"]))
        if r["kind"] == hs.REQ_UNLOAD:
            assert p in resident
            resident.remove(p)
        elif r["kind"] == hs.REQ_LOAD:
            assert p not in resident, "a chunk is loaded only once while resident"
            assert all(w.origin[a] <= p[a] < w.origin[a] + w.grid[a] for a in range(3))
            resident.add(p)
    # what stays resident is the view sphere around the player, less the loads not yet issued
    view = set(w.view(w.player))
    assert resident <= view and len(view - resident) == len(w.load_queue)
