"""Failure paths, on the GPU, through the C ABI.  Every failure here is made on
the host (bad coordinates, a flag, a cell too large for the slots): each call
returns a status and the context stays usable; nothing faults the GPU.

The reference panics in these situations instead (pool.rs:141-146,
polyhedron.rs:877, interface.rs:65)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("with_box", [True, False])
def test_non_finite_coordinates(tess, bad, with_box):
    L = tess.lib()
    pts = np.random.default_rng(1).random((2000, 3))
    pts[777, 1] = bad
    lo, hi = np.zeros(3), np.ones(3)
    h = C.c_void_p()
    st = L.tess_diagram_create(dp(pts), len(pts), None, dp(lo) if with_box else None, dp(hi) if with_box else None,
                               None, C.byref(h))
    assert st == tess._capi.TESS_E_INVALID
    assert "finite" in tess.last_error()
    assert not h.value
    # the context is still usable: the same points without the bad value work
    pts[777, 1] = 0.5
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1)) as d:
        d.compute_all("fp32")
        assert abs(d.volumes().sum() - 1.0) < 1e-6


def test_non_finite_update_and_batch(tess):
    rng = np.random.default_rng(2)
    pts = rng.random((3000, 3))
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1)) as d:
        bad = pts.copy()
        bad[5, 2] = np.nan
        with pytest.raises(tess.TessError) as e:
            d.update_points(bad)
        assert e.value.status == tess._capi.TESS_E_INVALID
        d.update_points(pts)                 # and back to finite points
        d.compute_all("fp64")
        assert abs(d.volumes().sum() - 1.0) < 1e-11
    offs = np.array([0, 1000, 3000], dtype=np.uint64)
    boxes = np.array([[0, 0, 0, 1, 1, 1], [0, 0, 0, 1, 1, 1]], dtype=np.float64)
    bad = pts.copy()
    bad[2500, 0] = np.inf
    with pytest.raises(tess.TessError) as e:
        tess.Batch(bad, offs, boxes)
    assert e.value.status == tess._capi.TESS_E_INVALID
    b = tess.Batch(pts, offs, boxes)
    try:
        b.compute("fp32")
        b.update_points(bad)
        with pytest.raises(tess.TessError) as e:
            b.compute("fp32")
        assert e.value.status == tess._capi.TESS_E_INVALID
        b.update_points(pts)
        b.compute("fp32")
        v = b.volumes()
        assert abs(v[:1000].sum() - 1.0) < 1e-6 and abs(v[1000:].sum() - 1.0) < 1e-6
    finally:
        b.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_points_outside_the_container(tess, oracle_mod, prec):
    """A point outside the box gets the part of the box nearer to it than to
    any other point (the box start cut by its bisectors, polyhedron.rs:268-392,
    interface.rs:257-313): empty (volume 0, no faces) when every other point is
    nearer everywhere in the box.  The volumes still add up to the box."""
    from oracle import report

    rng = np.random.default_rng(5)
    pts = rng.random((3000, 3))
    pts[0] = [1.5, 0.5, 0.5]
    pts[1] = [-0.004, 0.31, 0.29]     # just outside x_min: a small non-empty cell
    pts[2] = [0.5, 0.5, 3.0]
    pts[3] = [1.0001, 0.999, -0.0001]
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1)) as d:
        d.compute_all(prec)
        vol = d.volumes()
        offs, nbr, area = d.neighbors_csr()
        assert d.stats()["failed"] == 0
    r = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    rv, ro, ri, ra, _, _ = r.compute_all()
    assert rv[0] == 0.0 and rv[2] == 0.0 and rv[1] > 0.0 and rv[3] > 0.0   # the oracle's answer
    c = report.compare_sample((vol, offs.astype(np.int64), nbr, area), np.arange(len(pts)), (rv, ro, ri, ra))
    assert c["identical_neighbour_lists_pct"] == 100.0, c
    assert vol[0] == 0.0 and vol[2] == 0.0
    assert c["max_rel_vol_err"] <= (1e-6 if prec == "fp32" else 1e-12)
    assert abs(vol.sum() - 1.0) <= (1e-6 if prec == "fp32" else 1e-11)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_face_pool_regrow(tess, prec):
    """A face pool started at 1,024 faces overflows; the library grows it and
    recomputes, with results identical to the default run."""
    from tessellator import workloads

    pts = workloads.uniform(20000, seed=7)
    box = tess.Polyhedron(0, 0, 0, 1, 1, 1)
    out = []
    for flags in (0, tess.FLAG_SMALL_FACE_POOL):
        with tess.Diagram(pts, container=box, config=tess.default_config(flags=flags)) as d:
            d.compute_all(prec)
            out.append((d.volumes(), *d.neighbors_csr(), d.stats()))
    assert out[1][4]["face_pool_regrows"] >= 1 and out[0][4]["face_pool_regrows"] == 0
    for a, b in zip(out[0][:4], out[1][:4]):
        assert np.array_equal(a, b)
    # the batch path regrows too (its captured graph is rebuilt)
    offs = np.array([0, 5000, 20000], dtype=np.uint64)
    boxes = np.array([[0, 0, 0, 1, 1, 1]] * 2, dtype=np.float64)
    res = []
    for flags in (0, tess.FLAG_SMALL_FACE_POOL):
        b = tess.Batch(pts, offs, boxes, config=tess.default_config(flags=flags))
        try:
            b.compute(prec)
            res.append((b.volumes(), *b.neighbors_csr(), b.stats()))
        finally:
            b.close()
    assert res[1][4]["face_pool_regrows"] >= 1
    for a, b in zip(res[0][:4], res[1][:4]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_capacity_overflow_is_reported(tess, oracle_mod, prec):
    """Without the larger-capacity re-runs, a cell of ~300 vertices cannot fit
    the first pass's 64 slots: compute_all returns TESS_E_OVERFLOW, the cell
    is reported with volume 0 and no faces, and every other cell is right."""
    from oracle import report

    rng = np.random.default_rng(14)
    m = 150
    u = rng.standard_normal((m, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = np.concatenate([[[0.5, 0.5, 0.5]], 0.5 + 0.1 * u, rng.random((200, 3))])
    cfg = tess.default_config(flags=tess.FLAG_NO_CAPACITY_RERUN)
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1), config=cfg) as d:
        with pytest.raises(tess.TessError) as e:
            d.compute_all(prec)
        assert e.value.status == tess._capi.TESS_E_OVERFLOW
        st = d.stats()
        vol = d.volumes()
        offs, nbr, area = d.neighbors_csr()
    assert st["failed"] >= 1
    offs = offs.astype(np.int64)
    failed = np.nonzero(np.diff(offs) == 0)[0]
    assert 0 in failed and len(failed) == st["failed"]
    assert np.all(vol[failed] == 0.0)
    r = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    keep = np.setdiff1d(np.arange(len(pts)), failed)
    v, o, i, a, _, _ = r.compute_all(subset=keep.astype(np.uint32))
    c = report.compare_sample((vol, offs, nbr, area), keep, (v, o, i, a))
    assert c["identical_neighbour_lists_pct"] == 100.0, c
    assert c["max_rel_vol_err"] <= (1e-6 if prec == "fp32" else 1e-12)
