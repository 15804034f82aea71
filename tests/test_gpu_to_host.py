"""tess_diagram_compute_all_to_host: every cell's faces written by the GPU into
the caller's pinned host pool as the cells finish.

The results must be those of tess_diagram_compute_all + tess_volumes +
tess_neighbors_csr, bit for bit (the same kernels compute every cell; only the
pool the faces land in differs), and the oracle's.  Also: a pool too small is
TESS_E_CAPACITY with the size needed, pageable buffers are refused, a device
pool works, and afterwards the device-side face queries report TESS_E_STATE
until the next compute_all."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def T():
    import tessellator

    return tessellator


def _box(T):
    return T.Polyhedron(0, 0, 0, 1, 1, 1)


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
@pytest.mark.parametrize("kind", ["uniform", "clustered"])
def test_same_results_as_compute_all(T, kind, prec):
    from tessellator import workloads

    pts = workloads.uniform(30_000, seed=11) if kind == "uniform" else workloads.clustered(30_000, seed=12)
    with T.Diagram(pts, container=_box(T)) as d:
        d.compute_all(prec)
        vol = d.volumes()
        offs, nbr, area = d.neighbors_csr()
        r = d.compute_all_to_host(prec)
        assert np.array_equal(r.volumes, vol)
        o2, n2, a2 = r.csr()
        assert np.array_equal(o2, offs)
        assert np.array_equal(n2, nbr)
        assert np.array_equal(a2, area)
        assert r.faces_used >= int(offs[-1])
        # per-cell access agrees with the CSR
        for i in (0, 17, len(pts) - 1):
            fn, fa = r.faces(i)
            assert np.array_equal(fn, nbr[offs[i]:offs[i + 1]])
            assert np.array_equal(fa, area[offs[i]:offs[i + 1]])


def test_matches_the_oracle(T):
    import oracle
    from oracle import report
    from tessellator import workloads

    pts = workloads.uniform(20_000, seed=13)
    ref = oracle.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    rv, ro, ri, ra, _, _ = ref.compute_all()
    with T.Diagram(pts, container=_box(T)) as d:
        r = d.compute_all_to_host("mixed")
    offs, nbr, area = r.csr()
    c = report.compare_sample((r.volumes, offs.astype(np.int64), nbr, area), np.arange(len(pts)), (rv, ro, ri, ra))
    assert c["identical_neighbour_lists_pct"] == 100.0, c
    assert c["max_rel_vol_err"] <= 1e-11, c


def test_reused_pool_and_capacity(T):
    from tessellator import workloads

    L = T.lib()
    pts = workloads.uniform(10_000, seed=14)
    with T.Diagram(pts, container=_box(T)) as d:
        d.compute_all("fp32")
        faces = int(d.neighbors_csr()[0][-1])
        small = (T.pinned_empty(1000, np.int32), T.pinned_empty(1000, np.float64))
        vol = np.empty(len(pts))
        fs = np.empty(len(pts), dtype=np.uint64)
        fc = np.empty(len(pts), dtype=np.uint32)
        used = C.c_size_t(0)
        st = L.tess_diagram_compute_all_to_host(d._h, T.PRECISION_FP32_GUARD, -1.0, -1, vol.ctypes.data,
                                                fs.ctypes.data, fc.ctypes.data, small[0].ctypes.data,
                                                small[1].ctypes.data, 1000, C.byref(used))
        assert st == T._capi.TESS_E_CAPACITY
        assert used.value >= faces
        # the diagram is not computed after a refused pool
        with pytest.raises(T.TessError) as e:
            d.volumes()
        assert e.value.status == T._capi.TESS_E_STATE
        pool = (T.pinned_empty(used.value, np.int32), T.pinned_empty(used.value, np.float64))
        r1 = d.compute_all_to_host("fp32", face_pool=pool)
        c1 = [x.copy() for x in r1.csr()]
        r2 = d.compute_all_to_host("fp32", face_pool=pool)   # the same pool again
        for a, b in zip(c1, r2.csr()):
            assert np.array_equal(a, b)
        assert int(c1[0][-1]) == faces


def test_pageable_pool_is_refused(T):
    from tessellator import workloads

    L = T.lib()
    pts = workloads.uniform(2000, seed=15)
    with T.Diagram(pts, container=_box(T)) as d:
        n = len(pts)
        vol, fs, fc = np.empty(n), np.empty(n, dtype=np.uint64), np.empty(n, dtype=np.uint32)
        nbr, area = np.empty(40 * n, dtype=np.int32), np.empty(40 * n)
        st = L.tess_diagram_compute_all_to_host(d._h, T.PRECISION_FP32_GUARD, -1.0, -1, vol.ctypes.data,
                                                fs.ctypes.data, fc.ctypes.data, nbr.ctypes.data, area.ctypes.data,
                                                len(nbr), None)
        assert st == T._capi.TESS_E_INVALID
        assert "face_nbr" in T.last_error()


def test_device_pool(T):
    torch = pytest.importorskip("torch")
    from tessellator import workloads

    L = T.lib()
    pts = workloads.uniform(8000, seed=16)
    with T.Diagram(pts, container=_box(T)) as d:
        d.compute_all("fp32")
        offs, nbr, area = d.neighbors_csr()
        n = len(pts)
        cap = 30 * n
        dn = torch.empty(cap, dtype=torch.int32, device="cuda")
        da = torch.empty(cap, dtype=torch.float64, device="cuda")
        vol, fs, fc = np.empty(n), np.empty(n, dtype=np.uint64), np.empty(n, dtype=np.uint32)
        used = C.c_size_t(0)
        T.check(L.tess_diagram_compute_all_to_host(d._h, T.PRECISION_FP32_GUARD, -1.0, -1, vol.ctypes.data,
                                                   fs.ctypes.data, fc.ctypes.data, dn.data_ptr(), da.data_ptr(),
                                                   cap, C.byref(used)))
        r = T.HostResults(vol, fs, fc, dn[:used.value].cpu().numpy(), da[:used.value].cpu().numpy(), used.value)
        o2, n2, a2 = r.csr()
        assert np.array_equal(o2, offs) and np.array_equal(n2, nbr) and np.array_equal(a2, area)


def test_device_face_queries_need_a_new_compute(T):
    from tessellator import workloads

    pts = workloads.uniform(3000, seed=17)
    with T.Diagram(pts, container=_box(T)) as d:
        r = d.compute_all_to_host("fp32")
        assert np.array_equal(d.volumes(), r.volumes)   # volumes stay on the device too
        for call in (d.neighbors_csr, d.results_device, lambda: d.cell_faces(5)):
            with pytest.raises(T.TessError) as e:
                call()
            assert e.value.status == T._capi.TESS_E_STATE
        d.compute_all("fp32")
        offs, nbr, _ = d.neighbors_csr()
        assert np.array_equal(r.csr()[1], nbr)


def test_one_million_cells_properties(T):
    """At 1,048,576 uniform points: volumes sum to the box, and the neighbour
    relation read from the host pool is symmetric."""
    from tessellator import workloads

    pts = workloads.uniform(1_048_576, seed=18)
    with T.Diagram(pts, container=_box(T)) as d:
        r = d.compute_all_to_host("fp32")
    assert abs(r.volumes.sum() - 1.0) < 1e-6   # the FP32 form's per-cell bound
    offs, nbr, _ = r.csr()
    src = np.repeat(np.arange(len(pts), dtype=np.int64), np.diff(offs.astype(np.int64)))
    inner = nbr >= 0
    a = src[inner] * len(pts) + nbr[inner]
    b = nbr[inner].astype(np.int64) * len(pts) + src[inner]
    assert np.array_equal(np.sort(a), np.sort(b))


def _batch_inputs(sizes, seed):
    from tessellator import workloads

    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    pts = np.concatenate([workloads.uniform(s, seed=seed + k) for k, s in enumerate(sizes)])
    boxes = np.array([[0, 0, 0, 1, 1, 1]] * len(sizes), dtype=np.float64)
    return pts, offs, boxes


@pytest.mark.parametrize("prec", ["fp32", "mixed"])
def test_batch_same_results_as_compute(T, prec):
    pts, offs, boxes = _batch_inputs([64, 3000, 999, 5000, 17, 2048], 60)
    b = T.Batch(pts, offs, boxes)
    try:
        b.compute(prec)
        vol = b.volumes()
        co, cn, ca = b.neighbors_csr()
        pool_a = (T.pinned_empty(20 * len(pts), np.int32), T.pinned_empty(20 * len(pts), np.float64))
        pool_b = (T.pinned_empty(21 * len(pts), np.int32), T.pinned_empty(21 * len(pts), np.float64))
        # two pools in turn: each keeps its own captured graph valid
        for pool in (pool_a, pool_b, pool_a):
            r = b.compute_to_host(prec, face_pool=pool)
            assert np.array_equal(r.volumes, vol)
            o2, n2, a2 = r.csr()
            assert np.array_equal(o2, co) and np.array_equal(n2, cn) and np.array_equal(a2, ca)
        with pytest.raises(T.TessError) as e:
            b.neighbors_csr()
        assert e.value.status == T._capi.TESS_E_STATE
        # the library's own pool again
        b.compute(prec)
        assert np.array_equal(b.neighbors_csr()[1], cn)
    finally:
        b.close()


def test_batch_pool_too_small(T):
    pts, offs, boxes = _batch_inputs([2000, 3000], 70)
    L = T.lib()
    b = T.Batch(pts, offs, boxes)
    try:
        n = len(pts)
        small = (T.pinned_empty(500, np.int32), T.pinned_empty(500, np.float64))
        vol, fs, fc = np.empty(n), np.empty(n, dtype=np.uint64), np.empty(n, dtype=np.uint32)
        used = C.c_size_t(0)
        st = L.tess_batch_compute_to_host(b._h, T.PRECISION_FP32_GUARD, vol.ctypes.data, fs.ctypes.data,
                                          fc.ctypes.data, small[0].ctypes.data, small[1].ctypes.data, 500,
                                          C.byref(used))
        assert st == T._capi.TESS_E_CAPACITY and used.value > 500
        r = b.compute_to_host("fp32")   # allocates, and grows once if needed
        assert abs(r.volumes[:2000].sum() - 1.0) < 1e-6 and abs(r.volumes[2000:].sum() - 1.0) < 1e-6
    finally:
        b.close()


@pytest.mark.parametrize("radius,group", [(0.05, None), (None, 2), (0.08, 1)])
def test_radius_and_group_pass_through(T, radius, group):
    """search_radius and target_group mean what they mean for compute_all."""
    rng = np.random.default_rng(19)
    pts = rng.random((4000, 3))
    groups = (np.arange(len(pts)) % 3).astype(np.uint32)
    with T.Diagram(pts, groups=groups, container=_box(T)) as d:
        d.compute_all("fp32", search_radius=radius, target_group=group)
        vol = d.volumes()
        offs, nbr, area = d.neighbors_csr()
        r = d.compute_all_to_host("fp32", search_radius=radius, target_group=group)
    o2, n2, a2 = r.csr()
    assert np.array_equal(r.volumes, vol)
    assert np.array_equal(o2, offs) and np.array_equal(n2, nbr) and np.array_equal(a2, area)


@pytest.mark.parametrize("n", [1, 2, 9])
def test_tiny_diagrams(T, n):
    import oracle

    pts = np.random.default_rng(20 + n).random((n, 3))
    ref = oracle.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    rv, ro, ri, _, _, _ = ref.compute_all()
    with T.Diagram(pts, container=_box(T)) as d:
        r = d.compute_all_to_host("mixed")
    offs, nbr, _ = r.csr()
    assert np.allclose(r.volumes, rv, rtol=1e-11, atol=0)
    assert np.array_equal(offs.astype(np.int64), ro) and np.array_equal(nbr.astype(np.int64), ri)


def test_batch_fp64(T):
    pts, offs, boxes = _batch_inputs([500, 64, 2000], 80)
    b = T.Batch(pts, offs, boxes)
    try:
        b.compute("fp64")
        vol = b.volumes()
        co, cn, ca = b.neighbors_csr()
        r = b.compute_to_host("fp64")
        o2, n2, a2 = r.csr()
        assert np.array_equal(r.volumes, vol)
        assert np.array_equal(o2, co) and np.array_equal(n2, cn) and np.array_equal(a2, ca)
    finally:
        b.close()
