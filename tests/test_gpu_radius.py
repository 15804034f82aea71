"""Fixed-radius queries on the GPU (find_cells_in_radius,
find_neighbors_in_{cell,real}_radius: celery.rs:753-855; compute_neighbor_cloud:
interface.rs:348-365) through the C ABI, against the reference's own unit
tests (celery.rs:1459-1900) and bit for bit against the oracle: the same bins
and points in the same order."""
import ctypes as C

import numpy as np
import pytest

import radius_cases as RC

pytestmark = pytest.mark.gpu


def _same(got, want):
    (go, gv), (wo, wv) = got, want
    assert np.array_equal(go.astype(np.uint64), wo.astype(np.uint64))
    assert np.array_equal(gv.astype(np.uint32), wv.astype(np.uint32))


# ---- the reference's unit tests --------------------------------------------------
def test_find_cells_in_radius_kat(tess, oracle_mod):          # celery.rs:1665-1753
    pts = RC.celery4(2)
    with tess.Diagram(pts) as d:
        for q, r in RC.FIND_CELLS_CASES:
            got = set(d.find_cells_in_radius(q, q, q, r))
            want = {RC.bin_id(i, j, k) for i in range(4) for j in range(4) for k in range(4)
                    if RC.find_cells_expected(q, r, i, j, k)}
            assert got == want, (q, r)


@pytest.mark.parametrize("real", [False, True])
def test_find_neighbors_kat(tess, real):                      # celery.rs:1756-1900
    pts = RC.celery4_marked(-0.1 if real else -0.3, seed=3)
    with tess.Diagram(pts) as d:
        ids = np.array(d.find_neighbors_in_real_radius(0.5, 0.5, 0.5, 1.73) if real else
                       d.find_neighbors_in_cell_radius(0.5, 0.5, 0.5, 1.73))
    want = RC.REAL_RADIUS_MARKED if real else RC.CELL_RADIUS_MARKED
    for idx, count in want.items():
        assert int(np.count_nonzero(ids == idx)) == count, idx


def test_neighbor_cloud_kat(tess):                            # celery.rs:1459-1487
    pts = RC.celery4(4)
    with tess.Diagram(pts) as d:
        ids = d.get_cell_at_particle([0.0, 0.0, 0.0]).compute_neighbor_cloud(0.5)
        assert 77 in ids and 78 not in ids and len(ids) < 79
        ids = d.get_cell_at_particle([0.0, 0.0, 0.0]).compute_neighbor_cloud(10.0)
        assert 77 in ids and 78 in ids and len(ids) == 79


# ---- parity with the oracle ------------------------------------------------------
@pytest.fixture(scope="module")
def uniform(tess, oracle_mod):
    rng = np.random.default_rng(71)
    pts = rng.random((20000, 3))
    groups = rng.integers(0, 4, len(pts)).astype(np.uint32)
    q = np.vstack([rng.uniform(-0.1, 1.1, (1500, 3)), pts[:500], [[0.5, 0.5, 0.5], [2.0, -1.0, 0.5]]])
    d = tess.Diagram(pts, groups=groups)
    yield pts, groups, q, d, oracle_mod.Diagram(pts, groups=groups)
    d.close()


@pytest.mark.parametrize("r", [-2.0, -0.5, 0.0, 0.004, 0.02, 0.05, 0.11, float("nan"), float("inf")])
def test_find_cells_parity(uniform, r):
    _, _, q, d, o = uniform
    if not np.isfinite(r):
        q = q[::20]                     # every bin for every query: keep the output small
    _same(d.find_cells_in_radius_batch(q, r), o.find_cells_in_radius(q, r))


@pytest.mark.parametrize("real", [False, True])
@pytest.mark.parametrize("r", [-0.5, 0.0, 0.004, 0.02, 0.05, 0.11, float("nan")])
def test_find_neighbors_parity(uniform, r, real):
    _, _, q, d, o = uniform
    _same(d.find_neighbors_in_radius_batch(q, r, real), o.find_neighbors_in_radius(q, r, real))


@pytest.mark.parametrize("group", [-1, 0, 3, 7])
@pytest.mark.parametrize("r", [-2.0, -1.0, -0.5, 0.0, 0.0004, 0.003, 0.02, float("nan")])
def test_neighbor_cloud_parity(uniform, r, group):
    pts, _, q, d, o = uniform
    if np.isnan(r) and group == -1:
        q = q[:50]                      # every point for every query: keep the output small
    cells = np.arange(0, len(pts), 97, dtype=np.uint32)
    _same(d.neighbor_cloud(r, cells, None if group < 0 else group), o.neighbor_cloud(pts[cells], r, group))
    _same(d.neighbor_cloud_at(q, r, None if group < 0 else group), o.neighbor_cloud(q, r, group))


def test_neighbor_cloud_every_cell(uniform):
    pts, _, _, d, o = uniform
    _same(d.neighbor_cloud(0.002), o.neighbor_cloud(pts, 0.002))


def test_clustered_bins(tess, oracle_mod):
    """Bins holding hundreds of points: the point stream spans many 32-lane steps."""
    rng = np.random.default_rng(72)
    pts = np.vstack([rng.normal(0.5, 0.004, (6000, 3)), rng.random((2000, 3))])
    q = np.vstack([pts[::40], rng.random((100, 3))])
    with tess.Diagram(pts) as d:
        o = oracle_mod.Diagram(pts)
        for r in (0.003, 0.01, 0.06):
            _same(d.find_neighbors_in_radius_batch(q, r, True), o.find_neighbors_in_radius(q, r, True))
            _same(d.find_neighbors_in_radius_batch(q, r, False), o.find_neighbors_in_radius(q, r, False))
        for r in (0.0, 0.001, 0.01):
            _same(d.neighbor_cloud_at(q, r), o.neighbor_cloud(q, r))


@pytest.mark.parametrize("r", [1.0, 2.0, 2.0 ** 0.5, 3.0 ** 0.5, 0.999999999])
def test_real_radius_ties_on_the_sphere(tess, oracle_mod, r):
    """Integer lattice: many candidates at exactly the radius (d^2 == r^2), where
    the FP32 pre-filter must defer to the exact FP64 test."""
    g = np.arange(12, dtype=np.float64)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    q = np.vstack([pts[::7], pts[::11] + 0.5])
    with tess.Diagram(pts) as d:
        o = oracle_mod.Diagram(pts)
        _same(d.find_neighbors_in_radius_batch(q, r, True), o.find_neighbors_in_radius(q, r, True))


def test_real_radius_far_from_the_origin(tess, oracle_mod):
    """Coordinates near 1e6: the FP32 filter's error band is wide and most
    decisions fall back to FP64."""
    rng = np.random.default_rng(75)
    pts = 1.0e6 + rng.random((20000, 3))
    q = 1.0e6 + rng.uniform(-0.1, 1.1, (500, 3))
    with tess.Diagram(pts) as d:
        o = oracle_mod.Diagram(pts)
        for r in (0.03, 0.1):
            _same(d.find_neighbors_in_radius_batch(q, r, True), o.find_neighbors_in_radius(q, r, True))
            _same(d.find_cells_in_radius_batch(q, r), o.find_cells_in_radius(q, r))


def test_real_radius_million_points(tess, oracle_mod):
    """1,000,000 points, 100,000 queries, radius 0.012 (about 9 neighbours each)."""
    rng = np.random.default_rng(73)
    pts = rng.random((1_000_000, 3))
    q = rng.random((100_000, 3))
    with tess.Diagram(pts) as d:
        got = d.find_neighbors_in_radius_batch(q, 0.012, True)
    _same(got, oracle_mod.Diagram(pts).find_neighbors_in_radius(q, 0.012, True))
    assert 5 < len(got[1]) / len(q) < 12


def test_large_batches_in_spatial_order(tess, oracle_mod):
    """Batches of 65,536 queries or more are processed in coarse-bin order;
    results stay in query order."""
    rng = np.random.default_rng(74)
    pts = rng.random((300_000, 3))
    cells = rng.permutation(len(pts)).astype(np.uint32)[:150_000]
    q = rng.uniform(-0.05, 1.05, (120_000, 3))
    with tess.Diagram(pts) as d:
        o = oracle_mod.Diagram(pts)
        _same(d.neighbor_cloud(0.0002, cells), o.neighbor_cloud(pts[cells], 0.0002))
        _same(d.neighbor_cloud_at(q, 0.0002), o.neighbor_cloud(q, 0.0002))
        _same(d.find_neighbors_in_radius_batch(q, 0.02, True), o.find_neighbors_in_radius(q, 0.02, True))
        _same(d.find_cells_in_radius_batch(q, 0.01), o.find_cells_in_radius(q, 0.01))


# ---- the C ABI's contract ---------------------------------------------------------
def test_capacity_and_errors(tess, uniform):
    _, _, q, d, _ = uniform
    L = tess.lib()
    qq = np.ascontiguousarray(q[:10])
    offs = np.zeros(11, dtype=np.uint64)
    out = np.zeros(4, dtype=np.uint32)
    total = C.c_size_t(0)
    st = L.tess_find_neighbors_in_radius(d._h, C.c_void_p(qq.ctypes.data), 10, 0.05, 0, 0,
                                         C.c_void_p(offs.ctypes.data), C.c_void_p(out.ctypes.data), 4,
                                         C.byref(total))
    assert st == 3 and total.value > 4 and offs[10] == total.value       # TESS_E_CAPACITY, sizes reported
    bad = np.array([0, 20000], dtype=np.uint32)
    st = L.tess_neighbor_cloud(d._h, C.c_void_p(bad.ctypes.data), 2, 0.01, -1, 0, None, None, 0, C.byref(total))
    assert st == 1 and "out of range" in tess.last_error()
    st = L.tess_neighbor_cloud(d._h, None, 5, 0.01, -1, 0, None, None, 0, C.byref(total))
    assert st == 1                                                        # NULL cells needs ncells = n
    offs1 = np.ones(1, dtype=np.uint64)
    st = L.tess_find_cells_in_radius(d._h, None, 0, 0.1, 0, C.c_void_p(offs1.ctypes.data), None, 0,
                                     C.byref(total))
    assert st == 0 and total.value == 0 and offs1[0] == 0                 # no queries


def test_device_pointers(tess, uniform):
    torch = pytest.importorskip("torch")
    _, _, q, d, _ = uniform
    L = tess.lib()
    want_offs, want = d.find_neighbors_in_radius_batch(q, 0.03, True)
    dq = torch.from_numpy(np.ascontiguousarray(q)).to("cuda:0")
    doffs = torch.zeros(len(q) + 1, dtype=torch.int64, device="cuda:0")
    dout = torch.zeros(len(want) + 5, dtype=torch.int32, device="cuda:0")
    total = C.c_size_t(0)
    torch.cuda.synchronize()            # the library runs on its own stream
    st = L.tess_find_neighbors_in_radius(d._h, C.c_void_p(dq.data_ptr()), len(q), 0.03, 1, 1,
                                         C.c_void_p(doffs.data_ptr()), C.c_void_p(dout.data_ptr()), dout.numel(),
                                         C.byref(total))
    assert st == 0, tess.last_error()
    torch.cuda.synchronize()
    assert total.value == len(want)
    assert doffs.cpu().numpy().astype(np.uint64).tolist() == want_offs.tolist()
    assert dout[: len(want)].cpu().numpy().astype(np.uint32).tolist() == want.tolist()
    bad = torch.tensor([3, 20000], dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    st = L.tess_neighbor_cloud(d._h, C.c_void_p(bad.data_ptr()), 2, 0.01, -1, 1, None, None, 0, C.byref(total))
    assert st == 1 and "out of range" in tess.last_error()                # flagged on the device
