"""The reference-facing API on the GPU (Diagram / Cell / VoronoiFace of
interface.rs, through the C ABI) against the oracle, plus the batch path."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted_rows(a):
    a = np.round(np.asarray(a), 12)
    return a[np.lexsort(a.T[::-1])]


@pytest.fixture(scope="module")
def setup(tess, oracle_mod):
    rng = np.random.default_rng(31)
    pts = rng.random((2000, 3))
    d = tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1))
    d.compute_all("fp64")
    r = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    yield pts, d, r
    d.close()


@pytest.mark.parametrize("i", [0, 17, 999, 1999])
@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_cell_geometry(setup, i, prec):
    """Single-cell geometry; "mixed" runs these queries in the FP64 form."""
    pts, d, r = setup
    cell = d.get_cell_at_index(i, precision=prec).compute_voronoi_cell()
    ref = r.cell(i)
    tol = 1e-6 if prec == "fp32" else 1e-12
    assert math.isclose(cell.compute_volume(), ref.volume, rel_tol=tol)
    assert cell.compute_neighbors() == ref.ids.tolist()
    assert cell.original_index() == i
    # vertices: the same point set (site-relative, as the reference leaves them)
    v = cell.compute_vertices()
    assert len(v) == len(ref.vertices)
    np.testing.assert_allclose(_sorted_rows(v), _sorted_rows(ref.vertices), atol=1e-6 if prec == "fp32" else 1e-12)
    faces = cell.compute_faces()
    assert len(faces) == len(ref.ids)
    for f, (rid, rarea, rfv) in enumerate(zip(ref.ids, ref.areas, ref.face_vertices)):
        face = faces[f]
        assert face.compute_neighbor() == rid
        assert math.isclose(face.compute_area(), rarea, rel_tol=1e-5 if prec == "fp32" else 1e-10)
        fv = face.compute_vertices()
        assert len(fv) == len(rfv)
        # same cycle up to rotation, counter-clockwise seen from outside
        k = int(np.argmin(np.linalg.norm(fv - rfv[0], axis=1)))
        np.testing.assert_allclose(np.roll(fv, -k, axis=0), rfv, atol=1e-6 if prec == "fp32" else 1e-12)


def test_bulk_queries_match_cell_queries(setup):
    pts, d, r = setup
    offs, nbr, area = d.neighbors_csr()
    vol = d.volumes()
    for i in (3, 400, 1500):
        ids, ar = d.cell_faces(i)
        assert ids.tolist() == nbr[offs[i]:offs[i + 1]].tolist()
        np.testing.assert_array_equal(ar, area[offs[i]:offs[i + 1]])
        assert d.cell_volume(i) == vol[i]
        assert d.cell_neighbors(i).tolist() == ids.tolist()
        v = d.cell_vertices(i)
        assert len(v) == len(r.cell(i).vertices)
        fv = d.cell_face_vertices(i, 0)
        assert len(fv) >= 3


def test_cell_at_particle(setup, tess):
    pts, d, r = setup
    for p in ([0.5, 0.5, 0.5], [0.01, 0.99, 0.3], [0.0, 0.0, 0.0]):
        cell = d.get_cell_at_particle(p).compute_voronoi_cell()
        ref = r.cell_at(p)
        assert math.isclose(cell.compute_volume(), ref.volume, rel_tol=1e-12)
        assert cell.compute_neighbors() == ref.ids.tolist()
        assert cell.original_index() is None


def test_cell_with_own_container(tess, oracle_mod):
    """The Polyhedron argument of get_cell_at_index sets the walls of that cell."""
    rng = np.random.default_rng(32)
    pts = rng.random((500, 3))
    d = tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1))
    poly = tess.Polyhedron(0.2, 0.2, 0.2, 0.8, 0.8, 0.8)
    r = oracle_mod.Diagram(pts, lo=[0.2] * 3, hi=[0.8] * 3)
    i = int(np.argmin(np.linalg.norm(pts - 0.5, axis=1)))
    cell = d.get_cell_at_index(i, polyhedron=poly).compute_voronoi_cell()
    ref = r.cell(i)
    assert math.isclose(cell.compute_volume(), ref.volume, rel_tol=1e-12)
    assert cell.compute_neighbors() == ref.ids.tolist()
    d.close()


def test_cell_radius_and_group(tess, oracle_mod):
    rng = np.random.default_rng(33)
    pts = rng.random((1500, 3))
    groups = (np.arange(1500) % 4).astype(np.uint32)
    d = tess.Diagram(pts, groups=groups, container=tess.Polyhedron(0, 0, 0, 1, 1, 1))
    r = oracle_mod.Diagram(pts, groups=groups, lo=[0, 0, 0], hi=[1, 1, 1])
    for i in (5, 77):
        c = d.get_cell_at_index(i, search_radius=0.003, target_group=2).compute_voronoi_cell()
        ref = r.cell(i, mode=oracle_mod.MODE_RADIUS, radius=0.003, target_group=2)
        assert math.isclose(c.compute_volume(), ref.volume, rel_tol=1e-12)
        assert c.compute_neighbors() == ref.ids.tolist()
    d.close()


def test_update_points_and_rebuild(tess, oracle_mod):
    rng = np.random.default_rng(34)
    a, b = rng.random((3000, 3)), rng.random((3000, 3))
    d = tess.Diagram(a, container=tess.Polyhedron(0, 0, 0, 1, 1, 1))
    d.compute_all("fp32")
    va = d.volumes()
    d.update_points(b)
    d.compute_all("fp32")
    vb = d.volumes()
    rb = oracle_mod.Diagram(b, lo=[0, 0, 0], hi=[1, 1, 1]).compute_all()[0]
    assert np.max(np.abs(vb - rb) / rb) <= 1e-6
    d.update_points(a)
    d.rebuild()
    d.compute_all("fp32")
    assert np.array_equal(d.volumes(), va)      # deterministic
    d.close()


def test_batch_matches_single_diagrams(tess, oracle_mod):
    from tessellator import workloads

    pts, offs, boxes = workloads.batched(ndiag=40, seed=35, nmin=64, nmax=4096)
    for prec in ("fp64", "fp32", "mixed"):
        b = tess.Batch(pts, offs, boxes)
        b.compute(prec)
        vol = b.volumes()
        coffs, nbr, area = b.neighbors_csr()
        st = b.stats()
        assert st["failed"] == 0
        for dgi in range(len(offs) - 1):
            s, e = int(offs[dgi]), int(offs[dgi + 1])
            r = oracle_mod.Diagram(pts[s:e], lo=boxes[dgi, :3], hi=boxes[dgi, 3:])
            rv, ro, ri, ra, _, _ = r.compute_all()
            tol = 1e-6 if prec == "fp32" else 1e-12
            assert np.max(np.abs(vol[s:e] - rv) / rv) <= tol
            assert math.isclose(vol[s:e].sum(), float(np.prod(boxes[dgi, 3:])), rel_tol=tol * 10)
            got = nbr[int(coffs[s]):int(coffs[e])].astype(np.int64)
            assert np.array_equal(got, ri)
        # a second launch replays the captured graph with the same results
        b.compute(prec)
        assert np.array_equal(b.volumes(), vol)
        b.close()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_timing_flag(tess, oracle_mod, prec):
    """With TESS_FLAG_TIMING the per-pass times are recorded and every later
    call still succeeds (twice in a row, CSR and a radius query included)."""
    rng = np.random.default_rng(33)
    pts = rng.random((30000, 3))
    cfg = tess.default_config(flags=tess.FLAG_TIMING)
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1), config=cfg) as d:
        for _ in range(2):
            d.rebuild()
            d.compute_all(prec)
            offs, nbr, area = d.neighbors_csr()
            st = d.stats()
            assert st["ms_grid"] > 0 and st["ms_clip"] > 0 and st["ms_csr"] > 0
            qo, qi = d.find_neighbors_in_radius_batch(pts[:20000], 0.03, True)
            assert len(qi) > 20000 and qo[-1] == len(qi)
            assert d.stats()["ms_query_count"] > 0 and d.stats()["ms_query_fill"] > 0
        vol = d.volumes()
    rvol, roffs, rids, _, _, _ = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1]).compute_all()
    assert offs.astype(np.int64).tolist() == roffs.tolist()
    assert nbr.astype(np.int64).tolist() == rids.tolist()
    np.testing.assert_allclose(vol, rvol, rtol=1e-6 if prec == "fp32" else 1e-12)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_work_counters_flag(tess, prec):
    """TESS_FLAG_COUNTERS counts the clipping work (every pass, every form)
    and leaves the results as they are without it."""
    rng = np.random.default_rng(34)
    pts = rng.random((20000, 3))
    box = tess.Polyhedron(0, 0, 0, 1, 1, 1)
    with tess.Diagram(pts, container=box) as d:
        d.compute_all(prec)
        plain = (d.volumes(), *d.neighbors_csr())
        assert d.stats()["candidates_tested"] == 0
    cfg = tess.default_config(flags=tess.FLAG_COUNTERS)
    with tess.Diagram(pts, container=box, config=cfg) as d:
        d.compute_all(prec)
        counted = (d.volumes(), *d.neighbors_csr())
        st = d.stats()
    n = len(pts)
    assert 5 * n < st["cuts"] < 40 * n
    assert st["cuts"] < st["candidates_tested"] < 200 * n
    assert st["new_vertices"] > 2 * st["cuts"]
    # the counting form may send a different few cells to a re-run: FP32-form
    # values agree to their tolerance, neighbour lists exactly
    tol = 1e-6 if prec == "fp32" else 0.0
    np.testing.assert_allclose(counted[0], plain[0], rtol=tol)
    assert np.array_equal(counted[1], plain[1]) and np.array_equal(counted[2], plain[2])
    np.testing.assert_allclose(counted[3], plain[3], rtol=0, atol=1e-5 if prec == "fp32" else 0.0)

