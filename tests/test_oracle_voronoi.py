"""Pins the oracle's Voronoi outputs, which the reference's tests leave
unpinned: against scipy/Qhull (committed golden fixtures and live), analytic
lattices, exact invariants, and the reference semantics of its search modes."""
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def csr_sets(offs, ids):
    return [set(ids[offs[i]:offs[i + 1]].tolist()) for i in range(len(offs) - 1)]


def test_golden_qhull_uniform(oracle_mod):
    """Interior cells of 2,000 uniform points against Qhull volumes and ridge
    neighbours (fixture made by tests/golden/make_golden.py)."""
    z = np.load(os.path.join(GOLDEN, "qhull_uniform_2000.npz"))
    d = oracle_mod.Diagram(z["points"], lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, areas, _, _ = d.compute_all()
    cells = z["cells"]
    assert len(cells) > 1200
    np.testing.assert_allclose(vol[cells], z["volumes"], rtol=1e-10)
    noffs = z["nbr_offsets"]
    for t, i in enumerate(cells):
        assert set(ids[offs[i]:offs[i + 1]].tolist()) == set(z["nbr"][noffs[t]:noffs[t + 1]].tolist())


def test_golden_oracle_small(oracle_mod):
    """A small diagram's full output, pinned so regressions show."""
    z = np.load(os.path.join(GOLDEN, "oracle_uniform_500.npz"))
    d = oracle_mod.Diagram(z["points"], lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, areas, _, _ = d.compute_all()
    np.testing.assert_allclose(vol, z["volumes"], rtol=1e-13)
    assert np.array_equal(offs, z["offsets"])
    assert np.array_equal(ids, z["ids"])
    np.testing.assert_allclose(areas, z["areas"], rtol=1e-10, atol=1e-15)


def test_qhull_live(oracle_mod):
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(21)
    pts = rng.random((1500, 3))
    d = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, _, _, _ = d.compute_all()
    vor = spatial.Voronoi(pts)
    checked = 0
    for i in range(len(pts)):
        reg = vor.regions[vor.point_region[i]]
        if -1 in reg or not reg:
            continue
        V = vor.vertices[reg]
        if V.min() < 0 or V.max() > 1:
            continue
        assert math.isclose(spatial.ConvexHull(V).volume, vol[i], rel_tol=1e-10)
        checked += 1
    assert checked > 800


@pytest.mark.parametrize("gen", ["uniform", "clustered", "crowded"])
def test_secure_equals_brute_bit_exact(oracle_mod, gen):
    """The security-radius stop changes nothing: the same cuts happen in the
    same order as the reference's walk over every point (celery.rs:971).
    "crowded": bins of several hundred points, as in clustered inputs."""
    rng = np.random.default_rng(22)
    if gen == "uniform":
        pts = rng.random((1200, 3))
    elif gen == "clustered":
        c = 0.2 + 0.6 * rng.random((4, 3))
        pts = np.clip(c[rng.integers(0, 4, 1200)] + 0.03 * rng.standard_normal((1200, 3)), 0, 1)
    else:
        c = 0.2 + 0.6 * rng.random((3, 3))
        pts = np.vstack([c[rng.integers(0, 3, 2400)] + 0.004 * rng.standard_normal((2400, 3)),
                         rng.random((300, 3))])
        pts = np.clip(pts, 0, 1)
        counts = np.diff(oracle_mod.Diagram(pts).delimiters())
        assert counts.max() >= 300
    d = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    a = d.compute_all(mode=oracle_mod.MODE_SECURE)
    b = d.compute_all(mode=oracle_mod.MODE_BRUTE)
    for x, y in zip(a[:4], b[:4]):
        assert np.array_equal(x, y)


def test_volume_sum_and_symmetry(oracle_mod):
    rng = np.random.default_rng(23)
    lo, hi = np.array([-1.0, 0.5, 2.0]), np.array([2.0, 1.5, 2.5])
    pts = lo + (hi - lo) * rng.random((3000, 3))
    d = oracle_mod.Diagram(pts, lo=lo, hi=hi)
    vol, offs, ids, _, _, _ = d.compute_all()
    assert abs(vol.sum() - np.prod(hi - lo)) <= 1e-12 * np.prod(hi - lo)
    sets = csr_sets(offs, ids)
    assert all(i in sets[j] for i, s in enumerate(sets) for j in s if j >= 0)


def test_simple_cubic_lattice(oracle_mod):
    """Exact lattice: every cell is the cube of side h with 6 faces of area h^2."""
    m = 6
    h = 1.0 / m
    g = (np.arange(m) + 0.5) * h
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    d = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, areas, _, _ = d.compute_all()
    np.testing.assert_allclose(vol, h ** 3, rtol=1e-12)
    assert np.all(np.diff(offs) == 6)
    np.testing.assert_allclose(areas, h * h, rtol=1e-12)


def test_bcc_lattice(oracle_mod):
    """Interior cells of a BCC lattice are truncated octahedra: volume a^3 / 2,
    8 hexagons of area 3 sqrt(3) a^2 / 16 and 6 squares of area a^2 / 8."""
    m = 5
    a = 1.0 / m
    g1, g2 = (np.arange(m) + 0.25) * a, (np.arange(m) + 0.75) * a
    pts = np.concatenate([np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) for g in (g1, g2)])
    d = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, areas, _, _ = d.compute_all()
    assert abs(vol.sum() - 1.0) < 1e-12
    inner = np.where(np.all((pts > 1.5 * a) & (pts < 1 - 1.5 * a), axis=1))[0]
    assert len(inner) > 10
    hexa, sq = 3 * math.sqrt(3) * a * a / 16, a * a / 8
    for i in inner:
        assert math.isclose(vol[i], a ** 3 / 2, rel_tol=1e-12)
        ar = np.sort(areas[offs[i]:offs[i + 1]])
        assert len(ar) == 14
        np.testing.assert_allclose(ar[:6], sq, rtol=1e-12)
        np.testing.assert_allclose(ar[6:], hexa, rtol=1e-12)


def test_radius_mode_is_a_superset_limit(oracle_mod):
    """Some(radius): a large radius reproduces the exact cells; radius 0 keeps
    only the own bin and the 26 touching bins."""
    rng = np.random.default_rng(24)
    pts = rng.random((800, 3))
    d = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    exact = d.compute_all()
    big = d.compute_all(mode=oracle_mod.MODE_RADIUS, radius=10.0)
    for x, y in zip(exact[:4], big[:4]):
        assert np.array_equal(x, y)
    small = d.compute_all(mode=oracle_mod.MODE_RADIUS, radius=0.0)
    assert np.all(small[0] >= exact[0] * (1 - 1e-12))


def test_target_group_and_external_point(oracle_mod):
    rng = np.random.default_rng(25)
    pts = rng.random((600, 3))
    groups = (np.arange(600) % 2).astype(np.uint32)
    d = oracle_mod.Diagram(pts, groups=groups, lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, _, _, _ = d.compute_all(target_group=1)
    sets = csr_sets(offs, ids)
    assert all(j < 0 or groups[j] == 1 for s in sets for j in s)
    # group-1 cells cut by group-1 points only tile the box among themselves
    assert abs(vol[groups == 1].sum() - 1.0) < 1e-12
    # a point not in the diagram (get_cell_at_particle): no self exclusion
    c = d.cell_at([0.5, 0.5, 0.5])
    assert 0 < c.volume < 1
    c2 = d.cell_at(pts[7])
    assert c2.volume == 0.0 or 7 not in c2.ids.tolist()


def test_face_vertex_cycles_are_outward(oracle_mod):
    rng = np.random.default_rng(26)
    pts = rng.random((300, 3))
    d = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    c = d.cell(17)
    vol = 0.0
    for fv, area in zip(c.face_vertices, c.areas):
        a = fv[0]
        wn = sum(np.cross(fv[t] - a, fv[t + 1] - a) for t in range(1, len(fv) - 1))
        assert math.isclose(0.5 * np.linalg.norm(wn), area, rel_tol=1e-12)
        vol += a @ wn / 6
    assert math.isclose(vol, c.volume, rel_tol=1e-12)
