"""The oracle against the known answers the reference's own unit tests pin
(mcomstock/the-tessellator: src/vector3.rs:301-477, src/celery.rs:1078-1487,
src/polyhedron.rs:938-1119).  Values are restated from those tests."""
import math

import numpy as np
import pytest


# ---- vector3.rs --------------------------------------------------------------
def test_dot(oracle_mod):                      # vector3.rs:315-322
    O = oracle_mod
    assert O.dot([1, 2, 3], [4, 5, 6]) == 32.0
    assert O.dot([4, 5, 6], [1, 2, 3]) == 32.0


def test_location_with_tolerance(oracle_mod):  # vector3.rs:352-365
    O = oracle_mod
    plane = [1.0, 0.0, 0.0, 0.0]               # signed distance = x
    assert O.vector_location(plane, [1.0, 0, 0], 0.01) == 1      # Outside
    assert O.vector_location(plane, [-1.0, 0, 0], 0.01) == -1    # Inside
    assert O.vector_location(plane, [0.005, 0, 0], 0.01) == 0    # Incident


def test_vector_location(oracle_mod):          # vector3.rs:367-384
    O = oracle_mod
    p = [1.0, 0.0, 0.0, 1.0]                   # plane x = 1
    assert O.vector_location(p, [4, 2, -6], 0.05) == 1
    assert O.vector_location(p, [-3, -3, -3], 0.05) == -1
    assert O.vector_location(p, [1, -6, 0], 0.05) == 0


def test_intersection(oracle_mod):             # vector3.rs:386-398
    O = oracle_mod
    out = O.intersection([1.0, 0.0, 0.0, 1.0], [20, 0, 0], [10, 10, 0])
    assert out.tolist() == [1.0, 19.0, 0.0]


@pytest.mark.parametrize("p", [[1, 1, 1], [-1, 1, 1], [-1, -1, -1]])
def test_halfway_from_origin_to(oracle_mod, p):  # vector3.rs:440-476
    O = oracle_mod
    got = O.halfway_from_origin_to(p)
    half = 0.5 * np.asarray(p, dtype=float)
    want = O.plane_from_non_unit_normal_and_point(half, half)
    assert got.tolist() == want.tolist()       # bitwise equal, as assert_eq! on Float64


def test_cross(oracle_mod):
    assert oracle_mod.cross([1, 0, 0], [0, 1, 0]).tolist() == [0, 0, 1]


# ---- celery.rs ---------------------------------------------------------------
def check_delimiters(cells, sorted_indices, delimiters):
    """The reference's CSR invariant checker (celery.rs:1131-1172)."""
    assert delimiters[0] == 0
    assert delimiters[-1] == len(sorted_indices)
    assert len(set(sorted_indices.tolist())) == len(sorted_indices)
    for i in range(1, len(delimiters)):
        assert delimiters[i] == 0 or i > cells[sorted_indices[delimiters[i] - 1]]
        if delimiters[i] == len(sorted_indices):
            assert np.all(delimiters[i + 1:] == len(sorted_indices))
            return
        same = i == cells[sorted_indices[delimiters[i]]]
        greater = i > cells[sorted_indices[delimiters[i]]]
        empty = delimiters[i] == delimiters[i + 1]
        assert same or greater or empty


BOXES = [((0, 1), (0, 1), (0, 1)), ((-1000, 500),) * 3, ((-5, -4), (12, 1000), (-10000, 1))]


@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("n,cpd,so,dl", [(1, 1, 1, 2), (1000, 10, 6859, 1001)])
def test_insert_points(oracle_mod, box, n, cpd, so, dl):   # celery.rs:1226-1301
    O = oracle_mod
    rng = np.random.default_rng(n)
    lo = np.array([b[0] for b in box], float)
    hi = np.array([b[1] for b in box], float)
    pts = lo + (hi - lo) * rng.random((n, 3))
    d = O.Diagram(pts)
    g = d.grid()
    assert g.cpd == cpd
    ijk, dist = O.search_order(g)
    assert len(ijk) == so
    delims = d.delimiters()
    assert len(delims) == dl
    check_delimiters(d.bins(), d.sorted_indices(), delims)


def test_insert_one_million_points_sizes(oracle_mod):      # celery.rs:1303-1315 (commented out there)
    O = oracle_mod
    assert O.cells_per_dimension(1_000_000) == 93
    assert (2 * 93 - 1) ** 3 == 6331625
    assert 93 ** 3 + 1 == 804358


@pytest.mark.parametrize("n,cpd", [(10000, 21), (16_777_216, 238), (4_194_304, 150), (128 ** 3, 119),
                                   (2_000_000, 117), (79, 4), (100, 5)])
def test_cells_per_dimension(oracle_mod, n, cpd):
    """(n / 1.25).cbrt() as usize + 1; 10000 / 1.25 = 8000 is an exact cube."""
    assert oracle_mod.cells_per_dimension(n) == cpd


def test_search_order_keys_sorted_and_self_first(oracle_mod):
    O = oracle_mod
    pts = np.random.default_rng(3).random((1000, 3))
    g = O.Diagram(pts).grid()
    ijk, dist = O.search_order(g)
    assert ijk[0].tolist() == [0, 0, 0] and dist[0] == -1.0     # celery.rs:438-443
    assert np.all(np.diff(dist) >= 0)
    # the 26 neighbouring bins have gap distance 0
    assert np.sum(dist == 0.0) == 26
    for t in range(0, len(ijk), 97):
        assert dist[t] == O.gap_key(g, *ijk[t])


@pytest.mark.parametrize("query,bins", [((0.5, 0.5, 0.5), (2, 2, 2)), ((0.0, 0.0, 0.0), (0, 0, 0))])
def test_expanding_search_visits_all(oracle_mod, query, bins):   # celery.rs:1343-1404
    O = oracle_mod
    pts = np.random.default_rng(5).random((100, 3))
    d = O.Diagram(pts)
    g = d.grid()
    assert g.cpd == 5
    assert len(d.delimiters()) == 126
    ijk, _ = O.search_order(g)
    assert len(ijk) == 729
    b = [O.axis_index(query[0], g.xmin, g.xmax, g.ix, g.cpd),
         O.axis_index(query[1], g.ymin, g.ymax, g.iy, g.cpd),
         O.axis_index(query[2], g.zmin, g.zmax, g.iz, g.cpd)]
    assert tuple(b) == bins
    dl, srt = d.delimiters(), d.sorted_indices()
    found = []
    for o in ijk:                               # one bin per expand(.., 1) call
        x, y, z = b[0] + o[0], b[1] + o[1], b[2] + o[2]
        if min(x, y, z) < 0 or max(x, y, z) >= g.cpd:
            continue
        c = (x * g.cpd + y) * g.cpd + z
        found.extend(srt[dl[c]:dl[c + 1]].tolist())
    assert sorted(found) == list(range(100))


def test_expand_all_in_radius(oracle_mod):      # celery.rs:1459-1487
    O = oracle_mod
    pts = -2.0 + 4.0 * np.random.default_rng(6).random((79, 3))
    pts[77] = [2.0, 2.0, 2.0]
    pts[78] = [-2.0, -2.0, -2.0]
    d = O.Diagram(pts)
    g = d.grid()
    assert g.cpd == 4
    ijk, dist = O.search_order(g)
    b = [O.axis_index(0.0, g.xmin, g.xmax, g.ix, 4)] * 3
    assert b == [2, 2, 2]
    dl, srt = d.delimiters(), d.sorted_indices()

    def expand(radius):
        out = []
        for o, key in zip(ijk, dist):
            if key > radius:                     # squared gap vs radius (celery.rs:1036)
                break
            x, y, z = b[0] + o[0], b[1] + o[1], b[2] + o[2]
            if min(x, y, z) < 0 or max(x, y, z) >= 4:
                continue
            c = (x * 4 + y) * 4 + z
            out.extend(srt[dl[c]:dl[c + 1]].tolist())
        return out

    r = expand(0.5)
    assert 77 in r and 78 not in r and len(r) < 79
    r = expand(10.0)
    assert 77 in r and 78 in r and len(r) == 79


# ---- polyhedron.rs -----------------------------------------------------------
def test_box_cell(oracle_mod):                  # polyhedron.rs:952-974 (new_test)
    O = oracle_mod
    d = O.Diagram([[-1.0, 70.0, -0.15]], lo=[-3.0, 40.0, -0.2], hi=[0.0, 100.0, -0.1])
    c = d.cell(0)
    assert len(c.vertices) == 8 and len(c.ids) == 6
    assert c.ids.tolist() == [-6, -5, -4, -3, -2, -1]
    site = np.array([-1.0, 70.0, -0.15])
    for v in c.vertices + site:
        assert v[0] in (0.0, -3.0) or abs(v[0]) < 1e-12 or abs(v[0] + 3.0) < 1e-12
    assert math.isclose(c.volume, 3.0 * 60.0 * 0.1, rel_tol=1e-12)


def test_plane_outside_the_cube_cuts_nothing(oracle_mod):   # polyhedron.rs:1021-1034
    O = oracle_mod
    # the bisector of the origin and (4,4,4) is the plane through (2,2,2)
    d = O.Diagram([[0.0, 0.0, 0.0], [4.0, 4.0, 4.0]], lo=[-1, -1, -1], hi=[1, 1, 1])
    c = d.cell(0)
    assert c.volume == 8.0 and len(c.ids) == 6


def test_corner_cut(oracle_mod):                 # polyhedron.rs:1036-1118
    """The bisector of the origin and (1,1,1) (plane n=(1,1,1) through
    (.5,.5,.5)) cuts only the corner (1,1,1) off the cube [-1,1]^3."""
    O = oracle_mod
    d = O.Diagram([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]], lo=[-1, -1, -1], hi=[1, 1, 1])
    c = d.cell(0)
    assert c.ids.tolist() == [-6, -5, -4, -3, -2, -1, 1]
    assert math.isclose(c.volume, 8.0 - 1.5 ** 3 / 6.0, rel_tol=1e-14)
    assert len(c.vertices) == 10
    # the new face is a triangle of side 1.5 * sqrt(2)
    f = c.ids.tolist().index(1)
    assert c.degrees[f] == 3
    assert math.isclose(c.areas[f], math.sqrt(3) / 4 * (1.5 * math.sqrt(2)) ** 2, rel_tol=1e-14)
    # no remaining vertex is Outside the plane
    n = np.ones(3) / math.sqrt(3)
    assert np.all(c.vertices @ n - math.sqrt(3) / 2 <= 1e-12)
