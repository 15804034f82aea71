"""The oracle's radius queries (celery.rs:682-855, celery.rs:1023-1075,
interface.rs:348-365) against the known answers of the reference's own tests
(celery.rs:1459-1900) and against brute-force restatements."""
import numpy as np
import pytest

import radius_cases as RC


def _split(offs, vals):
    return [vals[offs[t]:offs[t + 1]] for t in range(len(offs) - 1)]


def test_check_cell_in_range_kat(oracle_mod):            # celery.rs:1490-1662
    d = oracle_mod.Diagram(RC.celery4(1))
    assert d.grid().cpd == 4 and d.grid().sx == 1.0
    for q in (0.1, 0.9):
        for r in (0.5, 1.1, 1.7, 1.8):
            for i in range(4):
                for j in range(4):
                    for k in range(4):
                        got = d.check_cell_in_range([q, q, q], r, i, j, k)
                        assert got == RC.in_range_expected(q, r, i, j, k), (q, r, i, j, k)


def test_find_cells_in_radius_kat(oracle_mod):            # celery.rs:1665-1753
    d = oracle_mod.Diagram(RC.celery4(2))
    qs = [[q, q, q] for q, _ in RC.FIND_CELLS_CASES]
    for (q, r), p in zip(RC.FIND_CELLS_CASES, qs):
        offs, cells = d.find_cells_in_radius([p], r)
        got = set(cells.tolist())
        want = {RC.bin_id(i, j, k) for i in range(4) for j in range(4) for k in range(4)
                if RC.find_cells_expected(q, r, i, j, k)}
        assert got == want, (q, r)
        assert cells.tolist() == sorted(cells.tolist())   # i, j, k loop order


@pytest.mark.parametrize("real", [False, True])
def test_find_neighbors_kat(oracle_mod, real):            # celery.rs:1756-1900
    pts = RC.celery4_marked(-0.1 if real else -0.3, seed=3)
    d = oracle_mod.Diagram(pts)
    offs, ids = d.find_neighbors_in_radius([[0.5, 0.5, 0.5]], 1.73, real)
    want = RC.REAL_RADIUS_MARKED if real else RC.CELL_RADIUS_MARKED
    for idx, count in want.items():
        assert int(np.count_nonzero(ids == idx)) == count, idx


def test_neighbor_cloud_kat(oracle_mod):                  # celery.rs:1459-1487
    d = oracle_mod.Diagram(RC.celery4(4))
    _, ids = d.neighbor_cloud([[0.0, 0.0, 0.0]], 0.5)
    assert 77 in ids and 78 not in ids and len(ids) < 79
    _, ids = d.neighbor_cloud([[0.0, 0.0, 0.0]], 10.0)
    assert 77 in ids and 78 in ids and len(ids) == 79


def _queries(rng, n):
    q = rng.uniform(-0.1, 1.1, (n, 3))       # some outside the point bounds
    return q


@pytest.mark.parametrize("r", [0.0, 0.02, 0.05, 0.13])
def test_real_radius_is_the_ball(oracle_mod, r):
    rng = np.random.default_rng(11)
    pts = rng.uniform(0, 1, (3000, 3))
    d = oracle_mod.Diagram(pts)
    q = np.vstack([_queries(rng, 150), pts[:50]])
    offs, ids = d.find_neighbors_in_radius(q, r, True)
    offs_c, ids_c = d.find_neighbors_in_radius(q, r, False)
    for t, (got, cell) in enumerate(zip(_split(offs, ids), _split(offs_c, ids_c))):
        assert sorted(got.tolist()) == RC.brute_ball(pts, q[t], r).tolist()
        assert set(got.tolist()) <= set(cell.tolist())
        assert len(set(cell.tolist())) == len(cell)


def test_cell_radius_is_the_union_of_the_cells(oracle_mod):
    rng = np.random.default_rng(12)
    pts = rng.uniform(0, 1, (2000, 3))
    d = oracle_mod.Diagram(pts)
    bins = d.bins()
    q = _queries(rng, 100)
    for r in (0.03, 0.1):
        offs, ids = d.find_neighbors_in_radius(q, r, False)
        offs_b, cells = d.find_cells_in_radius(q, r)
        for got, cb in zip(_split(offs, ids), _split(offs_b, cells)):
            # bin order, then ascending index within a bin
            want = [i for b in cb.tolist() for i in np.nonzero(bins == b)[0].tolist()]
            assert got.tolist() == want


@pytest.mark.parametrize("r", [-2.0, -1.0, -0.5, 0.0, 0.004, 0.02, 0.3])
def test_neighbor_cloud_is_the_gap_key_walk(oracle_mod, r):
    rng = np.random.default_rng(13)
    pts = rng.uniform(0, 1, (1500, 3))
    groups = rng.integers(0, 3, 1500).astype(np.uint32)
    d = oracle_mod.Diagram(pts, groups=groups)
    g = d.grid()
    bins = d.bins().astype(np.int64)
    c = g.cpd
    bi, bj, bk = bins // (c * c), (bins // c) % c, bins % c
    for t in range(40):
        p = pts[t] if t % 2 else rng.uniform(0, 1, 3)
        qi = [oracle_mod.axis_index(p[a], lo, hi, inv, c) for a, lo, hi, inv in
              ((0, g.xmin, g.xmax, g.ix), (1, g.ymin, g.ymax, g.iy), (2, g.zmin, g.zmax, g.iz))]
        gaps = [np.maximum(np.abs(b - qi[a]) - 1, 0).astype(np.float64) for a, b in enumerate((bi, bj, bk))]
        a, b, cc = gaps[0] * g.sx, gaps[1] * g.sy, gaps[2] * g.sz
        key = a * a + b * b + cc * cc
        same = (bi == qi[0]) & (bj == qi[1]) & (bk == qi[2])
        key[same] = -1.0
        for grp in (-1, 1):
            _, ids = d.neighbor_cloud([p], r, grp)
            want = np.nonzero((key <= r) & ((groups == grp) if grp >= 0 else True))[0]
            assert sorted(ids.tolist()) == want.tolist()
            k = key[ids]
            assert np.all(np.diff(k) >= 0)            # search order: nondecreasing keys


def test_neighbor_cloud_nan_radius_walks_everything(oracle_mod):
    pts = np.random.default_rng(14).uniform(0, 1, (300, 3))
    d = oracle_mod.Diagram(pts)
    _, ids = d.neighbor_cloud([[0.5, 0.5, 0.5]], float("nan"))
    assert sorted(ids.tolist()) == list(range(300))
    _, cells = d.find_cells_in_radius([[0.5, 0.5, 0.5]], float("nan"))
    assert len(cells) == 0                              # ds <= NaN never holds
