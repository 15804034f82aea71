"""Inputs of the reference's radius-query unit tests (mcomstock/the-tessellator
src/celery.rs:1459-1900), restated with seeded points: a 79-point cloud in
[-2, 2]^3 whose extreme points (2, 2, 2) and (-2, -2, -2) make a 4 x 4 x 4 grid
of unit bins, and the expected bin and point memberships those tests assert.
Shared by the oracle tests and the GPU parity tests."""
import numpy as np

BIG, LITTLE = (2.0, 2.0, 2.0), (-2.0, -2.0, -2.0)


def celery4(seed=0):
    """77 random points, then the big point (index 77) and the little point (78)
    (celery.rs:1462-1470)."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-2.0, 2.0, (77, 3))
    return np.vstack([pts, [BIG, LITTLE]])


def celery4_marked(in_radius_low, seed=0):
    """71 random points, big (71), little (72), then the six marked points at
    indices 73..78 of find_neighbors_in_{cell,real}_radius_test
    (celery.rs:1756-1900)."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-2.0, 2.0, (71, 3))
    marked = [(0.1,) * 3, (in_radius_low,) * 3, (-0.7,) * 3, (-1.1,) * 3, (1.3,) * 3, (1.7,) * 3]
    return np.vstack([pts, [BIG, LITTLE], marked])


def bin_id(i, j, k):
    return 16 * i + 4 * j + k          # get_cell_from_indices at cpd = 4


def in_range_expected(q, r, i, j, k):
    """Memberships check_cell_in_range_test asserts (celery.rs:1490-1662);
    q is 0.1 or 0.9 on every axis."""
    if r == 0.5:
        return i != 0 and j != 0 and k != 0
    if r == 1.1:
        return (i == 0 and j >= 1 and k >= 1) or (i >= 1 and j == 0 and k >= 1) or \
            (i >= 1 and j >= 1 and k == 0) or (i >= 1 and j >= 1 and k >= 1)
    if r == 1.7:
        return i + j + k > 0
    if r == 1.8:
        return True
    raise ValueError(r)


def find_cells_expected(q, r, i, j, k):
    """Memberships find_cells_in_radius_test asserts (celery.rs:1665-1753)."""
    if q == 0.1:
        if r == 0.5:
            return i in (1, 2) and j in (1, 2) and k in (1, 2)
        if r == 1.2:
            return in_range_expected(q, 1.1, i, j, k)
        if r == 1.7:
            return i + j + k > 0
        if r == 1.8:
            return True
    if q == 0.9:
        if r == 0.5:
            return i in (2, 3) and j in (2, 3) and k in (2, 3)
        if r == 1.2:
            return i >= 1 and j >= 1 and k >= 1
        if r in (1.7, 1.8):
            return i != 0 and j != 0 and k != 0
    raise ValueError((q, r))


FIND_CELLS_CASES = [(q, r) for q in (0.1, 0.9) for r in (0.5, 1.2, 1.7, 1.8)]

# (index, expected count) for the marked points, query (0.5, 0.5, 0.5), radius 1.73
CELL_RADIUS_MARKED = {73: 1, 74: 1, 75: 1, 76: 0, 77: 1, 78: 1}   # celery.rs:1818-1827
REAL_RADIUS_MARKED = {73: 1, 74: 1, 75: 0, 76: 0, 77: 1, 78: 0}   # celery.rs:1892-1899


def brute_ball(pts, q, r):
    """Points within r of q, with distance_squared's own arithmetic
    (celery.rs:700-702) and the <= of celery.rs:849."""
    d2 = (q[0] - pts[:, 0]) * (q[0] - pts[:, 0]) + (q[1] - pts[:, 1]) * (q[1] - pts[:, 1]) \
        + (q[2] - pts[:, 2]) * (q[2] - pts[:, 2])
    return np.nonzero(d2 <= r * r)[0]
