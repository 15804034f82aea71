"""The MIXED precision's finish, checked on the CPU: the kernel computes a
face's area from its projection on the coordinate plane across the dominant
axis m of the face normal q (shoelace), A = w_m |q| / (2 q_m), and the cell's
volume as the sum of pyramids from the site, qh w_m / (6 q_m), with the face
plane q.x = qh (a bisector of the site and point j: q = p_j - site,
qh = q.q / 2; a wall: q = +-e_a, qh = its distance).  Applied in numpy to the
oracle's own FP64 cells, these formulas must give the oracle's areas and
volumes (compute_volume, polyhedron.rs:838-855; compute_area,
interface.rs:408-410)."""
import numpy as np
import pytest


def face_plane(pts, site, nbr, lo, hi):
    if nbr >= 0:
        q = pts[nbr] - site
        return q, 0.5 * q.dot(q)
    w = -1 - nbr                       # -1 x_min, -2 x_max, -3 y_min, ...
    a, mx = w // 2, w % 2
    q = np.zeros(3)
    q[a] = 1.0 if mx else -1.0
    return q, (hi[a] - site[a]) if mx else (site[a] - lo[a])


def shoelace(cycle, q):
    """w_m over the face's vertex cycle, anchor-relative, for the dominant
    axis m of q, with (X1, X2) the other two axes in cyclic order."""
    m = int(np.argmax(np.abs(q)))
    a1, a2 = (m + 1) % 3, (m + 2) % 3
    rel = cycle - cycle[0]
    u, v = rel[:-1], rel[1:]
    return m, float((u[:, a1] * v[:, a2] - u[:, a2] * v[:, a1]).sum())


@pytest.mark.parametrize("seed,n", [(1, 300), (2, 2000)])
def test_shoelace_areas_and_pyramid_volumes(oracle_mod, seed, n):
    rng = np.random.default_rng(seed)
    lo, hi = np.array([0.0, -1.0, 2.0]), np.array([1.0, 0.5, 3.0])
    pts = lo + (hi - lo) * rng.random((n, 3))
    d = oracle_mod.Diagram(pts, lo=lo, hi=hi)
    for i in range(0, n, max(1, n // 60)):
        c = d.cell(i)
        vol = 0.0
        for f, nbr in enumerate(c.ids):
            cyc = np.asarray(c.face_vertices[f])          # the face's vertex cycle (site-relative)
            q, qh = face_plane(pts, pts[i], int(nbr), lo, hi)
            m, wm = shoelace(cyc, q)
            # the cycle runs counter-clockwise seen from outside: w is outward
            area = wm * np.linalg.norm(q) / (2.0 * q[m])
            assert area > 0
            assert abs(area - c.areas[f]) <= 1e-12 * max(c.areas.max(), 1e-300)
            vol += qh * wm / (6.0 * q[m])
        assert abs(vol - c.volume) <= 1e-12 * c.volume
