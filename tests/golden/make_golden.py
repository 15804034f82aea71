"""Generates the committed golden fixtures of tests/golden/.

    qhull_uniform_2000.npz   2,000 uniform points (seed 2000) in [0,1]^3 and,
                             for every cell whose Qhull region is bounded and
                             inside the box, its Qhull volume (ConvexHull of
                             the Voronoi region) and its ridge neighbours.
                             Independent of this project's code.
    oracle_uniform_500.npz   500 uniform points (seed 500): the oracle's full
                             output (volumes, CSR of neighbour ids and areas),
                             pinning it against regressions.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def qhull_fixture():
    from scipy.spatial import ConvexHull, Voronoi

    pts = np.random.default_rng(2000).random((2000, 3))
    vor = Voronoi(pts)
    nb = {i: set() for i in range(len(pts))}
    for a, b in vor.ridge_points:
        nb[a].add(int(b))
        nb[b].add(int(a))
    cells, vols, offs, ids = [], [], [0], []
    for i in range(len(pts)):
        reg = vor.regions[vor.point_region[i]]
        if -1 in reg or not reg:
            continue
        V = vor.vertices[reg]
        if V.min() < 0 or V.max() > 1:
            continue
        cells.append(i)
        vols.append(ConvexHull(V).volume)
        s = sorted(nb[i])
        ids.extend(s)
        offs.append(len(ids))
    np.savez_compressed(os.path.join(HERE, "qhull_uniform_2000.npz"), points=pts, cells=np.array(cells),
                        volumes=np.array(vols), nbr_offsets=np.array(offs), nbr=np.array(ids))


def oracle_fixture():
    import oracle

    pts = np.random.default_rng(500).random((500, 3))
    d = oracle.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    vol, offs, ids, areas, _, _ = d.compute_all()
    np.savez_compressed(os.path.join(HERE, "oracle_uniform_500.npz"), points=pts, volumes=vol, offsets=offs,
                        ids=ids, areas=areas)


if __name__ == "__main__":
    qhull_fixture()
    oracle_fixture()
    print("fixtures written to", HERE)
