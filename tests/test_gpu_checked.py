"""The bounds-checked build (libtessgpu_checked.so, TESS_CHECKED=1) on the GPU.

Its binning and clipping kernels test every data-dependent device index
(points, bins, vertex slots and the free-slot stack, plane sources, re-run
list entries, face-pool positions) before use; an index out of range is
recorded and replaced by an in-range one, and the call fails with
TESS_E_CHECK.  This test runs the parity workloads that reach every clipping
path through the checked library, in a child process (the package loads one
library per process), and requires every call to succeed with results equal
to the oracle's: no index of any path leaves its array.

Paths covered: the lean first pass, the crowded-bin (seeded) pass, the hybrid
and FP64 re-runs, the capacity re-runs at 128 and 255 slots, the FP64 and
MIXED forms, the batch graph, single-cell geometry, and a face pool that
must grow.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cases():
    """(name, points in the unit box, precisions, config flags)."""
    from tessellator import workloads

    rng = np.random.default_rng(21)
    cases = [("uniform", workloads.uniform(20_000, seed=5), ("fp32", "fp64", "mixed"), 0),
             ("clustered", workloads.clustered(20_000, seed=3), ("fp32", "fp64"), 0)]
    # points on walls and corners, coincident and near-coincident pairs
    pts = rng.random((3000, 3))
    pts[:8] = [[0, 0, 0], [1, 1, 1], [0, 1, 0], [1, 0, 1], [0.5, 0, 0.5], [0, 0.5, 1], [1, 0.5, 0.5], [0.5, 1, 0]]
    pts[100] = pts[101]
    pts[200] = pts[201] + 1e-9
    pts[300] = pts[301] + 3e-7
    cases.append(("edges_and_duplicates", pts, ("fp32", "fp64"), 0))
    # a cell that overflows 64 and 128 slots and fits 255 (the capacity
    # re-run test's cell: a site inside 150 points on a sphere)
    rb = np.random.default_rng(14)
    u = rb.standard_normal((150, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    big = np.concatenate([[[0.5, 0.5, 0.5]], 0.5 + 0.1 * u, rb.random((200, 3))])
    cases.append(("big_cell", big, ("fp32", "fp64", "mixed"), 0))
    # a face pool that starts too small and must grow
    cases.append(("small_face_pool", workloads.uniform(5000, seed=6), ("fp32",), 4))
    return cases


def _child():
    """Runs in the child process: every case through the checked library."""
    sys.path.insert(0, os.path.join(ROOT, "the-tessellator_gb300"))
    sys.path.insert(0, ROOT)
    import oracle
    import tessellator as T
    from oracle import report

    assert T._capi.LIB_PATH == os.environ["TESS_LIB"]

    box = T.Polyhedron(0, 0, 0, 1, 1, 1)
    for name, pts, precs, flags in _cases():
        ref = oracle.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
        rv, ro, ri, ra, _, _ = ref.compute_all()
        for prec in precs:
            cfg = T.default_config(flags=flags)
            with T.Diagram(pts, container=box, config=cfg) as d:
                d.compute_all(prec)
                vol = d.volumes()
                offs, nbr, area = d.neighbors_csr()
                st = d.stats()
                if name == "uniform" and prec == "fp64":
                    # single-cell geometry (the 255-slot geometry form)
                    cell = d.get_cell_at_index(17).compute_voronoi_cell()
                    assert abs(cell.compute_volume() - rv[17]) <= 1e-12 * rv[17]
            c = report.compare_sample((vol, offs.astype(np.int64), nbr, area), np.arange(len(pts)), (rv, ro, ri, ra))
            tol = 1e-6 if prec == "fp32" else 1e-11
            if name == "edges_and_duplicates":
                # coincident points: their cells overlap, compare per cell only
                assert c["max_rel_vol_err"] <= max(tol, 1e-9), (name, prec, c)
            else:
                assert c["identical_neighbour_lists_pct"] == 100.0, (name, prec, c)
                assert c["max_rel_vol_err"] <= tol, (name, prec, c)
            print(f"checked {name} {prec}: {len(pts)} cells, max rel vol err {c['max_rel_vol_err']:.1e}, "
                  f"capacity re-runs {st['rerun_capacity']}, pool regrows {st['face_pool_regrows']}", flush=True)
    # a batch (one CUDA graph) through the checked library
    from tessellator import workloads

    sizes = [64, 500, 3000, 120, 2048, 999]
    offs_b = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    bpts = np.concatenate([workloads.uniform(s, seed=40 + k) for k, s in enumerate(sizes)])
    boxes = np.array([[0, 0, 0, 1, 1, 1]] * len(sizes), dtype=np.float64)
    b = T.Batch(bpts, offs_b, boxes)
    try:
        b.compute("fp32")
        vol = b.volumes()
    finally:
        b.close()
    for k, s in enumerate(sizes):
        ref = oracle.Diagram(bpts[offs_b[k]:offs_b[k + 1]], lo=[0, 0, 0], hi=[1, 1, 1])
        rv = ref.compute_all()[0]
        err = np.max(np.abs(vol[offs_b[k]:offs_b[k + 1]] - rv) / rv)
        assert err <= 1e-6, (k, err)
    print("checked batch: ok", flush=True)


def test_checked_build_stays_in_bounds():
    import build_lib

    lib = build_lib.build(checked=True)
    env = dict(os.environ, TESS_LIB=lib, TESS_CHECKED_CHILD="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__)], env=env, capture_output=True, text=True,
                       timeout=900)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "checked batch: ok" in r.stdout


if __name__ == "__main__" and os.environ.get("TESS_CHECKED_CHILD"):
    _child()
