"""Parity report: GPU results against the oracle's, and whole-diagram invariants.

TEST INFRASTRUCTURE ONLY (the checker).  Used by ``tests/`` and by the
CPU-baseline leg of ``bench.py``; the library never imports it.

The report follows the per-run list of the measurement plan: maximum and mean
relative volume error against the FP64 oracle, the share of identical
neighbour lists, the largest face-area error relative to the cell's largest
face, the volume sum against the box volume, and the number of asymmetric
neighbour relations (j in N(i) but i not in N(j)).  Volumes follow
compute_volume (polyhedron.rs:838-855), neighbour ids the cutting particle's
original index (interface.rs:329), areas compute_area (interface.rs:408-410).
"""
from __future__ import annotations

import numpy as np


def _gather_rows(offs, vals, rows):
    """Concatenated CSR rows `rows` of (offs, vals), with their new offsets."""
    offs = np.asarray(offs, dtype=np.int64)
    rows = np.asarray(rows, dtype=np.int64)
    starts = offs[rows]
    counts = offs[rows + 1] - starts
    new = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum(counts, out=new[1:])
    idx = np.repeat(starts - new[:-1], counts) + np.arange(int(new[-1]), dtype=np.int64)
    return new, np.asarray(vals)[idx]


def compare_sample(gpu, sample, ref, all_mismatched=False):
    """Compare the GPU's results for the cells `sample` with the oracle's.

    gpu    = (volumes[n], offsets[n+1], neighbours, areas) of the whole diagram;
    sample = cell indices (original order) the oracle computed;
    ref    = (volumes, offsets, ids, areas) of the oracle for those cells.
    Returns a dict; 'mismatched_cells' lists up to 10 cells whose neighbour
    lists differ ('mismatched_all', with all_mismatched, every one of them)."""
    gv, go, gn, ga = gpu
    rv, ro, ri, ra = ref
    sample = np.asarray(sample, dtype=np.int64)
    ro = np.asarray(ro, dtype=np.int64)
    v = np.asarray(gv)[sample]
    rel = np.abs(v - rv) / np.maximum(np.abs(rv), 1e-300)
    so, sn = _gather_rows(go, gn, sample)
    _, sa = _gather_rows(go, ga, sample)
    gcount = np.diff(so)
    rcount = np.diff(ro)
    same_count = gcount == rcount
    # element-wise comparison inside the rows whose face counts agree
    ident = same_count.copy()
    area_err = 0.0
    if same_count.any():
        rows = np.nonzero(same_count)[0]
        go2, gn2 = _gather_rows(so, sn, rows)
        _, ga2 = _gather_rows(so, sa, rows)
        _, rn2 = _gather_rows(ro, ri, rows)
        _, ra2 = _gather_rows(ro, ra, rows)
        diff = gn2.astype(np.int64) != rn2.astype(np.int64)
        cnt = np.diff(go2)
        nz = cnt > 0
        if diff.size:
            bad_rows = np.zeros(len(rows), dtype=bool)
            bad_rows[nz] = np.add.reduceat(diff, go2[:-1][nz]) > 0
            ident[rows[bad_rows]] = False
            big = np.zeros(len(rows))
            big[nz] = np.maximum.reduceat(ra2, go2[:-1][nz])
            scale = np.repeat(big, cnt)
            ok = ~np.repeat(bad_rows, cnt)
            if ok.any():
                area_err = float(np.max(np.abs(ga2[ok] - ra2[ok]) / np.maximum(scale[ok], 1e-300)))
    bad = sample[~ident]
    extra = {"mismatched_all": bad} if all_mismatched else {}
    return {**extra,
        "cells": int(len(sample)),
        "max_rel_vol_err": float(rel.max()) if len(rel) else 0.0,
        "mean_rel_vol_err": float(rel.mean()) if len(rel) else 0.0,
        "identical_neighbour_lists_pct": 100.0 * float(ident.mean()) if len(ident) else 100.0,
        "max_area_err_rel_largest_face": area_err,
        "mismatched_cells": [int(x) for x in bad[:10]],
        "mismatched_count": int(len(bad)),
    }


def symmetry_violations(offs, nbr, n, device=None, areas=None, rel_area=None):
    """Number of (i, j) with j in N(i), j >= 0, and i not in N(j).  With
    `areas` and `rel_area`, only faces of at least rel_area of their cell's
    largest face count (near-degenerate inputs).  Runs on a CUDA device
    through torch when one is given (large diagrams), else numpy."""
    offs = np.asarray(offs, dtype=np.int64)
    counts = np.diff(offs)
    if device is not None:
        import torch

        o = torch.from_numpy(counts).to(device)
        rows = torch.repeat_interleave(torch.arange(n, device=device, dtype=torch.int64), o)
        cols = torch.from_numpy(np.ascontiguousarray(nbr)).to(device).to(torch.int64)
        keep = cols >= 0
        if areas is not None and rel_area is not None:
            ar = torch.from_numpy(np.ascontiguousarray(areas)).to(device)
            big = torch.zeros(n, dtype=ar.dtype, device=device).scatter_reduce_(0, rows, ar, "amax")
            keep &= ar >= rel_area * big[rows]
        rows_k, cols_k = rows[keep], cols[keep]
        key, _ = torch.sort(rows[cols >= 0] * n + cols[cols >= 0])
        rkey = cols_k * n + rows_k
        pos = torch.searchsorted(key, rkey).clamp_(max=max(int(key.numel()) - 1, 0))
        found = key[pos] == rkey if key.numel() else torch.zeros_like(rkey, dtype=torch.bool)
        res = int((~found).sum().item())
        del o, rows, cols, key, rkey, pos, found
        return res
    rows = np.repeat(np.arange(n, dtype=np.int64), counts)
    cols = np.asarray(nbr, dtype=np.int64)
    keep = cols >= 0
    if areas is not None and rel_area is not None:
        ar = np.asarray(areas)
        big = np.zeros(n)
        np.maximum.at(big, rows, ar)
        keep &= ar >= rel_area * big[rows]
    key = np.sort(rows[cols >= 0] * n + cols[cols >= 0])
    rkey = cols[keep] * n + rows[keep]
    if key.size == 0:
        return int(rkey.size)
    pos = np.minimum(np.searchsorted(key, rkey), key.size - 1)
    return int(np.count_nonzero(key[pos] != rkey))


SLIVER_AREA = 1e-9


def diagram_checks(vol, offs, nbr, box_volume, device=None, areas=None, rel_area=None):
    """Whole-diagram invariants: the volume sum against the box and the
    neighbour symmetry, counted strictly and, when areas are given, once more
    with faces below rel_area (default SLIVER_AREA) of their cell's largest
    face exempt: among tens of millions of random cells a few near-degenerate
    vertex clusters leave slivers whose presence FP64 rounding decides, on
    each side independently."""
    vol = np.asarray(vol)
    s = float(np.sum(vol, dtype=np.float64))
    out = {
        "vol_sum_minus_box": s - box_volume,
        "vol_sum_rel_err": abs(s - box_volume) / box_volume,
        "symmetry_violations": symmetry_violations(offs, nbr, len(vol), device),
        "faces": int(len(nbr)),
    }
    if areas is not None:
        ra = SLIVER_AREA if rel_area is None else rel_area
        out["symmetry_violations_above_sliver"] = symmetry_violations(offs, nbr, len(vol), device, areas, ra)
        out["sliver_area_rel"] = ra
    return out


def near_degenerate_ok(gpu_row, ref_row, rel_area=1e-9):
    """Criterion for near-degenerate inputs (jittered lattices, near-coincident
    pairs): the neighbour lists may differ only in faces whose area is below
    rel_area of the cell's largest face, on either side.  Each row is
    (ids, areas) of one cell.  Returns (ok, largest relative area of a
    differing face)."""
    gi, ga = np.asarray(gpu_row[0], dtype=np.int64), np.asarray(gpu_row[1])
    ri, ra = np.asarray(ref_row[0], dtype=np.int64), np.asarray(ref_row[1])
    scale = max(float(ga.max()) if ga.size else 0.0, float(ra.max()) if ra.size else 0.0, 1e-300)
    only_g = ~np.isin(gi, ri)
    only_r = ~np.isin(ri, gi)
    worst = 0.0
    if only_g.any():
        worst = max(worst, float(ga[only_g].max()) / scale)
    if only_r.any():
        worst = max(worst, float(ra[only_r].max()) / scale)
    return worst <= rel_area, worst


def near_degenerate_report(gpu, ref, cells, rel_area=1e-9):
    """Apply near_degenerate_ok to the given cells of two whole-diagram
    results (volumes, offsets, ids, areas), typically the cells whose lists
    differ.  Returns (cells that differ only in tiny faces, cells that violate
    the criterion (up to 10), the largest relative area of a differing face)."""
    _, go, gn, ga = gpu
    _, ro, ri, ra = ref
    go = np.asarray(go, dtype=np.int64)
    ro = np.asarray(ro, dtype=np.int64)
    tiny = 0
    bad = []
    worst = 0.0
    for i in cells:
        i = int(i)
        g = (gn[go[i]:go[i + 1]], ga[go[i]:go[i + 1]])
        r = (ri[ro[i]:ro[i + 1]], ra[ro[i]:ro[i + 1]])
        ok, w = near_degenerate_ok(g, r, rel_area)
        worst = max(worst, w)
        if ok:
            tiny += 1
        elif len(bad) < 10:
            bad.append(i)
    return tiny, bad, worst
