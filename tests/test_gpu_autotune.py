"""The autotuner on the GPU: it times candidate launch knobs on a sample of
the cells, keeps the fastest, caches the choice by input class, and never
changes what is computed (results still meet the oracle's bars)."""
import os

import numpy as np
import pytest

from oracle import report

pytestmark = pytest.mark.gpu

WPB = {4, 8}
CROWD = {8, 12, 24, 48}
DENSITY = {0.6, 1.25, 2.5}


def results(d):
    vol = d.volumes()
    offs, nbr, area = d.neighbors_csr()
    return vol, offs.astype(np.int64), nbr, area


def check_against_oracle(oracle_mod, pts, res, prec, sample=None, lo=(0, 0, 0), hi=(1, 1, 1)):
    r = oracle_mod.Diagram(pts, lo=list(lo), hi=list(hi))
    idx = np.arange(len(pts)) if sample is None else sample
    v, o, i, a, _, _ = r.compute_all(subset=None if sample is None else sample.astype(np.uint32))
    c = report.compare_sample(res, idx, (v, o, i, a))
    assert c["identical_neighbour_lists_pct"] == 100.0, c
    assert c["max_rel_vol_err"] <= (1e-6 if prec == "fp32" else 1e-11), c


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_diagram_autotune_and_cache(tess, oracle_mod, tmp_path, prec):
    from tessellator import workloads

    pts = workloads.clustered(200_000, seed=3)
    cache = str(tmp_path / "tuning.txt")
    box = tess.Polyhedron(0, 0, 0, 1, 1, 1)
    with tess.Diagram(pts, container=box) as d:
        t = d.autotune(prec, cache_path=cache)
        assert t["trials"] == 8 and t["from_cache"] == 0
        assert t["warps_per_block"] in WPB and t["crowded_bin"] in CROWD
        assert t["bin_density"] == 1.25                      # the Celery grid stays the reference's
        assert 0 < t["ms_chosen"] <= t["ms_default"]
        assert t["sample_cells"] == 200_000 and t["max_bin_points"] >= 48 and t["crowded_fraction"] > 0.3
        with pytest.raises(tess.TessError) as e:             # tuning leaves no results behind
            d.volumes()
        assert e.value.status == tess._capi.TESS_E_STATE
        d.compute_all(prec)
        res = results(d)
        cells, _, _ = d.celery()
    sample = np.linspace(0, len(pts) - 1, 5000).astype(np.int64)
    check_against_oracle(oracle_mod, pts, res, prec, sample)
    assert os.path.exists(cache)
    # a second handle for the same kind of input reads the cache
    with tess.Diagram(pts, container=box) as d2:
        t2 = d2.autotune(prec, cache_path=cache)
        assert t2["from_cache"] == 1 and t2["trials"] == 0
        assert (t2["warps_per_block"], t2["crowded_bin"]) == (t["warps_per_block"], t["crowded_bin"])
        d2.compute_all(prec)
        np.testing.assert_allclose(d2.volumes(), res[0], rtol=1e-6 if prec == "fp32" else 1e-12)
        assert np.array_equal(d2.celery()[0], cells)


def test_autotune_flag_uses_the_default_cache(tess, oracle_mod, tmp_path, monkeypatch):
    from tessellator import workloads

    cache = tmp_path / "env_tuning.txt"
    monkeypatch.setenv("TESS_TUNE_CACHE", str(cache))
    pts = workloads.uniform(50_000, seed=9)
    cfg = tess.default_config(flags=tess.FLAG_AUTOTUNE)
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1), config=cfg) as d:
        d.compute_all("fp32")                                # tunes first, then computes
        res = results(d)
    assert cache.exists() and "diagram|prec1" in cache.read_text()
    check_against_oracle(oracle_mod, pts, res, "fp32", np.arange(0, len(pts), 10))


def test_batch_autotune(tess, oracle_mod, tmp_path):
    from tessellator import workloads

    pts, offs, boxes = workloads.batched(256, seed=4)
    b = tess.Batch(pts, offs, boxes)
    try:
        t = b.autotune("fp32", cache_path="")
        assert t["trials"] == 24 and t["from_cache"] == 0
        assert t["bin_density"] in DENSITY and t["warps_per_block"] in WPB and t["crowded_bin"] in CROWD
        assert 0 < t["ms_chosen"] <= t["ms_default"]
        b.compute("fp32")
        vol = b.volumes()
        go, gn, ga = b.neighbors_csr()
        go = go.astype(np.int64)
    finally:
        b.close()
    offs64 = offs.astype(np.int64)
    bvol = np.prod(boxes[:, 3:] - boxes[:, :3], axis=1)
    assert np.max(np.abs(np.add.reduceat(vol, offs64[:-1]) - bvol) / bvol) <= 1e-6
    for d in np.linspace(0, len(boxes) - 1, 8).astype(np.int64):
        a, e = int(offs64[d]), int(offs64[d + 1])
        sub = (vol[a:e], go[a:e + 1] - go[a], gn[go[a]:go[e]], ga[go[a]:go[e]])
        check_against_oracle(oracle_mod, pts[a:e], sub, "fp32", lo=boxes[d, :3], hi=boxes[d, 3:])
