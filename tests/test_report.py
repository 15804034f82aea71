"""The parity checker (oracle/report.py) on the CPU: it finds planted
differences in neighbour lists, volumes and areas, counts asymmetric
neighbour relations, and applies the near-degenerate criterion (only faces
below a relative area bound may differ).  The mistakes are planted in copies
of the oracle's own results."""
import numpy as np
import pytest

from oracle import report


@pytest.fixture(scope="module")
def full(oracle_mod):
    pts = np.random.default_rng(3).random((3000, 3))
    r = oracle_mod.Diagram(pts, lo=[0, 0, 0], hi=[1, 1, 1])
    v, o, i, a, _, _ = r.compute_all()
    return pts, (v, o, i, a)


def test_identical_results_pass(full):
    _, res = full
    v, o, i, a = res
    sample = np.arange(0, len(v), 7)
    new_o, ids = report._gather_rows(o, i, sample)
    _, areas = report._gather_rows(o, a, sample)
    c = report.compare_sample((v, o, i.astype(np.int32), a), sample, (v[sample], new_o, ids, areas))
    assert c["identical_neighbour_lists_pct"] == 100.0
    assert c["max_rel_vol_err"] == 0.0 and c["max_area_err_rel_largest_face"] == 0.0
    d = report.diagram_checks(v, o, i, 1.0)
    assert d["symmetry_violations"] == 0 and abs(d["vol_sum_minus_box"]) < 1e-12


def test_planted_differences_are_found(full):
    _, (v, o, i, a) = full
    g_v, g_i, g_a = v.copy(), i.copy(), a.copy()
    cell = 1234
    g_i[o[cell]] = 2999 if g_i[o[cell]] != 2999 else 2998    # one wrong neighbour
    g_v[77] *= 1 + 3e-6                                        # one volume off by 3e-6
    g_a[o[500] + 1] *= 1.01                                    # one face area off by 1%
    sample = np.arange(len(v))
    c = report.compare_sample((g_v, o, g_i.astype(np.int32), g_a), sample, (v, o, i, a))
    assert c["mismatched_cells"] == [cell] and c["mismatched_count"] == 1
    assert 2.9e-6 < c["max_rel_vol_err"] < 3.1e-6
    assert c["max_area_err_rel_largest_face"] > 1e-3
    # a dropped face count shows up too
    g_o = o.copy()
    g_o[cell + 1:] -= 1
    g_i2 = np.delete(i, o[cell])
    g_a2 = np.delete(a, o[cell])
    c = report.compare_sample((v, g_o, g_i2.astype(np.int32), g_a2), sample, (v, o, i, a))
    assert c["mismatched_count"] == 1
    # asymmetric relations: the dropped entry leaves its partner unmatched
    assert report.symmetry_violations(g_o, g_i2, len(v)) == 1
    # unless that partner's face is below the area bound of the criterion
    j = int(i[o[cell]])
    k = o[j] + int(np.nonzero(i[o[j]:o[j + 1]] == cell)[0][0])
    k2 = k - 1 if k > o[cell] else k                  # its position after the deletion
    g_a3 = g_a2.copy()
    g_a3[k2] = 1e-16
    assert report.symmetry_violations(g_o, g_i2, len(v), areas=g_a3, rel_area=1e-9) == 0
    assert report.symmetry_violations(g_o, g_i2, len(v), areas=g_a2, rel_area=1e-9) == 1


def test_near_degenerate_criterion():
    ids_g, area_g = np.array([-1, 3, 5, 9]), np.array([0.5, 0.2, 1e-15, 0.3])
    ids_r, area_r = np.array([-1, 3, 9]), np.array([0.5, 0.2, 0.3])
    ok, worst = report.near_degenerate_ok((ids_g, area_g), (ids_r, area_r), rel_area=1e-9)
    assert ok and worst == pytest.approx(2e-15)
    area_g[2] = 1e-6                                         # a real face missing on one side
    ok, worst = report.near_degenerate_ok((ids_g, area_g), (ids_r, area_r), rel_area=1e-9)
    assert not ok
