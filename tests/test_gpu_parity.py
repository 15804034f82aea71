"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle on the
same seeded inputs.  Bars: neighbour lists bit-exact; volumes within 1e-12
relative (FP64 form, and the FP32 clipping with the FP64 finish, "mixed") or
1e-6 (FP32 + FP64-guard form); face areas within 1e-9 (FP64, mixed) or 1e-5
(FP32) of the cell's largest face; bin grid bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VOL_TOL = {"fp64": 1e-12, "mixed": 1e-12, "fp32": 1e-6}
AREA_TOL = {"fp64": 1e-9, "mixed": 1e-9, "fp32": 1e-5}


def unit_box(T):
    return T.Polyhedron(0, 0, 0, 1, 1, 1)


def compare(prec, gpu, ref, n, check_sum=None):
    vol, offs, nbr, area = gpu
    rv, ro, ri, ra = ref
    rel = np.abs(vol - rv) / np.maximum(np.abs(rv), 1e-300)
    assert rel.max() <= VOL_TOL[prec], f"max rel volume error {rel.max():.3e} at {int(rel.argmax())}"
    assert np.array_equal(offs.astype(np.int64), ro), "face counts differ"
    assert np.array_equal(nbr.astype(np.int64), ri), "neighbour lists differ"
    # areas, relative to the largest face of each cell
    counts = np.diff(ro)
    cellmax = np.maximum.reduceat(ra, ro[:-1][counts > 0]) if len(ra) else np.zeros(0)
    scale = np.repeat(cellmax, counts[counts > 0])
    assert np.all(np.abs(area - ra) <= AREA_TOL[prec] * scale)
    if check_sum is not None:
        assert abs(vol.sum() - check_sum) <= (1e-6 if prec == "fp32" else 1e-11) * check_sum


def assert_only_tiny_faces_differ(gpu, ref, rel_area=1e-9):
    """Near-degenerate inputs: the neighbour lists may differ only in faces
    below rel_area of the cell's largest face (their presence depends on the
    cut order); every other neighbour is identical."""
    from oracle import report

    c = report.compare_sample(gpu, np.arange(len(gpu[0])), ref, all_mismatched=True)
    tiny, bad, worst = report.near_degenerate_report(gpu, ref, c["mismatched_all"], rel_area)
    assert not bad, f"cells {bad} differ in faces up to {worst:.2e} of their largest face"
    assert tiny == c["mismatched_count"]


def canonical_lists(offs, nbr, rep):
    """Each cell's neighbour set with ids mapped through rep (walls kept)."""
    offs = np.asarray(offs, dtype=np.int64)
    out = []
    for i in range(len(offs) - 1):
        ids = np.asarray(nbr[offs[i]:offs[i + 1]], dtype=np.int64)
        out.append(sorted(set(np.where(ids >= 0, rep[np.maximum(ids, 0)], ids).tolist())))
    return out


def gpu_all(T, pts, prec, container=None, config=None, **kw):
    with T.Diagram(pts, container=container, config=config) as d:
        d.compute_all(prec, **kw)
        vol = d.volumes()
        offs, nbr, area = d.neighbors_csr()
        st = d.stats()
    return (vol, offs, nbr, area), st


def ref_all(O, pts, lo=None, hi=None, **kw):
    r = O.Diagram(pts, lo=lo, hi=hi)
    v, o, i, a, _, _ = r.compute_all(**kw)
    return v, o, i, a


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_uniform_10k(tess, oracle_mod, prec):
    from tessellator import workloads

    pts = workloads.uniform(10000, seed=0)
    gpu, st = gpu_all(tess, pts, prec, container=unit_box(tess))
    ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
    compare(prec, gpu, ref, len(pts), check_sum=1.0)
    assert st["failed"] == 0


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_symmetric_neighbours(tess, prec):
    from tessellator import workloads

    pts = workloads.uniform(5000, seed=11)
    (vol, offs, nbr, _), _ = gpu_all(tess, pts, prec, container=unit_box(tess))
    offs = offs.astype(np.int64)
    sets = [set(nbr[offs[i]:offs[i + 1]].tolist()) for i in range(len(pts))]
    bad = sum(1 for i, s in enumerate(sets) for j in s if j >= 0 and i not in sets[j])
    assert bad == 0


@pytest.mark.parametrize("n,lo,hi", [(1000, 0.0, 1.0), (1000, -1000.0, 500.0), (3, 0.0, 1.0),
                                     (1, 0.0, 1.0), (79, -2.0, 2.0), (20000, 0.0, 1.0)])
def test_celery_bit_exact(tess, oracle_mod, n, lo, hi):
    """Bin of every point, sorted order and delimiters equal the oracle's
    restatement of celery.rs:269-414."""
    rng = np.random.default_rng(n)
    pts = lo + (hi - lo) * rng.random((n, 3))
    if n == 79:   # the reference's expand_all_in_radius fixture (celery.rs:1459-1466)
        pts[-2] = [2.0, 2.0, 2.0]
        pts[-1] = [-2.0, -2.0, -2.0]
    with tess.Diagram(pts) as d:
        cells, srt, dl = d.celery()
        cpd, bounds = d.grid()
    r = oracle_mod.Diagram(pts)
    g = r.grid()
    assert cpd == g.cpd
    assert np.array_equal(bounds, [g.xmin, g.xmax, g.ymin, g.ymax, g.zmin, g.zmax])
    assert np.array_equal(cells, r.bins())
    assert np.array_equal(srt, r.sorted_indices())
    assert np.array_equal(dl, r.delimiters())


def test_celery_crowded_bins(tess, oracle_mod):
    """Bins of hundreds and of ~5,000 points (sorted by the whole block, in
    shared and in global memory): the same sorted order as the oracle's."""
    rng = np.random.default_rng(21)
    pts = np.vstack([0.5 + 1e-3 * rng.random((5000, 3)), 0.2 + 0.05 * rng.random((2000, 3)),
                     rng.random((1000, 3))])
    pts = pts[rng.permutation(len(pts))]
    with tess.Diagram(pts) as d:
        cells, srt, dl = d.celery()
    r = oracle_mod.Diagram(pts)
    counts = np.diff(r.delimiters())
    assert counts.max() > 4096 and ((counts > 32) & (counts <= 4096)).any()
    assert np.array_equal(cells, r.bins())
    assert np.array_equal(srt, r.sorted_indices())
    assert np.array_equal(dl, r.delimiters())


def test_oblong_and_offset_boxes(tess, oracle_mod):
    rng = np.random.default_rng(7)
    lo, hi = np.array([-5.0, 12.0, -10000.0]), np.array([-4.0, 1000.0, 1.0])
    pts = lo + (hi - lo) * rng.random((3000, 3))
    for prec in ("fp64", "fp32", "mixed"):
        gpu, _ = gpu_all(tess, pts, prec, container=tess.Polyhedron(*lo, *hi))
        ref = ref_all(oracle_mod, pts, lo, hi)
        compare(prec, gpu, ref, len(pts), check_sum=float(np.prod(hi - lo)))


def test_default_bounding_box(tess, oracle_mod):
    """No container: the Diagram bounding box, grown from the origin."""
    rng = np.random.default_rng(8)
    pts = 2.0 + rng.random((800, 3))   # the box becomes [0, max]^3, max < 3
    gpu, _ = gpu_all(tess, pts, "fp64")
    ref = ref_all(oracle_mod, pts)
    compare("fp64", gpu, ref, len(pts), check_sum=float(np.prod(pts.max(axis=0))))


@pytest.mark.parametrize("n", [1, 2, 5])
def test_tiny(tess, oracle_mod, n):
    rng = np.random.default_rng(100 + n)
    pts = rng.random((n, 3))
    for prec in ("fp64", "fp32", "mixed"):
        gpu, _ = gpu_all(tess, pts, prec, container=unit_box(tess))
        ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
        compare(prec, gpu, ref, n, check_sum=1.0)


def test_points_on_walls_and_corners(tess, oracle_mod):
    rng = np.random.default_rng(9)
    pts = rng.random((500, 3))
    pts[:8] = [[0, 0, 0], [1, 1, 1], [0, 1, 0], [1, 0, 1], [0.5, 0, 0.5], [0.5, 1, 0.25], [0, 0.3, 0.7],
               [1, 0.6, 0.2]]
    gpu, _ = gpu_all(tess, pts, "fp64", container=unit_box(tess))
    ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
    compare("fp64", gpu, ref, len(pts), check_sum=1.0)


def test_duplicate_points(tess, oracle_mod):
    """Coincident points cut nothing (the reference's bisector of a zero
    vector is NaN and classifies every vertex Incident)."""
    rng = np.random.default_rng(10)
    pts = rng.random((400, 3))
    pts[1] = pts[0]
    pts[2] = pts[0]
    gpu, _ = gpu_all(tess, pts, "fp64", container=unit_box(tess))
    ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
    compare("fp64", gpu, ref, len(pts))


@pytest.mark.parametrize("radius", [0.0, 0.001, 0.004, 0.02])
def test_search_radius(tess, oracle_mod, radius):
    """Some(radius): bins with squared gap distance <= radius only
    (expand_all_in_radius, celery.rs:1023-1036)."""
    from tessellator import workloads

    pts = workloads.uniform(3000, seed=12)
    gpu, _ = gpu_all(tess, pts, "fp64", container=unit_box(tess), search_radius=radius)
    ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1], mode=oracle_mod.MODE_RADIUS, radius=radius)
    compare("fp64", gpu, ref, len(pts))


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_target_group(tess, oracle_mod, prec):
    from tessellator import workloads

    pts = workloads.uniform(3000, seed=13)
    groups = (np.arange(3000) % 3).astype(np.uint32)
    with tess.Diagram(pts, groups=groups, container=unit_box(tess)) as d:
        d.compute_all(prec, target_group=1)
        vol = d.volumes()
        offs, nbr, area = d.neighbors_csr()
    r = oracle_mod.Diagram(pts, groups=groups, lo=[0, 0, 0], hi=[1, 1, 1])
    v, o, i, a, _, _ = r.compute_all(target_group=1)
    compare(prec, (vol, offs, nbr, area), (v, o, i, a), len(pts))


def test_capacity_reruns(tess, oracle_mod):
    """A site surrounded by 150 points on a sphere has ~300 vertices: the
    64- and 128-slot passes overflow and the 255-slot pass finishes it."""
    rng = np.random.default_rng(14)
    m = 150
    u = rng.standard_normal((m, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = np.concatenate([[[0.5, 0.5, 0.5]], 0.5 + 0.1 * u, rng.random((200, 3))])
    for prec in ("fp64", "fp32", "mixed"):
        gpu, st = gpu_all(tess, pts, prec, container=unit_box(tess))
        ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
        compare(prec, gpu, ref, len(pts), check_sum=1.0)
        assert st["rerun_capacity"] >= 1


def test_fp32_guard_reruns_on_lattice(tess, oracle_mod):
    """A jittered cubic lattice puts many plane tests inside the guard band:
    those cells re-run with the guard-band tests decided in FP64 and agree
    with the oracle (FP32-form volumes, 1e-6 per cell)."""
    from tessellator import workloads

    pts = workloads.lattice_sc(12, seed=5)
    gpu, st = gpu_all(tess, pts, "fp32", container=unit_box(tess))
    assert st["rerun_fp64"] > 0
    vol, offs, nbr, area = gpu
    rv, ro, ri, ra = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
    assert np.max(np.abs(vol - rv) / rv) <= 1e-6
    assert abs(vol.sum() - 1.0) < 1e-6
    # 1e-7 jitter leaves faces of area ~1e-14 whose presence depends on the
    # cut order (the FP64 form differs from the oracle the same way): the
    # lists may differ only in faces below 1e-9 of the cell's largest face
    assert_only_tiny_faces_differ((vol, offs.astype(np.int64), nbr, area), (rv, ro, ri, ra))


def test_hybrid_rerun_on_bcc_lattice(tess, oracle_mod):
    """Every cell of a 1e-7-jittered BCC lattice lands in the guard band: the
    hybrid re-run decides those plane tests in FP64 and the cells keep their
    FP32-form accuracy; the few it cannot settle run in FP64."""
    from tessellator import workloads

    pts = workloads.lattice_bcc(10, seed=6)
    gpu, st = gpu_all(tess, pts, "fp32", container=unit_box(tess))
    assert st["rerun_fp64"] == len(pts)
    assert 0 <= st["rerun_fp64_full"] < st["rerun_fp64"]
    assert st["failed"] == 0
    vol, offs, nbr, area = gpu
    rv, ro, ri, ra = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
    assert np.max(np.abs(vol - rv) / rv) <= 1e-6
    assert abs(vol.sum() - 1.0) < 1e-6
    assert_only_tiny_faces_differ((vol, offs.astype(np.int64), nbr, area), (rv, ro, ri, ra))


def test_clustered_small(tess, oracle_mod):
    """Crowded bins: the FP32 first pass hands their cells to the seeded pass."""
    from tessellator import workloads

    pts = workloads.clustered(20000, seed=3)
    for prec in ("fp64", "fp32", "mixed"):
        gpu, st = gpu_all(tess, pts, prec, container=unit_box(tess))
        ref = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
        compare(prec, gpu, ref, len(pts), check_sum=1.0)
        if prec != "fp64":
            assert st["dense_cells"] > 1000


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_far_from_the_origin(tess, oracle_mod, prec):
    """Coordinates near 1e6 in a unit box: the FP32 positions are split
    relative to the diagram's centre, so the FP32 form keeps its accuracy."""
    rng = np.random.default_rng(15)
    lo = np.array([1.0e6, -2.0e6, 3.0e5])
    pts = lo + rng.random((4000, 3))
    gpu, st = gpu_all(tess, pts, prec, container=tess.Polyhedron(*lo, *(lo + 1)))
    ref = ref_all(oracle_mod, pts, lo, lo + 1)
    compare(prec, gpu, ref, len(pts), check_sum=1.0)
    if prec != "fp64":
        assert st["rerun_fp64"] < 0.05 * len(pts)


def test_near_duplicates_fp32(tess, oracle_mod):
    """Pairs 1e-12 .. 1e-5 apart and exact duplicates: the FP32 form hands the
    cells of pairs nearer than ~1e-6 to the FP64 form (bit-identical results
    there).  Cells bordering a pair meet two bisectors ~d apart, an
    ill-conditioned sliver: volumes are held to 1e-9 there (FP64 against the
    oracle), and a pair that FP64 cannot separate counts as one site when the
    neighbour lists are compared."""
    rng = np.random.default_rng(16)
    pts = rng.random((2000, 3))
    k = 0
    for d in (0.0, 1e-12, 1e-9, 1e-7, 1e-5):
        for _ in range(4):
            u = rng.standard_normal(3)
            pts[k + 1] = pts[k] + d * u / np.linalg.norm(u)
            k += 2
    g32, st = gpu_all(tess, pts, "fp32", container=unit_box(tess))
    g64, _ = gpu_all(tess, pts, "fp64", container=unit_box(tess))
    assert st["rerun_fp64"] >= 32 and st["failed"] == 0
    v32, o32, n32, a32 = g32
    v64, o64, n64, a64 = g64
    o32, o64 = o32.astype(np.int64), o64.astype(np.int64)

    def lists(o, nb, i):
        return nb[o[i]:o[i + 1]].tolist()

    for i in range(32):                 # pairs 0 .. 1e-7 apart: computed in FP64
        assert v32[i] == v64[i] and lists(o32, n32, i) == lists(o64, n64, i)
    np.testing.assert_allclose(v32, v64, rtol=1e-6)
    # A cell bordering a pair nearer than FP64 can separate (0, 1e-12, 1e-9,
    # and 1e-7 apart) meets two nearly identical bisectors; which member of
    # the pair takes the face and which the sliver (or nothing) is decided by
    # rounding.  With each such pair counted as one site, every list is
    # identical; the pairs 1e-5 apart are resolved and stay separate.
    rep = np.arange(len(pts))
    rep[1:32:2] = np.arange(0, 32, 2)
    assert canonical_lists(o32, n32, rep) == canonical_lists(o64, n64, rep)
    rv, ro, ri, ra = ref_all(oracle_mod, pts, [0, 0, 0], [1, 1, 1])
    np.testing.assert_allclose(v64, rv, rtol=1e-9)
    assert canonical_lists(o64, n64, rep) == canonical_lists(ro, ri, rep)
