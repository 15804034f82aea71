"""The binning pass's FP32 bin index (axis_index_fast in tess_grid.cu),
restated in numpy float32 arithmetic, against the exact FP64 formula of
get_{x,y,z}_cell_index (celery.rs:269-314): whenever the FP32 estimate and its
error bound decide the bin, the bin is the FP64 formula's; the rest (points
within the bound of a boundary) fall back to that formula.  Checked on
uniform coordinates, on coordinates placed exactly at bin boundaries (and one
ulp either side), and in boxes far from the origin and at negative offsets."""
import numpy as np
import pytest


def exact_axis(x, lo, hi, inv, cpd):
    v = (x - lo) * inv                       # two FP64 roundings, no FMA (numpy)
    out = np.where(v > 0.0, np.minimum(np.floor(np.where(v > 0.0, v, 0.0)), cpd - 1), 0).astype(np.int64)
    return np.where(x >= hi, cpd - 1, out)


def trunc_f32(x):
    f = x.astype(np.float32)
    over = np.abs(f.astype(np.float64)) > np.abs(x)
    f[over] = np.nextafter(f[over], np.float32(0))
    return f


def fast_axis(x, lo, hi, inv, cpd):
    """(bin, decided) as the kernel computes them."""
    f32 = np.float32
    xf = trunc_f32(x)
    lf, invf = f32(lo), f32(inv)
    t = (xf - lf) * invf
    E = invf * (np.abs(xf) + np.abs(lf)) * f32(2.3841858e-7) + np.abs(t) * f32(4.7683716e-7)
    up, dn = t + E, t - E
    b = np.zeros(len(x), dtype=np.int64)
    ok = np.zeros(len(x), dtype=bool)
    with np.errstate(invalid="ignore", over="ignore"):
        hi_side = x >= hi
        b[hi_side], ok[hi_side] = cpd - 1, True
        low = ~ok & (up < f32(1))
        b[low], ok[low] = 0, True
        top = ~ok & (dn >= f32(cpd - 1))
        b[top], ok[top] = cpd - 1, True
        mid = ~ok & (dn > 0) & (np.floor(dn) == np.floor(up))
        b[mid], ok[mid] = np.floor(dn[mid]).astype(np.int64), True
    # the kernel sends zeros, subnormals and values outside FP32's normal
    # range to the FP64 formula
    tiny = (np.abs(x) < np.finfo(np.float32).tiny) | (np.abs(x) > np.finfo(np.float32).max)
    ok &= ~tiny
    return b, ok


@pytest.mark.parametrize("lo,hi,n,cpd", [(1.3e-7, 0.99999988, 16_777_216, 238), (0.0, 1.0, 1_000_000, 93),
                                         (-1000.0, 500.0, 4_194_304, 150), (1.0e6, 1.0e6 + 1.0, 1_000_000, 93),
                                         (-3.7e-3, 2.5e-3, 8000, 19)])
def test_fast_bin_index_is_exact(lo, hi, n, cpd):
    rng = np.random.default_rng(cpd)
    inv = cpd / (hi - lo)
    # uniform coordinates, boundaries k / inv + lo exactly and one ulp either
    # side, and the ends
    k = rng.integers(0, cpd + 1, 200_000)
    edges = lo + k / inv
    xs = np.concatenate([lo + (hi - lo) * rng.random(400_000), edges, np.nextafter(edges, np.inf),
                         np.nextafter(edges, -np.inf), [lo, hi, np.nextafter(hi, -np.inf), np.nextafter(lo, np.inf)]])
    xs = xs[(xs >= lo) & (xs <= hi)]
    want = exact_axis(xs, lo, hi, inv, cpd)
    got, ok = fast_axis(xs, lo, hi, inv, cpd)
    assert np.array_equal(got[ok], want[ok])
    unif = ok[:400_000]
    if abs(lo) < 1e3 and hi - lo > 1e-2:
        assert unif.mean() > 0.99           # the FP64 formula is rarely needed


def test_the_bound_is_needed():
    """Without the error bound, the FP32 estimate puts coordinates just above a
    bin boundary into the bin below (x truncated to FP32 falls under it)."""
    lo, hi, cpd = 1.3e-7, 0.99999988, 238
    inv = cpd / (hi - lo)
    k = np.arange(1, cpd)
    xs = np.nextafter(lo + k / inv, np.inf)
    want = exact_axis(xs, lo, hi, inv, cpd)
    f32 = np.float32
    naive = np.floor((trunc_f32(xs) - f32(lo)) * f32(inv)).astype(np.int64)
    assert (naive != want).any()
    got, ok = fast_axis(xs, lo, hi, inv, cpd)
    assert np.array_equal(got[ok], want[ok]) and not ok.all()
