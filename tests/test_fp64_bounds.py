"""The FP64 form's FP32 shortcuts, checked on the CPU against exact arithmetic.

The plain FP64 form keeps every plane test that decides the topology in FP64
and moves only bounds and filters to FP32 (csrc/tess_clip_impl.cuh).  Each is
restated here in numpy float32 arithmetic, with FMAs emulated exactly, and held
to the property the kernel relies on:

- the window pre-test keeps every candidate whose bisector has a live vertex
  beyond it (exact sign), however close to the plane;
- a vertex's radius term from its FP32 copies is at least its exact |v|^2;
- the search stop on the FP32 key never skips a candidate within twice the
  cell radius;
- the tolerance threshold 1e-12 |n| from the FP32 root is within 1e-6 of the
  exact one;
- the Newton-Raphson reciprocal of the edge interpolation is within a few ulp
  of 1/d.
"""
from fractions import Fraction

import numpy as np
import pytest

F32 = np.float32
K_STOP_MARGIN = 1.0 + 1e-5          # tess_internal.cuh


def fma32(a, b, c):
    """fmaf: the exact a*b + c rounded once to float32."""
    return F32(float(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))))


def fma64(a, b, c):
    """fma (double): the exact a*b + c rounded once to float64."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def pretest_keeps(r, verts, R2f):
    """The kernel's FP32 pre-test of candidate offset r (FP64) against the
    vertices (FP64): True when it keeps the candidate."""
    rx, ry, rz = r
    r2 = float(np.float64(rx) * rx + np.float64(ry) * ry + np.float64(rz) * rz)
    fx, fy, fz, f2 = F32(rx), F32(ry), F32(rz), F32(r2)
    Rf = F32(np.sqrt(F32(R2f))) * F32(1.0001)
    margin = F32(2.4e-7) * (F32(5.0) * (abs(fx) + abs(fy) + abs(fz)) * Rf + F32(2.0) * f2)
    foff = F32(0.5) * f2
    for v in verts:
        fvx, fvy, fvz = F32(v[0]), F32(v[1]), F32(v[2])
        sdf = fma32(fx, fvx, fma32(fy, fvy, fma32(fz, fvz, -foff)))
        if not (sdf <= -margin):
            return True
    return False


def exact_sd(r, v):
    """r.v - r.r / 2 exactly (the unnormalised bisector of the site and r)."""
    rr = [Fraction(float(x)) for x in r]
    vv = [Fraction(float(x)) for x in v]
    return sum(a * b for a, b in zip(rr, vv)) - sum(a * a for a in rr) / 2


def radius_term(v):
    """|v|^2 from the FP32 copies, inflated by 1 + 5 * 2^-23 (the kernel's S.vr)."""
    fx, fy, fz = F32(v[0]), F32(v[1]), F32(v[2])
    return F32(fma32(fx, fx, fma32(fy, fy, F32(fz * fz))) * F32(1.000000596))


@pytest.mark.parametrize("scale,offset", [(1.0, 0.0), (1e-3, 0.0), (1.0, 1e6), (1e-6, 0.0), (3e4, -2e5)])
def test_pretest_never_drops_a_cutter(scale, offset):
    """Candidates whose plane has a vertex just beyond it (exact sd in
    (0, 1e-9 |r|^2]) are always kept: the margin covers the FP32 error."""
    rng = np.random.default_rng(int(scale * 1000) + 7)
    kept_close = 0
    for _ in range(300):
        # a cell of radius ~scale around the site (coordinates site-relative;
        # `offset` only shifts how the FP64 inputs were formed)
        verts = [rng.normal(size=3) * scale for _ in range(12)]
        R2 = max(float(np.dot(v, v)) for v in verts)
        R2f = float(F32(R2) * F32(1.0 + 2.0 ** -20))
        r = rng.normal(size=3) * scale * 1.5
        r = (r + offset) - offset          # FP64 rounding as a centre-relative difference leaves
        # move one vertex onto the bisector, then just beyond it
        v = verts[0]
        rn2 = float(np.dot(r, r))
        t = (rn2 / 2 - float(np.dot(r, v))) / rn2
        v = v + t * r
        for eps in (1e-15, 1e-12, 1e-9):
            w = v + eps * r
            sd = exact_sd(r, w)
            if sd > 0:
                vs = [w] + verts[1:]
                R2w = max(R2, float(np.dot(w, w)))
                R2fw = float(F32(R2w) * F32(1.0 + 2.0 ** -20))
                assert pretest_keeps(r, vs, R2fw), (scale, offset, eps, float(sd))
                kept_close += 1
    assert kept_close > 300


def test_pretest_drops_far_candidates():
    """It still filters: candidates far beyond the cell are dropped."""
    rng = np.random.default_rng(3)
    dropped = 0
    for _ in range(200):
        verts = [rng.normal(size=3) for _ in range(12)]
        R2 = max(float(np.dot(v, v)) for v in verts)
        d = rng.normal(size=3)
        r = d / np.linalg.norm(d) * (2.2 * np.sqrt(R2))
        assert all(exact_sd(r, v) < 0 for v in verts)
        dropped += not pretest_keeps(r, verts, R2 * 1.0001)
    assert dropped == 200


def test_radius_term_is_an_upper_bound():
    rng = np.random.default_rng(5)
    for e in (-30, -5, 0, 5, 30):
        for _ in range(400):
            v = rng.normal(size=3) * 2.0 ** e
            # also values just above float32 rounding points
            if rng.random() < 0.5:
                v = np.array([float(F32(x)) * (1 + 2.0 ** -25) for x in v])
            exact = sum(Fraction(float(x)) ** 2 for x in v)
            assert Fraction(float(radius_term(v))) >= exact


def test_stop_on_the_key_keeps_every_candidate_within_reach():
    """Skipped (k2 >= l2) implies r2 >= 4 R2 exactly; and the early end of the
    window (k2 > 1.001 l2) implies every later candidate is beyond reach."""
    rng = np.random.default_rng(9)
    for _ in range(4000):
        R2 = float(abs(rng.normal()) * 10.0 ** rng.integers(-8, 8))
        R2f = F32(R2)
        if float(R2f) < R2:
            R2f = np.nextafter(R2f, F32(np.inf))          # the kernel's R2 is an upper bound
        # candidates around the reach 4 R2
        r2 = 4 * R2 * (1 + float(rng.normal()) * 10.0 ** rng.integers(-9, -3))
        key = F32(r2).view(np.uint32) & np.uint32(~31 & 0xFFFFFFFF)
        k2 = np.uint32(key).view(F32)
        l2 = F32(F32(4.0) * R2f) * F32(K_STOP_MARGIN)
        if not (k2 < l2):
            assert r2 >= 4 * R2, (r2, R2)
        if k2 > l2 * F32(1.001):
            # a later candidate's key is >= k2, so its r2 is at least k2 (rounded
            # to nearest, truncated: within 2^-19 relative)
            assert float(k2) * (1 - 2.0 ** -18) >= 4 * R2


def test_tolerance_threshold():
    rng = np.random.default_rng(11)
    for _ in range(2000):
        n2 = float(abs(rng.normal()) * 10.0 ** rng.integers(-30, 30))
        n2f = F32(n2)
        tol = float(F32(1e-12) * np.sqrt(n2f)) if n2f < F32(1e37) else 1e-12 * np.sqrt(n2)
        assert abs(tol - 1e-12 * np.sqrt(n2)) <= 1e-6 * 1e-12 * np.sqrt(n2)


def recip_nr(d):
    """The kernel's recip_nr: FP32 reciprocal, two Newton-Raphson steps in FP64."""
    df = F32(d)
    if not (1e-36 < abs(float(df)) < 1e36):
        return 1.0 / d
    y = float(F32(1.0) / df)                  # __frcp_rn: the correctly rounded FP32 reciprocal
    e = fma64(-d, y, 1.0)
    y = fma64(y, e, y)
    e = fma64(-d, y, 1.0)
    return fma64(y, e, y)


def test_newton_reciprocal_within_a_few_ulp():
    rng = np.random.default_rng(13)
    worst = 0.0
    for _ in range(3000):
        d = float(rng.uniform(1, 2) * 2.0 ** rng.integers(-100, 100)) * (1 if rng.random() < 0.5 else -1)
        y = recip_nr(d)
        exact = 1 / Fraction(d)
        ulp = np.spacing(abs(float(exact)))
        err = abs(float(Fraction(y) - exact)) / ulp
        worst = max(worst, err)
    assert worst <= 4.0, worst
