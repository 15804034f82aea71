"""The FP32 form's guard band, checked on the CPU: a restatement of the
kernel's FP32 plane test (centre-relative hi/lo offsets, unnormalised bisector,
FMA chain) in numpy float32 arithmetic, against the exact sign from rational
arithmetic.  Whenever |sd| exceeds the band the kernel uses,
rn (e_v + guard_rel (|v|_1 + rn)) + eC, the FP32 sign must be the exact one.

Vertices are placed within ~1e-6 relative of the bisector (where tests are
decided) and sites far from the diagram's centre (where the hi/lo split's
absolute error matters)."""
from fractions import Fraction

import numpy as np
import pytest

F32 = np.float32
GUARD_REL = 4e-7                    # tess_config_default
U = 2.0 ** -24


def f32(x):
    return np.float32(x)


def fma32(a, b, c):
    # a*b is exact in float64 (48 bits); one float64 rounding of the sum
    # before the float32 one stays within the bound of a true FMA
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def split(x):
    hi = f32(x)
    return hi, f32(x - np.float64(hi))


def kernel_test(s, p, v32, ev_true, R0):
    """The kernel's FP32 sd and band for site s, point p (FP64, relative to
    the centre) and FP32 vertex v32 (site-relative) with error ev_true."""
    r = []
    for a in range(3):
        hs, ls = split(s[a])
        hp, lp = split(p[a])
        r.append(f32(f32(hp - hs) + f32(lp - ls)))
    rx, ry, rz = r
    r2 = fma32(rz, rz, fma32(ry, ry, f32(rx * rx)))
    off = f32(F32(0.5) * r2)
    rn = f32(np.sqrt(np.float64(r2)) * (1.0 + 2.0 ** -20))        # sqrt_up: an upper bound
    sd = fma32(rx, v32[0], fma32(ry, v32[1], fma32(rz, v32[2], -off)))
    # vertex error bound with the folded guard_rel |v|_1 term (as stored)
    ev = f32(ev_true * (1 + 1e-6) + GUARD_REL * float(np.abs(v32.astype(np.float64)).sum()))
    sa = F32(max(abs(f32(s[0])), abs(f32(s[1])), abs(f32(s[2])))) * F32(1.001)
    R = F32(R0 * 1.001)
    eC = F32(1.3e-13) * (sa + R) * R
    band = fma32(rn, f32(ev + F32(GUARD_REL) * rn), eC)
    return sd, band, r2


def exact_sd(s, p, v):
    """n.v - off for the exact bisector of s and p (n = r = p - s, off = r.r / 2)."""
    r = [Fraction(float(p[a])) - Fraction(float(s[a])) for a in range(3)]
    vv = [Fraction(float(x)) for x in v]
    return sum(r[a] * vv[a] for a in range(3)) - sum(x * x for x in r) / 2


@pytest.mark.parametrize("site_scale,spacing", [(0.5, 1e-2), (0.5, 1e-4), (1e3, 1e-2), (1e3, 1e-5), (3.0, 3e-7)])
@pytest.mark.parametrize("offplane", [1e-7, 1e-6, 1e-5])
@pytest.mark.parametrize("verr", [0.0, 1e-7])
def test_band_decides_only_correct_signs(site_scale, spacing, offplane, verr):
    """verr = 0: the vertex is an exact FP32 point (e_v = 0), so only the
    test's own rounding, which guard_rel and eC must cover, is left."""
    rng = np.random.default_rng(int(site_scale * 1000 + spacing * 1e7 + offplane * 1e8 + verr * 1e9))
    decided = routed = violations = 0
    worst = 0.0
    for _ in range(2000):
        s = rng.uniform(-site_scale, site_scale, 3)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        p = s + d * spacing * rng.uniform(0.2, 2.0)
        r = p - s                                       # FP64; the exact offset is p - s as rationals
        rhat = r / np.linalg.norm(r)
        # a point on the bisector, nudged off it (relative to |r|)
        t = rng.standard_normal(3)
        t -= t.dot(rhat) * rhat
        m = r / 2 + t * np.linalg.norm(r) * rng.uniform(0.0, 2.0)
        v = m + rhat * np.linalg.norm(r) * rng.uniform(-offplane, offplane)
        # its FP32 value with a position error of up to verr |v| (the exact
        # vertex is then v; with verr = 0 the vertex is the FP32 point itself)
        dv = rng.standard_normal(3)
        dv *= rng.uniform(0, verr) * np.linalg.norm(v) / np.linalg.norm(dv)
        v32 = np.array([f32(x) for x in v + dv], dtype=np.float32)
        if verr == 0.0:
            v = v32.astype(np.float64)
        ev_true = float(np.linalg.norm(v32.astype(np.float64) - v)) * (1 + 1e-9)
        R0 = max(float(np.linalg.norm(v32)), 0.5 * float(np.linalg.norm(r))) * 1.01
        sd, band, r2 = kernel_test(s, p, v32, ev_true, R0)
        # near-duplicates go to the FP64 form before any FP32 test
        dup = 1.5e-6 * (float(np.abs(s).max()) + R0)
        if float(r2) <= dup * dup:
            routed += 1
            continue
        ex = exact_sd(s, p, v)
        worst = max(worst, abs(float(sd) - float(ex)) / float(band))
        if abs(sd) > band:
            decided += 1
            if ex == 0 or (ex > 0) != (sd > 0):
                violations += 1
    assert violations == 0
    assert worst < 1.0                       # the FP32 error stays inside the band
    if routed < 1000 and offplane >= 1e-6:
        assert decided >= 100, (decided, routed)   # and the band leaves tests to decide
