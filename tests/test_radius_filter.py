"""The FP32 pre-filter of find_neighbors_in_real_radius, checked on the CPU: a
numpy restatement of the kernel's filter (query and point FP32 coordinates
relative to the diagram's centre; the query truncated toward zero, the point
rounded), whose accept (below r^2 - band) and reject (above r^2 + band)
decisions must agree with the reference's FP64 test on absolute coordinates,
distance_squared(x, y, z, point) <= r * r (celery.rs:700-702, 825-855)."""
import numpy as np
import pytest

F32 = np.float32


def f32_rz(x):
    """Round a double toward zero to float (the kernel's f64_to_f32_rz)."""
    y = np.float32(x)
    if abs(np.float64(y)) > abs(x):
        y = np.nextafter(y, np.float32(0.0))
    return y


def fma32(a, b, c):
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def fp64_within(q, p, r):
    d = [q[a] - p[a] for a in range(3)]
    return (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2] <= r * r


@pytest.mark.parametrize("origin,extent,radius", [(0.0, 1.0, 0.006), (1e6, 1.0, 0.03), (-300.0, 50.0, 0.4),
                                                  (0.5, 1e-3, 1e-5)])
def test_filter_agrees_with_the_fp64_test(origin, extent, radius):
    rng = np.random.default_rng(int(abs(origin) + extent * 1000 + radius * 1e6))
    lo = np.full(3, origin)
    hi = lo + extent
    ctr = 0.5 * lo + 0.5 * hi
    gm = float(max(np.abs(lo - ctr).max(), np.abs(hi - ctr).max()))
    gmag = np.float32(gm)
    r = radius
    r2 = r * r
    fr, r2f = np.float32(r), np.float32(r2)
    accepted = rejected = 0
    for _ in range(20000):
        q = lo + extent * rng.random(3)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        # points near the sphere: |p - q| = r (1 + eps), eps down to 1e-9
        eps = rng.choice([-1, 1]) * 10.0 ** rng.uniform(-9, -2)
        p = q + d * r * (1 + eps)
        # the kernel's FP32 data: point rounded from (p - centre), query
        # truncated from (q - centre), both FP64-rounded differences
        hp = [np.float32(p[a] - ctr[a]) for a in range(3)]
        fq = [f32_rz(q[a] - ctr[a]) for a in range(3)]
        dx = [np.float32(fq[a] - hp[a]) for a in range(3)]
        d2 = fma32(dx[0], dx[0], fma32(dx[1], dx[1], np.float32(dx[2] * dx[2])))
        qmag = max(abs(x) for x in fq)
        m = np.float32(max(gmag, qmag) * np.float32(1.0001))
        e = np.float32(6.0e-8) * (np.float32(3.0) * m + np.float32(2.1) * fr)
        band = np.float32(2.0) * (np.float32(3.5) * fr * e + np.float32(3.0) * e * e) + np.float32(1.0e-6) * r2f
        lo_thr, hi_thr = r2f - band, r2f + band
        exact = fp64_within(q, p, r)
        if d2 < lo_thr:
            accepted += 1
            assert exact, (q, p, d2, lo_thr)
        elif d2 > hi_thr:
            rejected += 1
            assert not exact, (q, p, d2, hi_thr)
    # the filter decides most candidates away from the sphere
    assert accepted + rejected > 5000
