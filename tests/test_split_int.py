"""The binning pass's FP32 pair split (split_rn_int in tess_grid.cu: hi = u
rounded to FP32, lo = u - hi rounded to FP32) by integer operations, restated
in numpy, against the FP64 definition it replaces, bit for bit: random
magnitudes and signs, halfway cases (ties to even), carries into the exponent,
zeros, and the values that must take the FP64 path (subnormal or out of
FP32's normal range)."""
import numpy as np


def split_int(u):
    """(hi, lo, ok) as the kernel computes them; ok False -> FP64 path."""
    b = u.view(np.uint64)
    sign = (b >> np.uint64(63)).astype(bool)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (b & np.uint64((1 << 52) - 1)) | np.uint64(1 << 52)
    q = (m >> np.uint64(29)).astype(np.int64)
    rem = (m & np.uint64((1 << 29) - 1)).astype(np.int64)
    half = 1 << 28
    up = (rem > half) | ((rem == half) & ((q & 1) == 1))
    q = q + up
    diff = m.astype(np.int64) - (q << 29)
    carry = q == (1 << 24)
    qq = np.where(carry, q >> 1, q)
    ehi = e + carry
    fe = ehi - 1023 + 127
    ok = (e != 0) & (e != 0x7FF) & (fe >= 1) & (fe <= 254)
    pe = e - 1023 - 52 + 127
    ok &= (diff == 0) | (pe >= 1)
    hi_bits = (sign.astype(np.uint32) << np.uint32(31)) | (np.clip(fe, 0, 255).astype(np.uint32) << np.uint32(23)) | \
        (qq & 0x7FFFFF).astype(np.uint32)
    hi = hi_bits.view(np.float32)
    d = np.where(sign, -diff, diff).astype(np.float32)         # round to nearest
    scale = (np.clip(pe, 1, 254).astype(np.uint32) << np.uint32(23)).view(np.float32)
    lo = np.where(diff == 0, np.float32(0), d * scale)
    zero = (e == 0) & ((b << np.uint64(1)) == 0)
    hi = np.where(zero, np.where(sign, np.float32(-0.0), np.float32(0.0)), hi)
    lo = np.where(zero, np.float32(0), lo)
    return hi, lo, ok | zero


def reference(u):
    hi = u.astype(np.float32)
    lo = (u - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def test_split_bit_exact():
    rng = np.random.default_rng(0)
    u = np.concatenate([
        rng.standard_normal(500_000) * 10.0 ** rng.uniform(-30, 30, 500_000),
        rng.random(200_000) - 0.5,
        [0.0, -0.0, 1.0, -1.0, 3.0e38, -2.9e38, 1e-37, 2.0 ** -126, 2.0 ** -130],
    ])
    # halfway cases and carries: significands whose 29 low bits are exactly
    # half (ties to even) or round up into the next power of two
    base = rng.integers(1 << 23, 1 << 24, 20_000).astype(np.float64)
    exps = rng.integers(-60, 60, 20_000)
    ties = np.ldexp(base + 0.5, exps)                               # 24-bit value + half an ulp
    carry = np.ldexp(float((1 << 24) - 1) + 0.75, exps)            # rounds up to 2^24
    u = np.concatenate([u, ties, -ties, carry, np.nextafter(ties, np.inf), np.nextafter(ties, -np.inf)])
    hi, lo, ok = split_int(u)
    rh, rl = reference(u[ok])
    assert np.array_equal(hi[ok].view(np.uint32), rh.view(np.uint32))
    assert np.array_equal(lo[ok].view(np.uint32), rl.view(np.uint32))
    # the integer path declines only magnitudes whose low part would be
    # subnormal (below 2^-74) or whose high part leaves FP32's range
    bad = np.abs(u[~ok])
    assert np.all((bad < 2.0 ** -74) | (bad > 3.4e38))
    # coordinates of any sensible box take it: the unit-scale draws all do
    unit = np.abs(u) > 2.0 ** -60
    assert ok[unit & (np.abs(u) < 1e30)].all()
