"""Host restatement of the float-pair arithmetic of the restart kernels
(ed_pair / ed_pair_mac in lsquantumed_gb300/csrc/ed_device.cuh), checking the
error bounds the code and the header state:

- the split v -> hi + lo (integer operations on the bits of v) loses at most
  2^-47 |v|;
- one pair product (hi*hi exactly by FMA, the three other terms added in
  FP32) is within 2^-45 |v w| of the exact product;
- values below 2^-126 give 0 and non-finite values NaN;
- the largest exponent of a scaled vector taken from the high 32 bits of
  its largest magnitude (ed_fx64_emax_scaled) is exact wherever it is
  reported.

The FP32 operations are emulated in float64, where every FP32 product is
exact; exact references use fractions.  No GPU needed.
"""
from fractions import Fraction

import numpy as np


def pair_split(v):
    """ed_pair for an array of doubles: (hi, lo) as float32 arrays."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    bits = v.view(np.uint64)
    hw = (bits >> np.uint64(32)).astype(np.uint64)
    lw = (bits & np.uint64(0xFFFFFFFF)).astype(np.uint64)
    sign = hw & np.uint64(0x80000000)
    e = ((hw >> np.uint64(20)) & np.uint64(0x7FF)).astype(np.int64)
    funnel = ((hw << np.uint64(3)) | (lw >> np.uint64(29))) & np.uint64(0xFFFFFFFF)
    hb = (((funnel - np.uint64(896 << 23)) & np.uint64(0xFFFFFFFF)) & np.uint64(0x7FFFFFFF)) | sign
    m = (((lw & np.uint64(0x1FFFFFFF)) >> np.uint64(5)) + np.uint64(1)) >> np.uint64(1)
    base = ((e - 919).astype(np.uint64) << np.uint64(23)) & np.uint64(0xFFFFFFFF)
    f1 = ((base + m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.float32)
    f0 = base.astype(np.uint32).view(np.float32)
    with np.errstate(invalid='ignore', over='ignore'):
        lo = (f1.astype(np.float64) - f0.astype(np.float64)).astype(np.float32)  # exact (same exponent)
    lo = (lo.view(np.uint32) | sign.astype(np.uint32)).view(np.float32)
    hi_bad = (e - 897).astype(np.uint64) > np.uint64(253)
    hb = np.where(hi_bad, np.where(e > 1150, np.uint64(0x7FC00000), sign), hb)
    lo = np.where((e - 920).astype(np.uint64) > np.uint64(230), np.float32(0.0), lo)
    return hb.astype(np.uint32).view(np.float32), lo.astype(np.float32)


def f32(x):
    return np.float32(x)


def pair_product(a, b):
    """One ed_pair_mac product (p + e) for float pairs a = (ax, ay), b = (bx, by)."""
    ax, ay = (float(t) for t in a)
    bx, by = (float(t) for t in b)
    p = f32(ax * bx)                 # __fmul_rn
    e = f32(ax * bx - float(p))      # fma(ax, bx, -p): exact
    e = f32(ax * by + float(e))      # fma: one rounding (the float64 sum is exact here or rounds far below)
    e = f32(ay * bx + float(e))
    e = f32(ay * by + float(e))
    return Fraction(float(p)) + Fraction(float(e))


def test_split_error_bound():
    rng = np.random.default_rng(7)
    v = rng.standard_normal(20000) * np.exp2(rng.integers(-90, 90, 20000))
    v = np.concatenate([v, [1.0, -1.0, np.nextafter(1.0, 2.0), 0.1, 1 / 3, 2.0 ** -102, 2.0 ** 126]])
    hi, lo = pair_split(v)
    for k in range(len(v)):
        x = Fraction(float(v[k]))
        err = abs(x - Fraction(float(hi[k])) - Fraction(float(lo[k])))
        assert err <= abs(x) * Fraction(1, 2 ** 47), (v[k], hi[k], lo[k])


def test_split_range_edges():
    hi, lo = pair_split(np.array([0.0, -0.0, 2.0 ** -127, 2.0 ** -110, 2.0 ** 128, np.inf, np.nan, 5e-324]))
    assert hi[0] == 0 and lo[0] == 0 and hi[1] == 0 and lo[1] == 0
    assert hi[2] == 0 and lo[2] == 0                       # below 2^-126: zero
    assert hi[3] != 0 and lo[3] == 0                       # below 2^-103: hi only
    assert np.isnan(hi[4]) and np.isnan(hi[5]) and np.isnan(hi[6])
    assert hi[7] == 0                                      # subnormal


def test_pair_product_error_bound():
    rng = np.random.default_rng(11)
    v = rng.uniform(-1, 1, 3000) * np.exp2(rng.integers(-40, 1, 3000))
    w = rng.uniform(-1, 1, 3000) * np.exp2(rng.integers(-40, 1, 3000))
    hv, lv = pair_split(v)
    hw, lw = pair_split(w)
    for k in range(len(v)):
        exact = Fraction(float(v[k])) * Fraction(float(w[k]))
        got = pair_product((hv[k], lv[k]), (hw[k], lw[k]))
        assert abs(got - exact) <= abs(exact) * Fraction(1, 2 ** 45), (v[k], w[k])


def test_host_pair_matches_bound():
    # ed_host_pair: hi = (float)v, lo = (float)(v - hi): error below 2^-48 |v|
    rng = np.random.default_rng(3)
    for y in rng.uniform(-1, 1, 5000):
        hi = np.float32(y)
        lo = np.float32(y - float(hi))
        err = abs(Fraction(float(y)) - Fraction(float(hi)) - Fraction(float(lo)))
        assert err <= abs(Fraction(float(y))) * Fraction(1, 2 ** 48)


def emax_scaled(absmax_hi, s):
    """ed_fx64_emax_scaled: the largest biased exponent among fl(v_r * s) from
    max |v_r| with its low 32 bits cleared, or -1 when the bounds disagree."""
    lb = np.array([absmax_hi]).view(np.uint64)[0]
    u = np.array([lb | np.uint64(0xFFFFFFFF)], dtype=np.uint64).view(np.float64)[0]
    ml, mu = absmax_hi * s, u * s
    if not (np.isfinite(ml) and np.isfinite(mu) and s > 0):
        return -1
    el = int(np.array([ml]).view(np.uint64)[0] >> np.uint64(52)) & 0x7FF
    eu = int(np.array([mu]).view(np.uint64)[0] >> np.uint64(52)) & 0x7FF
    return el if el == eu else -1


def test_emax_from_high_words():
    """The one-pass scaling of the solver takes the largest exponent of the
    scaled vector from the high 32 bits of max |w|: where both bounds agree
    it equals the exponent k_max_exponent_r finds on fl(w * s), and they
    disagree only when fl(max |w| * s) sits within 2^-20 of a power of two."""
    rng = np.random.default_rng(5)
    undetermined = 0
    for trial in range(3000):
        w = rng.standard_normal(64) * np.exp2(rng.integers(-30, 30))
        s = 1.0 / np.linalg.norm(w) if trial % 3 else float(np.exp2(rng.integers(-5, 5)))
        bits = np.abs(w).view(np.uint64) >> np.uint64(32)
        hi = (bits.max() << np.uint64(32)).astype(np.uint64).view(np.float64)
        got = emax_scaled(float(hi), s)
        want = int(((np.abs(w) * s).view(np.uint64) >> np.uint64(52)).max() & np.uint64(0x7FF))
        if got < 0:
            undetermined += 1
        else:
            assert got == want, (trial, got, want)
    # undetermined needs fl(max |w| * s) within about 2^-20 of a power of two
    assert undetermined <= 3
    # a value just below a power of two whose low word decides the binade
    v = np.array([np.nextafter(2.0, 0.0)])
    hiv = float((v.view(np.uint64) >> np.uint64(32) << np.uint64(32)).view(np.float64)[0])
    assert emax_scaled(hiv, 1.0 + 2.0 ** -40) == -1
