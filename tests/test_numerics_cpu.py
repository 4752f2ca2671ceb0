"""Bit-level arithmetic the compensated disc kernels rely on, restated in
numpy and checked exhaustively or on many samples (no GPU).

  * f32_to_f64 (csrc/disc_comp.cu): the double of a float f >= 0 formed
    from its bit pattern -- high word (u >> 3) + bias, low word u << 29 with
    bias = 896 << 20 (+ the sign bit) -- is exact for every normal float and
    lands in [2^-127, 2^-126) for subnormals and zero;
  * the sin^2 series of the small-disc tiers and the asin^2 series stay
    within 1.8e-8 / 2.1e-8 (resp. their stated bounds) of the FP64
    functions at the tier limits;
  * ks - 1 is exact in FP32 for 1 <= ks < 2^24 (the offset normalisation
    sum), and Dekker's two-float division recovers a / b to ~2^-44;
  * the large discs' fitted asin^2(sqrt h) polynomial (g_near2 in
    csrc/comp_engine.cuh, its coefficients read from the source) is within
    2e-8 relative of asin^2(sqrt h) on [0, 1/2] in exact arithmetic (with
    the FP32-rounded coefficients) and within 1.5e-7 (two FP32 ulps) when
    evaluated in FP32.
"""
import os
import re

import numpy as np


def f32_to_f64_bits(f: np.ndarray, negative: bool = False) -> np.ndarray:
    u = f.astype(np.float32).view(np.uint32).astype(np.uint64)
    bias = np.uint64((896 << 20) + (0x80000000 if negative else 0))
    hi = ((u >> np.uint64(3)) + bias) & np.uint64(0xFFFFFFFF)
    lo = (u << np.uint64(29)) & np.uint64(0xFFFFFFFF)
    return ((hi << np.uint64(32)) | lo).view(np.float64)


def test_f32_to_f64_exact_for_every_exponent():
    rng = np.random.default_rng(7)
    # every biased exponent 1..254 with random mantissas, plus the extremes
    exps = np.repeat(np.arange(1, 255, dtype=np.uint32), 64)
    mant = rng.integers(0, 1 << 23, size=exps.size, dtype=np.uint32)
    mant[::64] = 0
    mant[1::64] = (1 << 23) - 1
    f = ((exps << 23) | mant).view(np.float32)
    got = f32_to_f64_bits(f)
    np.testing.assert_array_equal(got, f.astype(np.float64))
    np.testing.assert_array_equal(f32_to_f64_bits(f, negative=True), -f.astype(np.float64))


def test_f32_to_f64_subnormals_and_zero_stay_below_the_normal_range():
    sub = np.concatenate([[0], np.arange(1, 1 << 23, 4099, dtype=np.uint32)]).astype(np.uint32)
    got = f32_to_f64_bits(sub.view(np.float32))
    assert np.all(got >= 2.0 ** -127) and np.all(got < 2.0 ** -126)


def _sin2_series(x, tier):
    x2 = (x * x).astype(np.float32)
    if tier == 0:
        q = np.float32(1) - x2 / np.float32(3)
    else:
        q = np.float32(-1 / 315) * x2 + np.float32(2 / 45)
        q = q * x2 - np.float32(1 / 3)
        q = q * x2 + np.float32(1)
    return x2.astype(np.float64) * q.astype(np.float64)


def test_sin2_series_truncation_within_fp32_rounding_at_the_tier_limits():
    for tier, xmax, bound in ((0, 0.025, 1.8e-8), (1, 0.33, 2.1e-8)):
        x = np.linspace(1e-6, xmax, 20001)
        x32 = x.astype(np.float32).astype(np.float64)
        ref = np.sin(x32) ** 2
        # the series in exact arithmetic (FP64 here): truncation only
        x2 = x32 * x32
        if tier == 0:
            ser = x2 * (1 - x2 / 3)
        else:
            ser = x2 * (1 - x2 / 3 + 2 * x2 ** 2 / 45 - x2 ** 3 / 315)
        assert np.max(np.abs(ser - ref) / ref) < bound, tier
        # and the FP32 evaluation stays within a few FP32 ulps
        assert np.max(np.abs(_sin2_series(x32, tier) - ref) / ref) < 4e-7, tier


def test_asin2_series_truncation_at_the_tier_limits():
    for terms, hmax, bound in ((3, 4e-3, 7.4e-9), (5, 0.02, 3e-10)):
        h = np.linspace(1e-9, hmax, 20001)
        ref = np.arcsin(np.sqrt(h)) ** 2
        c = [1.0, 1 / 3, 8 / 45, 4 / 35, 128 / 1575][:terms]
        ser = h * sum(ck * h ** k for k, ck in enumerate(c))
        assert np.max(np.abs(ser - ref) / ref) < bound


def test_offset_sum_removal_is_exact_in_fp32():
    rng = np.random.default_rng(3)
    ks = (np.float32(1) + rng.random(100000, dtype=np.float32) * np.float32(1 << 23)).astype(np.float32)
    d = ks - np.float32(1)
    np.testing.assert_array_equal(d.astype(np.float64), ks.astype(np.float64) - 1.0)


def _div_ff(ah, al, bh, bl):
    f = np.float32
    b = f(bh + bl)
    b_lo = f(bl - f(b - bh))
    q1 = f(ah / b)
    p = f(q1 * b)
    pe = np.float32(np.float64(q1) * np.float64(b) - np.float64(p))   # FMA: exact product error
    r = f(f(f(f(ah - p) - pe) + al) - f(q1 * b_lo))
    q2 = f(r / b)
    hi = f(q1 + q2)
    return hi, f(q2 - f(hi - q1))


def test_two_float_division():
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(2000):
        a = rng.uniform(1e-3, 1e3)
        b = rng.uniform(1.0, 1e6)
        ah = np.float32(a); al = np.float32(a - float(ah))
        bh = np.float32(b); bl = np.float32(b - float(bh))
        hi, lo = _div_ff(ah, al, bh, bl)
        exact = (float(ah) + float(al)) / (float(bh) + float(bl))
        worst = max(worst, abs(float(hi) + float(lo) - exact) / exact)
    assert worst < 2.0 ** -42, worst


def _g_near_coefficients():
    """Q's coefficients, highest degree first, as g_near2 evaluates them."""
    src = open(os.path.join(os.path.dirname(__file__), "..", "dm-annihilation-cxx_gb300", "csrc",
                            "comp_engine.cuh")).read()
    body = src[src.index("float2 g_near2("):]
    body = body[:body.index("return mul2(h, q);")]
    nums = [float(v) for v in re.findall(r"f2\((-?[0-9.]+(?:e-?[0-9]+)?)f\)", body)]
    assert len(nums) == 9, nums
    return nums


def test_large_disc_asin2_polynomial():
    c = _g_near_coefficients()
    h = np.linspace(0.0, 0.5, 50001)[1:]
    ref = np.arcsin(np.sqrt(h)) ** 2
    q = np.zeros_like(h)
    for ck in c:
        q = q * h + ck
    assert np.max(np.abs(h * q - ref) / ref) < 2e-8
    # FP32 Horner with fused steps (one rounding per FMA), then g = h * q
    h32 = h.astype(np.float32)
    q32 = np.full_like(h32, np.float32(c[0]))
    for ck in c[1:]:
        q32 = (q32.astype(np.float64) * h32.astype(np.float64) + np.float64(np.float32(ck))).astype(np.float32)
    g32 = (h32 * q32).astype(np.float64)
    ref32 = np.arcsin(np.sqrt(h32.astype(np.float64))) ** 2
    assert np.max(np.abs(g32 - ref32) / ref32) < 1.5e-7
    assert c[-1] == 1.0   # Q(0) = 1: g = h + O(h^2) near the disc centre
