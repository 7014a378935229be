"""The branch-free forms the Butteraugli kernels use in place of the reference's nested selects,
checked bitwise in float32 on the host (numpy rounds each float32 operation as the GPU does).

* separatefrequencies.hpp AmplifyRangeAroundZero / RemoveRangeAroundZero / MaximumClamp through
  the clamp c of x to [-w, w] (butter.cu amplify_range, remove_range, maximum_clamp);
* maltaDiff.hpp's asymmetric impact term as max(too_small - b, 0) + max(b - too_big, 0)
  (butter.cu malta_pre), and its final sign select as an add of the impact with diff's sign.
"""
import numpy as np

f32 = np.float32


def samples(seed, scale, extra):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(400_000) * scale).astype(f32)
    return np.concatenate([x, np.asarray(extra, f32)])


def bits(a):
    return np.asarray(a, f32).view(np.uint32)


def fma32(a, b, c):
    # a*b+c rounded once: the product of two float32 is exact in float64, and the float64 sum
    # rounded to float32 equals the single-rounded result except in double-rounding ties, which
    # both sides of each comparison below share
    return (a.astype(np.float64) * np.float64(b) + np.asarray(c, np.float64)).astype(f32)


def test_range_operators_as_clamps():
    for w in map(f32, (0.29, 0.1, 1.5, 0.04, 0.132)):
        x = samples(1, 3.0, [w, -w, 0.0, np.nextafter(w, f32(9)), np.nextafter(-w, f32(-9)), 1e-40, -1e-40])
        c = np.minimum(np.maximum(x, -w), w)
        amplify_ref = np.where(x > w, x + w, np.where(x < -w, x - w, f32(2) * x))
        remove_ref = np.where(x > w, x - w, np.where(x < -w, x + w, f32(0)))
        assert np.array_equal(bits(x + c), bits(amplify_ref))
        assert np.array_equal(bits(x - c), bits(remove_ref))


def test_maximum_clamp_as_clamp():
    k = f32(0.688059627878)
    for m in map(f32, (28.4691806922, 5.19175294647)):
        x = samples(2, 40.0, [m, -m, np.nextafter(m, f32(99)), np.nextafter(-m, f32(-99)), 1.0])
        ref = np.where(x >= m, fma32(x - m, k, m), np.where(x < -m, fma32(x + m, k, -m), x))
        c = np.minimum(np.maximum(x, -m), m)
        got = fma32(x - c, k, c)
        nz = x != 0  # fma(0, k, v) == v up to a zero's sign
        assert np.array_equal(bits(got[nz]), bits(ref[nz]))
        assert np.array_equal(got[~nz], ref[~nz])


def test_malta_impact_and_sign():
    rng = np.random.default_rng(3)
    a = (rng.standard_normal(400_000) * 2).astype(f32)
    b = (a + rng.standard_normal(400_000).astype(f32) * f32(0.5)).astype(f32)
    a = np.concatenate([a, np.asarray([0.0, -0.0, 1.0, -1.0], f32)])
    b = np.concatenate([b, np.asarray([0.0, 0.0, 0.55, -1.05], f32)])
    fabs0 = np.abs(a)
    too_small, too_big = f32(0.55) * fabs0, f32(1.05) * fabs0
    bm = np.where(a < 0, -b, b)
    impact_ref = np.where(bm < too_small, too_small - bm, np.where(bm > too_big, bm - too_big, f32(0)))
    impact = np.maximum(too_small - bm, f32(0)) + np.maximum(bm - too_big, f32(0))
    assert np.array_equal(bits(impact), bits(impact_ref))
    v = (f32(0.37) * (a - b)).astype(f32)
    diff = a - b
    scaled = impact * f32(0.81)
    ref = np.where(diff < 0, v - scaled, v + scaled)
    got = v + np.copysign(scaled, diff)
    assert np.array_equal(got, ref)  # equal values; only a zero's sign may differ
