"""The kernels replace the reference's float-to-double threshold tests with
float comparisons (no FP64 instruction on GB300).  Each replacement is exact:
checked here on every float within 2^20 ulps of the threshold, on both signs,
and on zero, infinities and NaN.  Far from the threshold both forms are
monotone in z and agree trivially.

  Tracking/Pyrdown.cu:136      v.z > 0.1          ->  z >= 0.1f
  Tracking/Reduction.cu:232,
  Mapping/RenderScene.cu:402   z < 1e-3           ->  z < 0.001f
  Mapping/RenderScene.cu:73    pt3d.z < 2e-1      ->  z < 0.2f

  Tracking/Reduction.cu:487    w < 1e-3           ->  w < 0.001f
  Tracking/Reduction.cu:490    sigma < 1e-6       ->  sigma <= 1e-6f

The ICP inlier tests of Tracking/Reduction.cu:253-255 compare norms,
sqrtf(d) <= 0.1f and sqrtf(s) < 0.6f, and the photometric correspondence
test of :448 compares (double)sqrtf(d) < 0.1 (the float4 norm); the kernels
compare the squared norms with the float thresholds that make the forms
agree (sqrtf is correctly rounded and monotone), checked the same way
against numpy's float32 sqrt.  The photometric row's gradient
(float)((double)g / 9.0) equals the float quotient g / 9.0f for every short
g (checked exhaustively).
"""
import numpy as np
import pytest

CASES = [
    (0.1, lambda d, t: d > t, lambda f: f >= np.float32(0.1)),
    (1e-3, lambda d, t: d < t, lambda f: f < np.float32(0.001)),
    (2e-1, lambda d, t: d < t, lambda f: f < np.float32(0.2)),
    (1e-6, lambda d, t: d < t, lambda f: f <= np.float32(1e-6)),
]


def _floats_near(t, span=1 << 20):
    base = np.array([t], np.float32).view(np.int32)[0]
    bits = np.arange(base - span, base + span, dtype=np.int64).astype(np.int32)
    near = bits.view(np.float32)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 3.4e38, -3.4e38], np.float32)
    return np.concatenate([near, -near, special])


@pytest.mark.parametrize("t,ref,ours", CASES)
def test_float_threshold_is_exact(t, ref, ours):
    f = _floats_near(t)
    with np.errstate(invalid="ignore"):
        a = ref(f.astype(np.float64), t)
        b = ours(f)
    assert np.array_equal(a, b)


SQRT_CASES = [
    (0.1, 0x3c23d70b, lambda r, t: r <= t, lambda d, T: d <= T),
    (0.6, 0x3eb851ec, lambda r, t: r < t, lambda d, T: d < T),
    (0.1, 0x3c23d70a, lambda r, t: r.astype(np.float64) < 0.1, lambda d, T: d < T),
]


@pytest.mark.parametrize("t,bits,ref,ours", SQRT_CASES)
def test_squared_norm_threshold_is_exact(t, bits, ref, ours):
    T = np.array([bits], np.uint32).view(np.float32)[0]
    d = _floats_near(float(T))
    d = d[~(d < 0)]  # squared norms are never negative
    with np.errstate(invalid="ignore"):
        a = ref(np.sqrt(d), np.float32(t))
        b = ours(d, T)
    assert np.array_equal(a, b)


def test_gradient_over_nine_is_float_division():
    g = np.arange(-32768, 32768, dtype=np.float32)
    assert np.array_equal((g.astype(np.float64) / 9.0).astype(np.float32), g / np.float32(9.0))
