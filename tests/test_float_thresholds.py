"""The kernels replace the reference's float-to-double threshold tests with
float comparisons (no FP64 instruction on GB300).  Each replacement is exact:
checked here on every float within 2^20 ulps of the threshold, on both signs,
and on zero, infinities and NaN.  Far from the threshold both forms are
monotone in z and agree trivially.

  Tracking/Pyrdown.cu:136      v.z > 0.1          ->  z >= 0.1f
  Tracking/Reduction.cu:232,
  Mapping/RenderScene.cu:402   z < 1e-3           ->  z < 0.001f
  Mapping/RenderScene.cu:73    pt3d.z < 2e-1      ->  z < 0.2f

The ICP inlier tests of Tracking/Reduction.cu:253-255 compare norms,
sqrtf(d) <= 0.1f and sqrtf(s) < 0.6f; the kernel compares the squared norms
with the float thresholds that make the two forms agree (sqrtf is correctly
rounded and monotone), checked the same way against numpy's float32 sqrt.
"""
import numpy as np
import pytest

CASES = [
    (0.1, lambda d, t: d > t, lambda f: f >= np.float32(0.1)),
    (1e-3, lambda d, t: d < t, lambda f: f < np.float32(0.001)),
    (2e-1, lambda d, t: d < t, lambda f: f < np.float32(0.2)),
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
