"""The pass kernels' log1p of a volume increment (``log1p_increment`` in
phybs_gb300/csrc/tet_math.cuh): for |x| < 1/32 the Taylor series
x - x^2/2 + ... - x^6/6 by Horner's rule in FP32 with fused multiply-adds,
log1pf outside.  Checked here against the FP64 log1p: the series' truncation
(below 2^-26 |x|) and its rounding together stay within a few FP32 ulp."""
import math

import numpy as np

COEF = [-1.0 / 6.0, 0.2, -0.25, 1.0 / 3.0, -0.5, 1.0]  # highest order first, as the kernel applies them


def _fma32(a, b, c):
    # a*b is exact in FP64 for FP32 inputs; the sum rounds once more to FP32
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def _series32(x):
    x = np.float32(x)
    s = np.float32(COEF[0])
    for c in COEF[1:]:
        s = _fma32(x, s, np.float32(c))
    return np.float32(x * s)


def test_series_within_a_few_ulp():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-1 / 32, 1 / 32, 20000), 10.0 ** rng.uniform(-12, math.log10(1 / 32), 5000),
                         -(10.0 ** rng.uniform(-12, math.log10(1 / 32), 5000))]).astype(np.float32)
    worst = 0.0
    for x in xs:
        ref = math.log1p(float(x))
        got = float(_series32(x))
        ulp = float(np.spacing(np.float32(abs(ref)))) if ref != 0.0 else float(np.finfo(np.float32).tiny)
        worst = max(worst, abs(got - ref) / ulp)
    assert worst <= 3.0, worst
