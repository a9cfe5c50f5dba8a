"""The environment upload's half floats: to_half restates toHalf
(src/Renderer.mjs:1143-1160); to_half_array, which converts a whole map at
once, gives the same bits on every value, including exact powers of two,
their neighbours, the subnormal range and saturation."""

import numpy as np

from raymond_gb300.renderer import to_half, to_half_array


def test_known_half_values():
    assert to_half(1.0) == 0x3C00 and to_half(2.0) == 0x4000 and to_half(0.5) == 0x3800
    assert to_half(65504.0) == 0x7BFF and to_half(1e9) == 0x7BFF
    assert to_half(0.0) == 0 and to_half(-3.0) == 0 and to_half(float("nan")) == 0
    assert to_half(5.9605e-8) == 1  # the smallest subnormal


def test_array_conversion_matches_the_scalar_one():
    rng = np.random.default_rng(1)
    pw = np.ldexp(1.0, np.arange(-24, 16))
    vals = np.concatenate([
        rng.random(20000) * 10, np.exp(rng.uniform(-25, 12, 30000)), rng.random(1000) * 1e-4,
        pw, np.nextafter(pw, 0), np.nextafter(pw, np.inf), pw * 1.00048828125, pw * 0.999755859375,
        [0.0, -1.0, np.nan, np.inf, -np.inf, 65504.0, 65503.9, 6.1035e-5, 6.1034e-5, 2.98e-8],
    ]).astype(np.float32).astype(np.float64)  # environment data is float32
    want = np.array([to_half(float(v)) for v in vals], dtype=np.uint16)
    assert np.array_equal(to_half_array(vals), want)
