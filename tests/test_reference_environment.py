"""tests/unit/environment.test.mjs:9-85 of the reference, restated: the
equirectangular layout (directions round the horizon from -z, down from
straight up), procedural maps at pixel centres, the constructor's checks,
and Radiance .hdr files read back flat and run-length encoded. (The
importance table and the sky's radiance, environment.test.mjs:87-127, are
restated in test_reference_textures.py.)"""

import math

import numpy as np
import pytest

from raymond_gb300 import EnvironmentMap, Vec3


def test_directions_and_texture_coordinates():
    d = EnvironmentMap.direction(0.5, 0.5)
    assert np.allclose(d.tuple(), (0, 0, -1), atol=1e-12)  # the middle is ahead
    d = EnvironmentMap.direction(0.75, 0.5)
    assert np.allclose(d.tuple(), (1, 0, 0), atol=1e-12)  # three quarters is +x
    assert abs(EnvironmentMap.direction(0.3, 0).y - 1) <= 1e-12
    assert abs(EnvironmentMap.direction(0.3, 1).y + 1) <= 1e-12
    for u, v in ((0.1, 0.2), (0.6, 0.7), (0.95, 0.4)):
        u2, v2 = EnvironmentMap.uv(EnvironmentMap.direction(u, v))
        assert abs(u2 - u) <= 1e-12 and abs(v2 - v) <= 1e-12


def test_procedural_maps_take_pixel_centres():
    env = EnvironmentMap.procedural(64, 32, lambda d: Vec3(d.y + 1, 0, 0))
    assert abs(env.data[0] - (math.cos(math.pi / 64) + 1)) <= 1e-6  # the top row is half a pixel down
    assert abs(env.sample(Vec3(0, 0, -1)).x - 1) <= 0.02
    with pytest.raises(ValueError):
        EnvironmentMap(2, 2, [1, 2, 3])
    assert list(EnvironmentMap(1, 1, [-1, float("nan"), 2]).data) == [0, 0, 2]  # negative and broken values dropped

