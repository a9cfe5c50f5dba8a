"""The reference's texture and environment unit tests, restated
(tests/unit/texture.test.mjs:1-60, environment.test.mjs:87-127)."""

import math

import numpy as np
import pytest

from raymond_gb300 import EnvironmentMap, Material, Sky, Texture, Vec2, Vec3
from raymond_gb300.scenes import mulberry32


def quadrants():
    return Texture.procedural(2, 2, lambda u, v: (Vec3(1, 0, 0) if v < 0.5 else Vec3(0, 0, 1)) if u < 0.5 else
                              (Vec3(0, 1, 0) if v < 0.5 else Vec3(1, 1, 1)))


def close(a, b, eps=1e-6):
    return all(abs(x - y) <= eps for x, y in zip(a.tuple(), b.tuple()))


def test_srgb_bytes_and_linear_samples():
    grey = Texture.procedural(1, 1, lambda u, v: Vec3(0.2158605, 0.2158605, 0.2158605))
    assert list(grey.data) == [128, 128, 128, 255]
    q = quadrants()
    assert close(q.sample(0.25, 0.25), Vec3(1, 0, 0))
    assert close(q.sample(0.75, 0.25), Vec3(0, 1, 0))
    assert close(q.sample(0.25, 0.75), Vec3(0, 0, 1))


def test_bilinear_and_wrap():
    q = quadrants()
    assert close(q.sample(0.5, 0.25), Vec3(0.5, 0.5, 0))
    assert close(q.sample(0.0, 0.25), Vec3(0.5, 0.5, 0))
    assert close(q.sample(1.25, -0.75), q.sample(0.25, 0.25))


def test_resize_keeps_picture():
    q = quadrants()
    big = q.resized(8, 8)
    assert big.width == 8
    assert close(big.sample(0.1, 0.1), q.sample(0.1, 0.1), 0.01)
    assert q.resized(2, 2) is q


def test_textures_need_their_pixels():
    with pytest.raises(ValueError):
        Texture(2, 2, np.zeros(15, dtype=np.uint8))
    with pytest.raises(ValueError):
        Texture(0, 2, np.zeros(0, dtype=np.uint8))


def test_with_texture():
    q = quadrants()
    plastic = Material.plastic(Vec3(1, 0, 0), 0.3)
    t = plastic.withTexture(q, 4)
    assert t.type == "plastic" and t.roughness == 0.3 and t.texture is q
    assert close(t.color, Vec3(1, 1, 1))
    assert (t.textureScale.x, t.textureScale.y) == (4, 4)
    assert plastic.texture is None


def test_importance_table_picks_by_light():
    env = EnvironmentMap.procedural(256, 128, lambda d: Vec3(50, 40, 30) if d.y > 0.95 else
                                    Vec3(0.2, 0.3, 0.5 * (1 if d.x > 0 else 0)))
    rnd = mulberry32(5)
    n = 100000
    integral = 0.0
    for _ in range(n):
        z = 2 * rnd() - 1
        a = 2 * math.pi * rnd()
        r = math.sqrt(1 - z * z)
        integral += env.pdf(Vec3(r * math.cos(a), z, r * math.sin(a))) * 4 * math.pi / n
    assert abs(integral - 1) < 0.02, integral
    up = 0
    for _ in range(20000):
        s = env.sampleDirection([rnd(), rnd(), rnd(), rnd()])
        assert abs(s["pdf"] - env.pdf(s["direction"])) < 1e-9
        up += s["direction"].y > 0.95
    assert up / 20000 > 0.7
    black = EnvironmentMap(8, 4, np.zeros(96, dtype=np.float32))
    assert np.isfinite(black.importance()["data"]).all()


def test_sky_radiance_from_environment():
    env = EnvironmentMap.procedural(64, 32, lambda d: Vec3(1 if d.x > 0 else 0, 0, 0))
    ahead = Vec3(0.9, 0, -0.43).normalized()
    assert Sky.environment_sky(env, 2).radiance(ahead).x > 1.9
    assert Sky.environment_sky(env, 2, math.pi).radiance(ahead).x < 0.1
    assert Sky.environment_sky(env, 2, math.pi).radiance(Vec3(-0.9, 0, 0.43).normalized()).x > 1.9
    assert close(Sky().radiance(Vec3(0, 1, 0)), Sky().zenith, 1e-12)
