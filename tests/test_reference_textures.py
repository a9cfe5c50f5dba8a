"""The reference's texture and environment unit tests, restated
(tests/unit/texture.test.mjs:1-60, environment.test.mjs:87-127)."""

import math

import numpy as np
import pytest

from raymond_gb300 import EnvironmentMap, Material, Sky, Texture, Vec3
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


def importance_loop(env):
    """EnvironmentMap.importance (src/EnvironmentMap.mjs:202-247) value by
    value, for small maps: the check on the vectorised table."""
    W, H = env.width, env.height
    px = env.data.astype(np.float64)
    cw, ch = min(W, 512), min(H, 256, min(W, 512))
    data = np.zeros(cw * (ch + 1), dtype=np.float32)
    rows = []
    for y in range(ch):
        y0 = math.floor(y * H / ch)
        y1 = max(y0 + 1, math.floor((y + 1) * H / ch))
        sin = math.sin((y + 0.5) / ch * math.pi)
        s = 0.0
        for x in range(cw):
            x0 = math.floor(x * W / cw)
            x1 = max(x0 + 1, math.floor((x + 1) * W / cw))
            light = 0.0
            for yy in range(y0, y1):
                for xx in range(x0, x1):
                    i = (yy * W + xx) * 3
                    light += 0.2126 * px[i] + 0.7152 * px[i + 1] + 0.0722 * px[i + 2]
            s += light / ((y1 - y0) * (x1 - x0)) * sin
            data[y * cw + x] = s
        for x in range(cw):
            data[y * cw + x] = float(data[y * cw + x]) / s if s > 0 else (x + 1) / cw
        rows.append(s)
    total = 0.0
    for r in rows:
        total += r
    running = 0.0
    for y in range(ch):
        running += rows[y]
        data[ch * cw + y] = running / total if total > 0 else (y + 1) / ch
    data[ch * cw + ch - 1] = 1.0
    for y in range(ch):
        data[y * cw + cw - 1] = 1.0
    return cw, ch, data


@pytest.mark.parametrize("w,h", [(8, 4), (37, 19), (600, 300), (700, 333)])
def test_importance_table_is_bit_identical_to_the_loop(w, h):
    rng = np.random.default_rng(w * 1000 + h)
    values = rng.exponential(1.0, size=w * h * 3) ** 3  # a few bright pixels among dim ones
    values[: w * 3 * (h // 3)] = 0.0  # and dark rows, which fall back to uniform
    env = EnvironmentMap(w, h, values)
    imp = env.importance()
    cw, ch, data = importance_loop(env)
    assert (imp["width"], imp["height"]) == (cw, ch)
    assert np.array_equal(imp["data"].view(np.uint32), data.view(np.uint32))


@pytest.mark.parametrize("srgb", [True, False])
def test_resizing_samples_as_sample_many_does(srgb):
    """Texture.resized samples at texel centres (src/Texture.mjs:193-209);
    its row-and-column gather gives sample_many's values bit for bit."""
    rng = np.random.default_rng(7)
    t = Texture(37, 19, rng.integers(0, 256, 37 * 19 * 4, dtype=np.uint8))
    w, h = 64, 40
    ys, xs = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    expected = t.sample_many((xs + 0.5) / w, (ys + 0.5) / h, srgb)
    got = t._sample_grid((np.arange(w) + 0.5) / w, (np.arange(h) + 0.5) / h, srgb)
    assert np.array_equal(got.view(np.uint64), expected.view(np.uint64))
    out = t.resized(w, h, srgb).data.reshape(h, w, 4)
    assert (out[..., 3] == 255).all()
