"""Light transport against exact answers (tests/browser/app.test.mjs:244-510)
on the CUDA path, with the reference's tolerances."""

import math

import numpy as np
import pytest

from fixtures import interior, rgb, trace

pytestmark = pytest.mark.gpu


def mean(v):
    return float(np.mean(v)) if len(v) else float("nan")


def test_white_furnace_diffuse(gpu):
    size = 32
    r = trace("furnaceDiffuse", spp=64, size=size)
    hits = r["hits"]
    ball = [mean(rgb(r["pixels"], i)) for i in interior(hits, size, 0)]
    sky = [mean(rgb(r["pixels"], i)) for i in range(size * size)
           if all(0 <= j < len(hits) and hits[j] is None for j in (i, i - 1, i + 1, i - size, i + size))]
    assert abs(mean(ball) - 0.8) < 0.01, mean(ball)
    assert abs(mean(sky) - 1.0) < 1e-4, mean(sky)


def test_white_furnace_glass(gpu):
    size = 32
    r = trace("furnaceGlass", spp=128, size=size, bounces=32)
    ball = [mean(rgb(r["pixels"], i)) for i in interior(r["hits"], size, 0)]
    assert abs(mean(ball) - 1.0) < 0.015, mean(ball)


def test_white_furnace_dispersive_glass(gpu):
    size = 32
    r = trace("furnaceDispersive", spp=256, size=size, bounces=32)
    ball = interior(r["hits"], size, 0)
    for c in range(3):
        ch = mean([r["pixels"][i * 4 + c] for i in ball])
        assert abs(ch - 1.0) < 0.03, (c, ch)


def test_dispersion_fringes(gpu):
    size = 48

    def colourfulness(res):
        best = 0.0
        for i in range(size * size):
            p = rgb(res["pixels"], i)
            total = p.sum()
            if total > 0.05:
                best = max(best, (p.max() - p.min()) / total)
        return best

    plain = colourfulness(trace("stripThroughGlass", arg="0", spp=64, size=size, bounces=8))
    split = colourfulness(trace("stripThroughGlass", arg="15", spp=64, size=size, bounces=8))
    assert plain < 1e-3, plain
    assert split > 0.3, split


def test_white_furnace_fog(gpu):
    size = 32
    r = trace("furnaceFog", spp=128, size=size, bounces=64)
    allm = mean([mean(rgb(r["pixels"], i)) for i in range(size * size)])
    assert abs(allm - 1.0) < 0.01, allm


def test_black_smoke_falls_off_exponentially(gpu):
    size = 48
    r = trace("blackSmoke", spp=256, size=size)
    rays = r["rays"].astype(np.float64)

    def sphere_chord(o, d):
        oc = o - np.array([-0.7, 0, 0])
        a, b, c = d @ d, oc @ d, oc @ oc - 0.64
        disc = b * b - a * c
        return 2 * math.sqrt(disc) / a * math.sqrt(a) if disc > 0 else 0.0

    ry, rx = 0.6, 0.4

    def to_box(v):
        cy, sy, cx, sx = math.cos(-ry), math.sin(-ry), math.cos(-rx), math.sin(-rx)
        y = [cy * v[0] + sy * v[2], v[1], -sy * v[0] + cy * v[2]]
        return [y[0], cx * y[1] - sx * y[2], sx * y[1] + cx * y[2]]

    size_b = [0.6, 0.5, 0.4]

    def box_chord(o, d):
        ob = [c / size_b[k] for k, c in enumerate(to_box(o - np.array([0.6, 0, 0])))]
        db = [c / size_b[k] for k, c in enumerate(to_box(d))]
        near, far = -math.inf, math.inf
        for k in range(3):
            if db[k] == 0:
                if abs(ob[k]) > 1:
                    return 0.0
                continue
            t0, t1 = (-1 - ob[k]) / db[k], (1 - ob[k]) / db[k]
            near, far = max(near, min(t0, t1)), min(far, max(t0, t1))
        return (far - max(near, 0)) * math.sqrt(d @ d) if far > near and far > 0 else 0.0

    expected = np.array([math.exp(-1.5 * (sphere_chord(r_[:3], r_[3:]) + box_chord(r_[:3], r_[3:]))) for r_ in rays])
    smooth = []
    for y in range(1, size - 1):
        for x in range(1, size - 1):
            i = y * size + x
            if expected[i] < 0.98 and all(abs(expected[j] - expected[i]) < 0.05 for j in (i - 1, i + 1, i - size, i + size)):
                smooth.append(i)
    assert len(smooth) > 100
    ratio = mean([r["pixels"][i * 4] / expected[i] for i in smooth])
    assert abs(ratio - 1.0) < 0.02, ratio


def assert_floor_matches(result, size, irradiance, tol):
    ratios = []
    for i in interior(result["hits"], size, 0):
        exp = 0.5 / math.pi * irradiance(result["hits"][i]["point"])
        if exp > 0.02:
            ratios.append(result["pixels"][i * 4] / exp)
    assert len(ratios) > 200, len(ratios)
    assert abs(mean(ratios) - 1.0) < tol, mean(ratios)


def test_sphere_light_exact(gpu):
    size = 48
    r = trace("sphereLight", spp=64, size=size, bounces=1)
    centre, radius, emission = np.array([0.5, 1.5, -1]), 0.5, 6.0

    def irr(p):
        to = centre - p
        d = np.linalg.norm(to)
        cos_t = to[1] / d
        return 0 if cos_t < radius / d else math.pi * emission * (radius / d) ** 2 * cos_t

    assert_floor_matches(r, size, irr, 0.015)


def test_quad_light_exact(gpu):
    size = 48
    r = trace("quadLight", spp=128, size=size, bounces=1)
    corners = np.array([[-0.5, 1.5, -1.5], [0.7, 1.5, -1.5], [0.7, 1.5, -0.7], [-0.5, 1.5, -0.7]])

    def irr(p):
        s = 0.0
        for k in range(4):
            a, b = corners[k] - p, corners[(k + 1) % 4] - p
            c = np.cross(a, b)
            angle = math.acos(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)))
            s += angle * c[1] / np.linalg.norm(c)
        return 6.0 / 2 * abs(s)

    assert_floor_matches(r, size, irr, 0.015)


def test_overhead_sun_exact(gpu):
    size = 32
    r = trace("sun", spp=16, size=size, bounces=1)
    irradiance = 2.0 * (1 + math.cos(0.05)) / 2
    assert_floor_matches(r, size, lambda p: irradiance, 0.005)


@pytest.mark.parametrize("material", ["diffuse", "plastic", "metal"])
def test_mis_direct_agrees_with_bounced(gpu, material):
    size = 32
    direct = trace("lightAsSphere", arg=material, spp=256, size=size, bounces=1)
    bounced = trace("lightAsMesh", arg=material, spp=1024, size=size, bounces=1)
    fl = [i for i in interior(direct["hits"], size, 0) if bounced["hits"][i] and bounced["hits"][i]["object"] == 0]
    a = mean([mean(rgb(direct["pixels"], i)) for i in fl])
    b = mean([mean(rgb(bounced["pixels"], i)) for i in fl])
    assert len(fl) > 200
    assert abs(a / b - 1.0) < 0.03, (a, b)


def test_light_through_fog_agrees_with_scattering(gpu):
    size = 32
    direct = trace("lampInFog", arg="light", spp=256, size=size, bounces=1)
    bounced = trace("lampInFog", arg="mesh", spp=1024, size=size, bounces=1)
    a = mean([mean(rgb(direct["pixels"], i)) for i in range(size * size)])
    b = mean([mean(rgb(bounced["pixels"], i)) for i in range(size * size)])
    assert abs(a / b - 1.0) < 0.03, (a, b)
