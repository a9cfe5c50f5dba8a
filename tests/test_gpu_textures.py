"""Textures, normal maps, patterned lamps and the environment map on the
GPU against the CPU (tests/browser/app.test.mjs:188-240, 353-394), with the
reference's tolerances."""

import math

import numpy as np
import pytest

from fixtures import ENV_ROTATION, ENV_STRENGTH, ENVIRONMENT, interior, rgb, trace
from raymond_gb300 import Sky, Vec3

pytestmark = pytest.mark.gpu


def mean(v):
    return float(np.mean(v)) if len(v) else float("nan")


def test_gpu_textures_match_cpu(gpu):
    size = 64
    r = trace("textured", view="albedo", spp=1, size=size)
    compared = wrong = 0
    for i in interior(r["hits"], size):
        compared += 1
        if np.any(np.abs(rgb(r["pixels"], i) - r["hits"][i]["albedo"]) > 0.02):
            wrong += 1
    assert compared > size * size * 0.6, compared
    assert wrong <= compared * 0.01, (wrong, compared)


def test_gpu_normal_maps_match_cpu(gpu):
    size = 64
    r = trace("bumpy", view="normal", spp=1, size=size)
    compared = wrong = tilted = 0
    for i in interior(r["hits"], size):
        compared += 1
        n = r["hits"][i]["normal"]
        if np.dot(rgb(r["pixels"], i), n) < 0.995:
            wrong += 1
        if abs(n[1]) < 0.98 and r["hits"][i]["object"] == 0:
            tilted += 1
    assert compared > size * size * 0.6
    assert tilted > 100, tilted
    assert wrong <= compared * 0.01, (wrong, compared)


def test_gpu_patterned_lamps_match_cpu(gpu):
    size = 48
    r = trace("patternedLamps", view="albedo", spp=1, size=size)
    compared = wrong = 0
    for i in interior(r["hits"], size):
        compared += 1
        a = r["hits"][i]["albedo"]
        # the albedo view shows a lamp's light scaled to at most 1 (inspect())
        a = a / max(a.max(), 1.0)
        if np.any(np.abs(rgb(r["pixels"], i) - a) > 0.02):
            wrong += 1
    assert compared > size * size * 0.4
    assert wrong <= compared * 0.01, (wrong, compared)


def test_patterned_lamp_direct_agrees_with_bounced(gpu):
    size = 32
    direct = trace("patternedLamp", arg="light", spp=256, size=size, bounces=1)
    bounced = trace("patternedLamp", arg="glow", spp=1024, size=size, bounces=1)
    fl = [i for i in interior(direct["hits"], size, 0) if bounced["hits"][i] and bounced["hits"][i]["object"] == 0]
    for q in ((0, 0), (1, 0), (0, 1), (1, 1)):
        patch = [i for i in fl if (i % size) // (size // 2) == q[0] and (i // size) // (size // 2) == q[1]]
        for c in range(3):
            a = mean([direct["pixels"][i * 4 + c] for i in patch])
            b = mean([bounced["pixels"][i * 4 + c] for i in patch])
            assert abs(a / b - 1.0) < 0.04, (q, c, a, b)


def test_gpu_environment_matches_cpu(gpu):
    size = 48
    r = trace("environmentSky", view="albedo", spp=1, size=size)
    sky = Sky.environment_sky(ENVIRONMENT, ENV_STRENGTH, ENV_ROTATION)
    wrong = 0
    for i in range(size * size):
        d = Vec3(*r["rays"][i][3:].astype(np.float64)).normalized()
        cpu = np.array(sky.radiance(d).tuple())
        gpu_ = rgb(r["pixels"], i)
        if np.any(np.abs(gpu_ - cpu) > 0.01 * cpu + 0.005):
            wrong += 1
    assert wrong <= size * size * 0.01, wrong


def test_environment_light_matches_exact(gpu):
    sky = Sky.environment_sky(ENVIRONMENT, ENV_STRENGTH, ENV_ROTATION)
    rows, cols = 200, 400
    irr = 0.0
    for i in range(rows):
        th = (i + 0.5) / rows * math.pi / 2
        for j in range(cols):
            ph = (j + 0.5) / cols * 2 * math.pi
            l = sky.radiance(Vec3(math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph)))
            irr += (l.x + l.y + l.z) / 3 * math.cos(th) * math.sin(th) * (math.pi / 2 / rows) * (2 * math.pi / cols)
    size = 32
    r = trace("environmentFloor", spp=64, size=size, bounces=1)
    ratios = [mean(rgb(r["pixels"], i)) / (0.5 / math.pi * irr) for i in interior(r["hits"], size, 0)]
    assert len(ratios) > 200
    assert abs(mean(ratios) - 1.0) < 0.015, mean(ratios)
