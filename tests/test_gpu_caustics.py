"""Light tracing and photon mapping against path tracing alone
(tests/browser/app.test.mjs:512-569), with the reference's tolerances:
the two must agree over the floor and in the caustic."""

import numpy as np
import pytest

from fixtures import interior, rgb, trace

pytestmark = pytest.mark.gpu


def mean(v):
    return float(np.mean(v)) if len(v) else float("nan")


@pytest.mark.parametrize("scene", ["causticLamp", "causticSun", "causticMirror", "causticLampMany", "causticSunMany"])
def test_light_tracing_agrees_with_path_tracing(gpu, scene):
    size = 32
    traced = trace(scene, spp=128, size=size, bounces=8, caustics=True)
    alone = trace(scene, spp=8192 if scene.endswith("Many") else 2048, size=size, bounces=8, caustics=False)
    fl = interior(traced["hits"], size, 0)

    def brightness(r, i):
        return mean(rgb(r["pixels"], i))

    def allf(r):
        return mean([brightness(r, i) for i in fl])

    assert len(fl) > 200
    assert abs(allf(traced) / allf(alone) - 1) < 0.04, (allf(traced), allf(alone))
    order = sorted(fl, key=lambda i: -brightness(alone, i))
    caustic = order[: -(-len(fl) // 10)]
    lit = lambda r: mean([brightness(r, i) for i in caustic])
    assert abs(lit(traced) / lit(alone) - 1) < 0.08, (lit(traced), lit(alone))


def test_photon_mapping_through_glass_agrees(gpu):
    size = 32
    mapped = trace("causticThroughGlass", spp=512, size=size, bounces=10, caustics=True)
    alone = trace("causticThroughGlass", spp=4096, size=size, bounces=10, caustics=False)

    def misses_ball(ray):
        o, d = ray[:3].astype(np.float64), ray[3:].astype(np.float64)
        oc = o - np.array([0, 0.9, 0])
        b, c = oc @ d, oc @ oc - 0.55 * 0.55
        return b * b - (d @ d) * c < 0

    pane = [i for i in interior(mapped["hits"], size, 3) if mapped["rays"][i][4] < 0 and misses_ball(mapped["rays"][i])]

    def brightness(r, i):
        return mean(rgb(r["pixels"], i))

    assert len(pane) > 300, len(pane)
    allf = lambda r: mean([brightness(r, i) for i in pane])
    assert abs(allf(mapped) / allf(alone) - 1) < 0.04, (allf(mapped), allf(alone))
    order = sorted(pane, key=lambda i: -brightness(alone, i))
    caustic = order[: -(-len(pane) // 4)]
    lit = lambda r: mean([brightness(r, i) for i in caustic])
    assert abs(lit(mapped) / lit(alone) - 1) < 0.15, (lit(mapped), lit(alone))
