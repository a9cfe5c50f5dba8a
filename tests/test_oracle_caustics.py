"""The reference's caustics tests (tests/browser/app.test.mjs:512-569) on
the oracle: its light tracer (light_trace with splat and deposit,
src/shaders.mjs:1436-1814) and photon map (photon_gather with gather,
:1499-1626) against its path tracer alone, with the reference's sizes,
sample counts and tolerances — the same checks the CUDA path's caustics
tests make."""

import time

import pytest

import fixtures
import test_gpu_caustics as cases


@pytest.fixture(autouse=True)
def on_the_oracle(monkeypatch):
    monkeypatch.setattr(cases, "trace", fixtures.oracle_trace)
    t = time.perf_counter()
    yield
    assert time.perf_counter() - t < 240, "an oracle case should take well under minutes"


@pytest.mark.parametrize("scene", ["causticLamp", "causticSun", "causticMirror", "causticLampMany", "causticSunMany"])
def test_light_tracing_agrees_with_path_tracing(scene):
    cases.test_light_tracing_agrees_with_path_tracing(None, scene)


def test_photon_mapping_through_glass_agrees():
    cases.test_photon_mapping_through_glass_agrees(None)


def test_light_tracing_is_the_same_on_any_number_of_threads():
    """Each photon draws from its own PCG stream and the splats are integer
    sums, so the frame's splats and stored photons do not depend on how the
    photons are shared out (as on the GPU, whose atomics only reorder)."""
    import numpy as np

    import oracle
    from raymond_gb300 import Camera
    from raymond_gb300.renderer import delta_objects, emitters_block, light_table, params_block

    scene, cam = fixtures.SCENES["causticLampMany"](None)
    camera = Camera(**cam)
    packed = scene.pack()
    words, powers = light_table(packed)
    deltas = delta_objects(scene)
    emitters = emitters_block(powers, len(powers), deltas, scene.sky)
    params = params_block(scene, camera, 32, 32, light_count=len(powers), max_bounces=8, spp=16, caustics=True,
                          deltas=deltas)
    one = oracle.light_trace(packed, words, params, emitters, 16384, nthreads=1)
    many = oracle.light_trace(packed, words, params, emitters, 16384, nthreads=7)
    assert np.array_equal(one["splats"], many["splats"]) and int(one["splats"].sum()) > 0
    assert np.array_equal(one["photons"].view(np.uint32), many["photons"].view(np.uint32)) and len(one["photons"])
    # a range of the photons is that part of the whole
    part = oracle.light_trace(packed, words, params, emitters, 16384, ids=(0, 8192), nthreads=3)
    rest = oracle.light_trace(packed, words, params, emitters, 16384, ids=(8192, 8192), nthreads=3)
    assert np.array_equal(part["splats"] + rest["splats"], one["splats"])
    g1 = oracle.photon_gather(packed, words, params, one["photons"], nthreads=1)
    g8 = oracle.photon_gather(packed, words, params, one["photons"], nthreads=8)
    assert np.array_equal(g1, g8)
