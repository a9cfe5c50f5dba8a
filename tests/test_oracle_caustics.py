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
