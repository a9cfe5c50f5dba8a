"""The oracle pinned to the reference's exact-answer tests
(tests/browser/app.test.mjs:244-510): the same checks, tolerances, sizes and
sample counts as the CUDA path's light-transport tests, with the oracle's
path tracer (the trace shader restated in f32 on the CPU) making the
images. An oracle that failed these could not vouch for the GPU."""

import time

import pytest

import fixtures
import test_gpu_light as cases


@pytest.fixture(autouse=True)
def on_the_oracle(monkeypatch):
    monkeypatch.setattr(cases, "trace", fixtures.oracle_trace)
    t = time.perf_counter()
    yield
    assert time.perf_counter() - t < 120, "an oracle case should take seconds"


def test_white_furnace_diffuse():
    cases.test_white_furnace_diffuse(None)


def test_white_furnace_glass():
    cases.test_white_furnace_glass(None)


def test_white_furnace_dispersive_glass():
    cases.test_white_furnace_dispersive_glass(None)


def test_dispersion_fringes():
    cases.test_dispersion_fringes(None)


def test_white_furnace_fog():
    cases.test_white_furnace_fog(None)


def test_black_smoke_falls_off_exponentially():
    cases.test_black_smoke_falls_off_exponentially(None)


def test_sphere_light_exact():
    cases.test_sphere_light_exact(None)


def test_quad_light_exact():
    cases.test_quad_light_exact(None)


def test_overhead_sun_exact():
    cases.test_overhead_sun_exact(None)


@pytest.mark.parametrize("material", ["diffuse", "plastic", "metal"])
def test_mis_direct_agrees_with_bounced(material):
    cases.test_mis_direct_agrees_with_bounced(None, material)


def test_light_through_fog_agrees_with_scattering():
    cases.test_light_through_fog_agrees_with_scattering(None)
