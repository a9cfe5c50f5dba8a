"""The reference's environment-map tests (tests/browser/app.test.mjs:353-410)
on the oracle: its path tracer under the environment map as the renderer
uploads it (half floats and the importance table) sees the CPU's
EnvironmentMap.sample through every pixel, and lights a floor with the
exact irradiance — the same checks the CUDA path's tests make."""

import pytest

import fixtures
import test_gpu_textures as cases


@pytest.fixture(autouse=True)
def on_the_oracle(monkeypatch):
    monkeypatch.setattr(cases, "trace", fixtures.oracle_trace)


def test_environment_matches_cpu():
    cases.test_gpu_environment_matches_cpu(None)


def test_environment_light_matches_exact():
    cases.test_environment_light_matches_exact(None)
