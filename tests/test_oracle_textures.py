"""The reference's texture tests (tests/browser/app.test.mjs:188-240, 482-499)
on the oracle: its path tracer with the texture arrays as the renderer
uploads them — colour textures, normal maps and patterned lamps seen
through every pixel against the CPU's Texture.sample and surface frames,
and a patterned lamp sampled directly against found by bouncing — the
same checks the CUDA path's texture tests make."""

import pytest

import fixtures
import test_gpu_textures as cases


@pytest.fixture(autouse=True)
def on_the_oracle(monkeypatch):
    monkeypatch.setattr(cases, "trace", fixtures.oracle_trace)


def test_textures_match_cpu():
    cases.test_gpu_textures_match_cpu(None)


def test_normal_maps_match_cpu():
    cases.test_gpu_normal_maps_match_cpu(None)


def test_patterned_lamps_match_cpu():
    cases.test_gpu_patterned_lamps_match_cpu(None)


def test_patterned_lamp_direct_agrees_with_bounced():
    cases.test_patterned_lamp_direct_agrees_with_bounced(None)
