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


def test_textured_and_environment_frames_are_the_same_on_any_number_of_threads():
    """Every sample draws from its own hashed streams: the oracle's frames
    with texture arrays, normal maps and an environment map do not depend
    on how the pixels are shared out."""
    import numpy as np

    import oracle
    from raymond_gb300 import Camera
    from raymond_gb300.renderer import environment_arrays, light_table, params_block, texture_array

    for name in ("bumpy", "environmentFloor"):
        scene, cam = fixtures.SCENES[name](None)
        camera = Camera(**cam)
        packed = scene.pack()
        words, powers = light_table(packed)
        params = params_block(scene, camera, 24, 24, light_count=len(powers), max_bounces=4, spp=4)
        kw = {}
        if packed.textures:
            kw["textures"] = texture_array(packed.textures, True)
        if packed.normalMaps:
            kw["normal_maps"] = texture_array(packed.normalMaps, False)
        if scene.sky.environment is not None:
            env = scene.sky.environment
            rgba, table = environment_arrays(env)
            kw["environment"] = (rgba, env.width, env.height, table)
        one = oracle.render(packed, words, params, nthreads=1, **kw)
        many = oracle.render(packed, words, params, nthreads=5, **kw)
        for key in ("accum", "albedo", "normal"):
            assert np.array_equal(one[key].view(np.uint32), many[key].view(np.uint32)), (name, key)
        assert one["albedo"][..., :3].sum() > 0, name  # (the bumpy scene is unlit: its colour is black)
