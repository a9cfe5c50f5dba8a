"""Batched frames (raymond_render_batch) against each renderer rendering on
its own: the same sample streams and bounce step, so every job's
accumulated image agrees — replayed as a CUDA graph over several frames,
with the shared path pool split into waves, and with the denoiser and tone
map run over all jobs at once."""

import numpy as np
import pytest

from fixtures import SCENES
from raymond_gb300 import BatchRenderer, Camera, Canvas, Renderer, _native, scenes

pytestmark = pytest.mark.gpu


def make_jobs():
    out = []
    specs = [("cornell", 48, 4), ("room", 32, 2), ("furnaceGlass", 24, 8), ("stripThroughGlass", 40, 1),
             ("furnaceFog", 16, 3)]
    for name, size, spp in specs:
        if name == "cornell":
            scene, camera = scenes.cornell_scene()
        else:
            scene, opts = SCENES[name]("15" if name == "stripThroughGlass" else None)
            camera = Camera(**opts)
        out.append((scene, camera, size, spp))
    return out


def renderers(specs):
    rs = []
    for scene, camera, size, spp in specs:
        r = Renderer.create(Canvas(size, size))
        r.scene, r.camera = scene, camera
        r.samplesPerFrame, r.fireflyClamp, r.caustics = spp, 20.0, False
        r.flags = _native.FLAG_WAVEFRONT
        rs.append(r)
    return rs


@pytest.mark.parametrize("graph,capacity", [(True, 0), (False, 0), (True, 3000)])
def test_batch_matches_single_renderers(gpu, graph, capacity):
    specs = make_jobs()
    alone = renderers(specs)
    for _ in range(3):
        for r in alone:
            r.render()
    expected = [r.readGuides() for r in alone]
    den_expected = [r.readPixels(denoised=True) for r in alone]

    batched = renderers(specs)
    batch = BatchRenderer(graph=graph, pathCapacity=capacity)
    for _ in range(3):
        batch.render(batched)
    batch.sync()
    for r, e, de in zip(batched, expected, den_expected):
        got = r.readGuides()
        for a, b in zip(got, e):
            assert np.isfinite(a).all()
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(r.readPixels(denoised=True), de, rtol=1e-4, atol=1e-5)
        assert r.samples == 3 * r.samplesPerFrame
    for r in alone + batched:
        r.dispose()
    batch.dispose()


def test_batch_rejects_bad_jobs(gpu):
    batch = BatchRenderer()
    r = Renderer.create(Canvas(8, 8))
    with pytest.raises(ValueError):
        batch.render([r])  # no scene
    r.dispose()
    batch.dispose()
