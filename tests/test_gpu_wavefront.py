"""The wavefront path (extend / shade / shadow kernels over queues in HBM,
a frame's samples in two groups on their own streams, shadow rays on side
streams) against the one-kernel path: the same bounce step on the same
sample streams. The wavefront sums a path's shadow-ray light apart from its
own radiance and adds the two at the frame's end, so the accumulated sums
agree to float rounding."""

import numpy as np
import pytest

from raymond_gb300 import Canvas, Renderer, _native, scenes
from fixtures import SCENES
from raymond_gb300 import Camera

pytestmark = pytest.mark.gpu


def frame(scene, camera, size, spp, flags, bounces=8, frames=1, capacity=0):
    r = Renderer.create(Canvas(size, size))
    r.scene, r.camera = scene, camera
    r.maxBounces, r.samplesPerFrame, r.fireflyClamp, r.denoise = bounces, spp, 20.0, False
    r.flags = flags
    for _ in range(frames):
        r.render()
    r.device.queue.onSubmittedWorkDone()
    out = r.readGuides()
    r.dispose()
    return out


@pytest.mark.parametrize("name", ["cornell", "furnaceFog", "stripThroughGlass", "room", "patternedLamp", "textured"])
def test_wavefront_matches_megakernel(gpu, name):
    if name == "cornell":
        scene, camera = scenes.cornell_scene()
    else:
        arg = {"stripThroughGlass": "15", "patternedLamp": "light"}.get(name)
        scene, opts = SCENES[name](arg)
        camera = Camera(**opts)
    mk = frame(scene, camera, 48, 4, _native.FLAG_MEGAKERNEL, frames=2)
    wf = frame(scene, camera, 48, 4, _native.FLAG_WAVEFRONT, frames=2)
    for a, b in zip(mk, wf):
        assert np.isfinite(b).all()
        np.testing.assert_allclose(b, a, rtol=1e-5, atol=1e-6)


def test_wavefront_in_sample_batches(gpu):
    """A path capacity below the frame's paths runs the frame in batches of whole samples."""
    scene, camera = scenes.cornell_scene()
    full = frame(scene, camera, 32, 8, _native.FLAG_WAVEFRONT)
    r = Renderer.create(Canvas(32, 32), seed=0, pathCapacity=3 * 32 * 32)
    r.scene, r.camera = scene, camera
    r.samplesPerFrame, r.fireflyClamp, r.denoise = 8, 20.0, False
    r.flags = _native.FLAG_WAVEFRONT
    r.render()
    r.device.queue.onSubmittedWorkDone()
    np.testing.assert_allclose(r.readGuides()[0], full[0], rtol=1e-5, atol=1e-6)
    r.dispose()


def test_wavefront_sphere_field(gpu):
    scene, camera, info = scenes.sphere_field()
    mk = frame(scene, camera, 128, 2, _native.FLAG_MEGAKERNEL)
    wf = frame(scene, camera, 128, 2, _native.FLAG_WAVEFRONT)
    np.testing.assert_allclose(wf[0], mk[0], rtol=1e-4, atol=1e-5)


def test_autotune_picks_a_working_shape(gpu, tmp_path):
    scene, camera = scenes.cornell_scene()
    r = Renderer.create(Canvas(64, 64))
    r.scene, r.camera = scene, camera
    r.samplesPerFrame = 2
    t = r.autotune(trials=1, cache=str(tmp_path / "t.json"))
    assert t["path"] in (_native.PATH_MEGAKERNEL, _native.PATH_WAVEFRONT)
    assert r.samples == 0
    r.render()
    r.render()
    r.device.queue.onSubmittedWorkDone()
    px = r.readPixels()
    assert np.isfinite(px).all() and px[0::4].mean() > 0
    # The cached answer is reused without timing again.
    r2 = Renderer.create(Canvas(64, 64))
    r2.scene, r2.camera, r2.samplesPerFrame = scene, camera, 2
    assert r2.autotune(trials=1, cache=str(tmp_path / "t.json")) == t
    r.dispose()
    r2.dispose()
