"""What the trained network gains over the method without it: on views it
was not trained on (sphere-field and water-caustics variants from another
seed), the learned denoiser's displayed image is closer to the converged
render than the à-trous filter's at the same sample count, through the
public Renderer API (Renderer.learnedDenoiser → raymond_denoise_learned).
The network only filters the display: the running average is bit-identical
with and without it."""

import os

import numpy as np
import pytest

from raymond_gb300 import Canvas, Renderer, scenes
from raymond_gb300.denoiser import DEFAULT_WEIGHTS, Denoiser

pytestmark = pytest.mark.gpu

SIZE = 256


def rmse(a, b):
    d = np.asarray(a, np.float64).reshape(-1, 4)[:, :3] - np.asarray(b, np.float64).reshape(-1, 4)[:, :3]
    return float(np.sqrt(np.mean(d * d)))


def _render(scene, camera, spp, seed=0, net=None, denoise=True):
    r = Renderer.create(Canvas(SIZE, SIZE), seed=seed)
    r.scene, r.camera = scene, camera
    r.caustics = False
    r.denoise = denoise
    r.learnedDenoiser = net
    r.samplesPerFrame = min(spp, 64)
    for _ in range(max(1, spp // 64)):
        r.render()
    out = (r.readPixels(), r.readPixels(denoised=True) if denoise else None, r.readDisplay())
    if net is not None:
        # filtering again leaves the running average as it was
        r._denoise_learned()
        assert np.array_equal(r.readPixels(), out[0])
    r.dispose()
    return out


@pytest.fixture(scope="module")
def net(gpu):
    if not os.path.exists(DEFAULT_WEIGHTS):
        pytest.fail(f"{DEFAULT_WEIGHTS} is missing: train it with python -m raymond_gb300.train_denoiser")
    d = Denoiser(weights=DEFAULT_WEIGHTS)
    yield d
    d.dispose()


def test_learned_beats_atrous_on_unseen_views(net):
    views = scenes.training_views(4, seed=99)
    rows = []
    for scene, camera, info in views:
        target = _render(scene, camera, 1024, denoise=False)[0]
        plain, atrous, _ = _render(scene, camera, 4, seed=0x5BD1E995)
        plain2, learned, display = _render(scene, camera, 4, seed=0x5BD1E995, net=net)
        # display only: the running average is the same with the network on
        np.testing.assert_allclose(plain2, plain, rtol=1e-5, atol=1e-6)
        assert np.isfinite(learned).all()
        assert display.shape == (SIZE, SIZE, 4) and display[..., :3].max() > 0
        rows.append((rmse(plain, target), rmse(atrous, target), rmse(learned, target)))
    rows = np.array(rows)
    noisy, atr, lrn = rows.mean(axis=0)
    print(f"4 spp RMSE over {len(rows)} unseen views: noisy {noisy:.4f}, à-trous {atr:.4f}, learned {lrn:.4f}")
    assert lrn < 0.85 * atr, rows
    assert lrn < 0.5 * noisy, rows
