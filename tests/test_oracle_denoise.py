"""The reference's denoiser tests (tests/browser/app.test.mjs:579-634)
restated on the oracle: its path tracer renders the room, its à-trous
denoiser (the reference's prepare, five passes and compose) filters it.
The CUDA denoiser equals the oracle's on the same input
(test_gpu_image.py), so these answers hold for it too. The errors the
reference's comment quotes (app.test.mjs:595-596: 0.035 noisy at 1 spp,
0.019 denoised) are checked as well."""

import numpy as np
import pytest

from fixtures import interior, oracle_trace

SIZE = 96


def rmse(a, b):
    a, b = a.reshape(-1, 4)[:, :3].astype(np.float64), b.reshape(-1, 4)[:, :3].astype(np.float64)
    return float(np.sqrt(((a - b) ** 2).mean()))


@pytest.fixture(scope="module")
def reference():
    return oracle_trace("room", spp=1024, size=SIZE, bounces=4)


@pytest.mark.parametrize("spp,factor", [(1, 0.6), (4, 0.7)])
def test_denoising_brings_few_samples_closer(reference, spp, factor):
    noisy = oracle_trace("room", spp=spp, size=SIZE, bounces=4, denoise=True)
    before = rmse(noisy["pixels"], reference["pixels"])
    after = rmse(noisy["denoised"], reference["pixels"])
    assert np.isfinite(noisy["denoised"]).all()
    assert after < before * factor, (spp, before, after)
    if spp == 1:
        assert abs(before - 0.035) < 0.004 and abs(after - 0.019) < 0.003, (before, after)


def test_denoising_keeps_the_checkerboard_edges(reference):
    noisy = oracle_trace("room", spp=4, size=SIZE, bounces=4, denoise=True)
    floor = interior(reference["hits"], SIZE, 0)
    ref = reference["pixels"].reshape(-1, 4)[:, :3].astype(np.float64)

    def error(pixels):
        p = pixels.reshape(-1, 4)[:, :3].astype(np.float64)
        return float(np.sqrt(np.mean([np.mean((p[i] - ref[i]) ** 2) for i in floor])))

    assert len(floor) > 1000
    assert error(noisy["denoised"]) < error(noisy["pixels"])


def test_denoised_image_becomes_the_average():
    r = oracle_trace("room", spp=512, size=32, bounces=4, denoise=True)
    difference = rmse(r["pixels"], r["denoised"])
    rgb = r["pixels"].reshape(-1, 4)[:, :3].astype(np.float64)
    brightness = float(np.sqrt((rgb ** 2).mean()))
    assert difference < 0.05 * brightness, (difference, brightness)
