"""raymond_denoise_static: the à-trous denoiser for callers that cannot
allocate device memory while they run (a host that gives the library a fixed
memory budget up front, or a frame loop that must not take cudaMalloc's
device-wide synchronization). It keeps its two intermediate buffers in a
fixed static device array, so it must give exactly what a renderer's own
denoising pass gives on the same accumulated buffers, call after call.

This file is collected last on purpose."""

import ctypes

import numpy as np
import pytest

from raymond_gb300 import Canvas, Renderer, _native, scenes

pytestmark = pytest.mark.gpu


def _static_denoise(r, out_tensor, stream):
    lib = _native.lib()
    bufs = _native.Buffers()
    _native.check(lib.raymond_get_buffers(r.handle, ctypes.byref(bufs)), r.handle)
    rc = lib.raymond_denoise_static(bufs.accum, bufs.guide_albedo, bufs.guide_normal, bufs.width, bufs.height,
                                    r.samples, out_tensor.data_ptr(), stream)
    _native.check(rc)
    _native.check(lib.raymond_sync(r.handle), r.handle)
    return out_tensor.cpu().numpy().reshape(-1)


@pytest.mark.parametrize("width,height", [(64, 64), (100, 37), (512, 512)])
def test_static_denoise_matches_renderer_denoise(gpu, width, height):
    """A square image; one whose sides are no multiple of the kernels' 16×8
    blocks (the scratch's second half starts at width·height, not at a
    rounded size); and one of exactly RAYMOND_DENOISE_STATIC_MAX_PIXELS,
    which the limit check (more pixels than the maximum) must accept."""
    import torch

    scene, camera = scenes.cornell_scene()
    r = Renderer.create(Canvas(width, height))
    r.scene, r.camera = scene, camera
    r.samplesPerFrame = 2
    r.denoise = True
    lib = _native.lib()
    stream = lib.raymond_get_stream(r.handle)
    out = torch.zeros(width * height * 4, dtype=torch.float32, device="cuda:0")
    for call in range(2):  # two calls in a row, the second on a further frame
        r.render()
        r.device.queue.onSubmittedWorkDone()
        expected = r.readPixels(denoised=True)
        got = _static_denoise(r, out, stream)
        assert np.isfinite(got).all()
        scale = np.maximum(np.abs(expected), 1.0)
        assert (np.abs(got - expected) / scale).max() <= 1e-6, call
    r.dispose()


def test_static_denoise_rejects_what_it_cannot_hold(gpu):
    lib = _native.lib()
    limit = 512 * 512
    one = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert lib.raymond_denoise_static(one, one, one, 1024, 1024, 1, one, None) == _native.ECAPACITY
    assert b"static scratch" in lib.raymond_last_error(None)
    assert lib.raymond_denoise_static(None, one, one, 8, 8, 1, one, None) == _native.EINVAL
    assert limit == 262144
