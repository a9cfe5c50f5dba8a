"""Texture arrays and the environment map built on the GPU
(raymond_upload_texture_images, raymond_upload_environment_rgb) equal the
host's restatements of the reference's upload, bit for bit: every layer
resampled as Texture.resized does (src/Texture.mjs:193-209) into an array of
the largest texture's size (src/Renderer.mjs:637-661), the half floats of
toHalf (src/Renderer.mjs:1143-1160) and the importance table
(src/EnvironmentMap.mjs:202-247). Integer and byte results: no tolerance."""

import ctypes

import numpy as np
import pytest

from raymond_gb300 import Canvas, EnvironmentMap, Renderer, Texture, _native
from raymond_gb300.renderer import byte_decoding, environment_arrays, table_row_sines, texture_array

pytestmark = pytest.mark.gpu


def random_texture(rng, w, h):
    return Texture(w, h, rng.integers(0, 256, size=w * h * 4, dtype=np.uint8))


def gpu_array(r, which, textures, srgb):
    images = [np.ascontiguousarray(t.data, dtype=np.uint8) for t in textures]
    ptrs = (ctypes.c_void_p * len(images))(*[_native.ptr(a) for a in images])
    widths = np.array([t.width for t in textures], dtype=np.uint32)
    heights = np.array([t.height for t in textures], dtype=np.uint32)
    decode = np.ascontiguousarray(byte_decoding(srgb), dtype=np.float64)
    lib = _native.lib()
    _native.check(lib.raymond_upload_texture_images(r.handle, which, ptrs, _native.ptr(widths), _native.ptr(heights),
                                                    len(images), 1 if srgb else 0, _native.ptr(decode)), r.handle)
    w, h = min(2048, int(widths.max())), min(2048, int(heights.max()))
    out = np.zeros(w * h * 4 * len(images), dtype=np.uint8)
    _native.check(lib.raymond_read_textures(r.handle, which, _native.ptr(out), out.nbytes), r.handle)
    return out, w, h


@pytest.mark.parametrize("srgb", [True, False], ids=["colour", "normal_maps"])
@pytest.mark.parametrize("sizes", [[(64, 64), (100, 37), (256, 128), (17, 300)], [(2500, 40), (1024, 1024), (3, 2)]],
                         ids=["mixed", "capped_at_2048"])
def test_texture_array_equals_the_host_resize(gpu, srgb, sizes):
    rng = np.random.default_rng(len(sizes) + srgb)
    textures = [random_texture(rng, w, h) for w, h in sizes]
    r = Renderer.create(Canvas(8, 8))
    got, w, h = gpu_array(r, 0 if srgb else 1, textures, srgb)
    r.dispose()
    want, ww, wh = texture_array(textures, srgb)
    assert (w, h) == (ww, wh)
    diff = np.nonzero(got != want)[0]
    assert diff.size == 0, (diff[:10], got[diff[:10]], want[diff[:10]])


def random_environment(rng, w, h):
    """HDR values over the half float's whole range: zeros, subnormal halves,
    exact powers of two and values just under them, ordinary skies, and
    values past 65504 that saturate."""
    n = w * h * 3
    v = np.exp(rng.uniform(np.log(1e-9), np.log(2e5), n)).astype(np.float32)
    k = rng.integers(0, 8, n)
    v[k == 0] = 0.0
    v[k == 1] = np.float32(2.0) ** rng.integers(-20, 17, int((k == 1).sum())).astype(np.float32)
    v[k == 2] = np.nextafter(np.float32(2.0) ** rng.integers(-20, 17, int((k == 2).sum())).astype(np.float32),
                             np.float32(0))
    v[k == 3] = rng.uniform(0, 6.2e-5, int((k == 3).sum()))
    return EnvironmentMap(w, h, v)


@pytest.mark.parametrize("size", [(64, 32), (600, 300), (2048, 1024), (513, 7)])
def test_environment_equals_the_host_tables(gpu, size):
    w, h = size
    env = random_environment(np.random.default_rng(w + h), w, h)
    r = Renderer.create(Canvas(8, 8))
    lib = _native.lib()
    rgb = np.ascontiguousarray(env.data, dtype=np.float32)
    sines = np.ascontiguousarray(table_row_sines(w, h), dtype=np.float64)
    _native.check(lib.raymond_upload_environment_rgb(r.handle, _native.ptr(rgb), w, h, _native.ptr(sines), len(sines)),
                  r.handle)
    want_rgba, want_table = environment_arrays(env)
    rgba = np.zeros(w * h * 4, dtype=np.uint16)
    table = np.zeros(want_table["width"] * (want_table["height"] + 1), dtype=np.float32)
    _native.check(lib.raymond_read_environment(r.handle, _native.ptr(rgba), rgba.nbytes, _native.ptr(table),
                                               table.nbytes), r.handle)
    r.dispose()
    bad = np.nonzero(rgba != want_rgba.reshape(-1))[0]
    assert bad.size == 0, (bad[:5], rgba[bad[:5]], want_rgba.reshape(-1)[bad[:5]], rgb[(bad[:5] // 4) * 3])
    bad = np.nonzero(table.view(np.uint32) != want_table["data"].view(np.uint32))[0]
    assert bad.size == 0, (bad[:5], table[bad[:5]], want_table["data"][bad[:5]])


def test_upload_checks_its_arguments(gpu):
    r = Renderer.create(Canvas(8, 8))
    lib = _native.lib()
    sines = np.zeros(3, dtype=np.float64)
    rgb = np.zeros(64 * 32 * 3, dtype=np.float32)
    # 64 × 32 has 32 rows of cells, not 3
    assert lib.raymond_upload_environment_rgb(r.handle, _native.ptr(rgb), 64, 32, _native.ptr(sines), 3) == \
        _native.EINVAL
    assert lib.raymond_read_textures(r.handle, 2, None, 0) == _native.EINVAL
    r.dispose()
