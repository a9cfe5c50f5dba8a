"""tests/unit/environment.test.mjs:9-85 of the reference, restated: the
equirectangular layout (directions round the horizon from -z, down from
straight up), procedural maps at pixel centres, the constructor's checks,
and Radiance .hdr files read back flat and run-length encoded. (The
importance table and the sky's radiance, environment.test.mjs:87-127, are
restated in test_reference_textures.py.)"""

import math

import numpy as np
import pytest

from raymond_gb300 import EnvironmentMap, Vec3


def test_directions_and_texture_coordinates():
    d = EnvironmentMap.direction(0.5, 0.5)
    assert np.allclose(d.tuple(), (0, 0, -1), atol=1e-12)  # the middle is ahead
    d = EnvironmentMap.direction(0.75, 0.5)
    assert np.allclose(d.tuple(), (1, 0, 0), atol=1e-12)  # three quarters is +x
    assert abs(EnvironmentMap.direction(0.3, 0).y - 1) <= 1e-12
    assert abs(EnvironmentMap.direction(0.3, 1).y + 1) <= 1e-12
    for u, v in ((0.1, 0.2), (0.6, 0.7), (0.95, 0.4)):
        u2, v2 = EnvironmentMap.uv(EnvironmentMap.direction(u, v))
        assert abs(u2 - u) <= 1e-12 and abs(v2 - v) <= 1e-12


def test_procedural_maps_take_pixel_centres():
    env = EnvironmentMap.procedural(64, 32, lambda d: Vec3(d.y + 1, 0, 0))
    assert abs(env.data[0] - (math.cos(math.pi / 64) + 1)) <= 1e-6  # the top row is half a pixel down
    assert abs(env.sample(Vec3(0, 0, -1)).x - 1) <= 0.02
    with pytest.raises(ValueError):
        EnvironmentMap(2, 2, [1, 2, 3])
    assert list(EnvironmentMap(1, 1, [-1, float("nan"), 2]).data) == [0, 0, 2]  # negative and broken values dropped


def encode_hdr(width, height, pixels, rle):
    """A Radiance .hdr file of pixels(x, y) (environment.test.mjs:31-64): a
    header, then each row flat or, run-length encoded, as each channel's
    first value run three times and the rest as literals of up to 100."""
    out = bytearray(f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {height} +X {width}\n".encode())

    def rgbe(r, g, b):
        m = max(r, g, b)
        if m < 1e-32:
            return [0, 0, 0, 0]
        e = math.ceil(math.log2(m) + 1e-9)
        scale = 256 / 2 ** e
        return [math.floor(x) for x in (r * scale, g * scale, b * scale, e + 128)]

    for y in range(height):
        row = [rgbe(*pixels(x, y)) for x in range(width)]
        if not rle:
            out += bytes(c for p in row for c in p)
            continue
        out += bytes([2, 2, width >> 8, width & 255])
        for c in range(4):
            values = [p[c] for p in row]
            out += bytes([128 + 3, values[0]])
            for x in range(3, width, 100):
                chunk = values[x:min(x + 100, width)]
                out += bytes([len(chunk), *chunk])
    return bytes(out)


def pixels(x, y):
    # The first three pixels of each row match, for the run.
    return (0.5, 1, 2) if x < 3 else (x * 0.25, y * 3, 100 + x)


@pytest.mark.parametrize("rle", [False, True])
def test_radiance_files_read_back(rle, tmp_path):
    file = encode_hdr(16, 4, pixels, rle)
    path = tmp_path / "sky.hdr"
    path.write_bytes(file)
    for env in (EnvironmentMap.fromHDR(file), EnvironmentMap.fromHDR(np.frombuffer(file, np.uint8)),
                EnvironmentMap.load(path)):
        assert (env.width, env.height) == (16, 4)
        for x, y in ((0, 0), (2, 3), (5, 1), (15, 3)):
            expected = pixels(x, y)
            # RGBE shares one exponent across a pixel: each channel to 1/128 of the brightest.
            for c in range(3):
                assert abs(env.data[(y * 16 + x) * 3 + c] - expected[c]) <= max(expected) / 128


def test_radiance_files_refused():
    with pytest.raises(ValueError, match="Not a Radiance"):
        EnvironmentMap.fromHDR(b"P6\n1 1\n255\n")
    with pytest.raises(ValueError, match="top to bottom"):
        EnvironmentMap.fromHDR(b"#?RADIANCE\n\n+Y 1 +X 1\n")
    with pytest.raises(ValueError, match="Unsupported"):
        EnvironmentMap.fromHDR(b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 1\n")
    with pytest.raises(ValueError, match="ends in its header"):
        EnvironmentMap.fromHDR(b"#?RADIANCE\nEXPOSURE=1")
    with pytest.raises(ValueError, match="ends early"):
        EnvironmentMap.fromHDR(b"#?RADIANCE\n\n-Y 2 +X 2\n" + bytes(8))
    good = encode_hdr(16, 1, pixels, True)
    with pytest.raises(ValueError, match="runs over"):
        EnvironmentMap.fromHDR(good[:-5])  # the last channel's literal cut short
    wrong = bytearray(good)
    wrong[good.index(bytes([2, 2, 0, 16])) + 3] = 17
    with pytest.raises(ValueError, match="wrong length"):
        EnvironmentMap.fromHDR(bytes(wrong))


def test_zero_exponent_is_black_and_exponents_scale():
    header = b"#?RGBE\n\n-Y 1 +X 2\n"
    env = EnvironmentMap.fromHDR(header + bytes([200, 100, 50, 0, 128, 64, 32, 129]))
    assert list(env.data[:3]) == [0, 0, 0]
    # 2^(129-136) = 1/128
    assert list(env.data[3:]) == [1.0, 0.5, 0.25]
