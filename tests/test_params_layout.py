"""The layouts the reference's tests/unit/shaders.test.mjs pins, restated:
where Renderer.#writeParams puts each uniform (and that the device's Params
struct reads it there), which fields restart the image (the first 168
bytes), where Scene.#pack writes each material field, and the material and
primitive codes on both sides."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from raymond_gb300 import MATERIAL_TYPES, PRIMITIVE_KINDS, Camera, Material, Scene, Sky, Sphere, Vec3
from raymond_gb300.renderer import IMAGE_KEY_BYTES, PARAMS_BYTES, params_block

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "raymond_gb300", "csrc")

# The float or u32 index of each uniform (shaders.test.mjs:56-70).
WRITTEN = {
    "cam_pos": 0, "lens_radius": 3, "cam_right": 4, "tan_half_fov": 7, "cam_up": 8, "focus_distance": 11,
    "cam_forward": 12, "aspect": 15, "sky_zenith": 16, "sun_omc": 19, "sky_horizon": 20, "sun_on": 23,
    "sky_ground": 24, "firefly_clamp": 27, "sun_dir": 28, "light_count": 31, "sun_radiance": 32, "max_bounces": 35,
    "view": 36, "volume_count": 37, "env_strength": 38, "env_rotation": 39, "width": 40, "height": 41,
    "sample_offset": 42, "samples_per_frame": 43, "total_samples": 44, "exposure": 45, "denoise": 46, "caustics": 47,
    "photon_radius": 48, "photon_cell": 49,
}
RESTARTS = ["view", "volume_count", "env_strength", "env_rotation", "width", "height", "max_bounces", "firefly_clamp",
            "lens_radius"]
PER_FRAME = ["sample_offset", "samples_per_frame", "total_samples", "exposure", "denoise"]


def _scene_and_camera():
    scene = Scene(sky=Sky(sunStrength=3.0, sunSize=0.02))
    scene.add(Sphere(Vec3(0, 1, 0), 1.0, Material.diffuse(Vec3(0.5, 0.5, 0.5))))
    camera = Camera(position=Vec3(1.5, 2.5, -7.0), target=Vec3(0, 1, 0), fov=0.7)
    return scene, camera


def test_params_block_puts_each_uniform_at_its_index():
    scene, camera = _scene_and_camera()
    block = params_block(scene, camera, 640, 360, light_count=5, volume_count=2, max_bounces=7, view="depth",
                         firefly_clamp=12.5, samples=24, spp=3, exposure=1.75, denoise=False, caustics=True)
    assert len(block) == PARAMS_BYTES == 208
    f = np.frombuffer(block, dtype=np.float32)
    u = np.frombuffer(block, dtype=np.uint32)
    assert np.allclose(f[WRITTEN["cam_pos"]:WRITTEN["cam_pos"] + 3], [1.5, 2.5, -7.0])
    assert abs(f[WRITTEN["tan_half_fov"]] - np.tan(0.35)) < 1e-6
    assert abs(f[WRITTEN["aspect"]] - 640 / 360) < 1e-6
    assert u[WRITTEN["light_count"]] == 5 and u[WRITTEN["volume_count"]] == 2
    assert u[WRITTEN["max_bounces"]] == 7 and u[WRITTEN["view"]] == 3
    assert f[WRITTEN["firefly_clamp"]] == np.float32(12.5)
    assert (u[WRITTEN["width"]], u[WRITTEN["height"]]) == (640, 360)
    assert (u[WRITTEN["sample_offset"]], u[WRITTEN["samples_per_frame"]], u[WRITTEN["total_samples"]]) == (24, 3, 27)
    assert f[WRITTEN["exposure"]] == np.float32(1.75)
    assert (u[WRITTEN["denoise"]], u[WRITTEN["caustics"]]) == (0, 1)
    assert u[WRITTEN["sun_on"]] == 1
    fwd = f[WRITTEN["cam_forward"]:WRITTEN["cam_forward"] + 3]
    assert abs(np.linalg.norm(fwd) - 1) < 1e-6


def test_restart_key_covers_what_changes_the_image():
    assert IMAGE_KEY_BYTES == 168
    for field in RESTARTS:
        assert WRITTEN[field] * 4 < IMAGE_KEY_BYTES, field
    for field in PER_FRAME:
        assert WRITTEN[field] * 4 >= IMAGE_KEY_BYTES, field
    scene, camera = _scene_and_camera()
    base = params_block(scene, camera, 64, 64)
    # per-frame fields leave the key alone
    assert params_block(scene, camera, 64, 64, samples=8, spp=4, exposure=2.0, denoise=False)[:168] == base[:168]
    # image fields change it
    for kw in ({"max_bounces": 3}, {"view": "normal"}, {"firefly_clamp": 5.0}):
        assert params_block(scene, camera, 64, 64, **kw)[:168] != base[:168], kw
    assert params_block(scene, camera, 64, 32)[:168] != base[:168]


def test_pack_writes_each_material_field_at_its_index():
    """Scene.#pack's material words (shaders.test.mjs:45-51)."""
    m = Material(type="glass", color=Vec3(0.1, 0.2, 0.3), roughness=0.25, ior=1.33, emission=Vec3(1.0, 2.0, 3.0),
                 checker=Vec3(0.4, 0.5, 0.6), checkerSize=0.75, normalScale=0.5, density=2.5, anisotropy=0.3)
    scene = Scene()
    scene.add(Sphere(Vec3(0, 0, 0), 1.0, m))
    packed = scene.pack()
    w = packed.materials.reshape(-1, 24)
    f = w.view(np.float32)
    row = int(packed.primitives.reshape(-1, 16)[0, 1])
    assert np.allclose(f[row, 0:3], [0.1, 0.2, 0.3]) and w[row, 3] == MATERIAL_TYPES["glass"]
    assert np.allclose(f[row, 4:7], [1.0, 2.0, 3.0]) and abs(f[row, 7] - 0.25) < 1e-7
    assert np.allclose(f[row, 8:11], [0.4, 0.5, 0.6]) and abs(f[row, 11] - 0.75) < 1e-7
    assert abs(f[row, 12] - 1.33) < 1e-6
    assert abs(f[row, 17] - 0.5) < 1e-7
    assert abs(f[row, 20] - 2.5) < 1e-7 and abs(f[row, 21] - 0.3) < 1e-7
    NONE = 0xFFFFFFFF
    assert w[row, 13] == NONE and w[row, 16] == NONE and w[row, 18] == NONE  # no textures


DRIVER = r"""
#include <cstddef>
#include <cstdio>
#include "dev_common.cuh"
#define F(name) std::printf(#name " %zu\n", offsetof(rmd::Params, name));
int main() {
    F(cam_pos) F(lens_radius) F(cam_right) F(tan_half_fov) F(cam_up) F(focus_distance) F(cam_forward) F(aspect)
    F(sky_zenith) F(sun_omc) F(sky_horizon) F(sun_on) F(sky_ground) F(firefly_clamp) F(sun_dir) F(light_count)
    F(sun_radiance) F(max_bounces) F(view) F(volume_count) F(env_strength) F(env_rotation) F(width) F(height)
    F(sample_offset) F(samples_per_frame) F(total_samples) F(exposure) F(denoise) F(caustics) F(photon_radius)
    F(photon_cell)
    std::printf("sizeof %zu\n", sizeof(rmd::Params));
    std::printf("SPHERE %u\nQUAD %u\nBOX %u\nTRIANGLE %u\n", rmd::SPHERE, rmd::QUAD, rmd::BOX, rmd::TRIANGLE);
    std::printf("DIFFUSE %u\nMETAL %u\nPLASTIC %u\nGLASS %u\nLIGHT %u\nVOLUME %u\n", rmd::DIFFUSE, rmd::METAL,
                rmd::PLASTIC, rmd::GLASS, rmd::LIGHT, rmd::VOLUME);
    return 0;
}
"""


def test_device_params_struct_and_codes_match(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("no nvcc")
    src = tmp_path / "layout.cu"
    src.write_text(DRIVER)
    exe = tmp_path / "layout"
    subprocess.run([nvcc, "-std=c++17", f"-I{CSRC}", str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {k: int(v) for k, v in (line.split() for line in out.splitlines())}
    for field, index in WRITTEN.items():
        assert got[field] == 4 * index, field
    assert got["sizeof"] == 208
    for kind, code in PRIMITIVE_KINDS.items():
        assert got[kind.upper()] == code
    for mtype, code in MATERIAL_TYPES.items():
        assert got[mtype.upper()] == code
