"""tests/unit/material.test.mjs of the reference, restated for the Python
mirror: hex colours in linear light, the material factories and clamps,
the sun's radiance over its disc, and Sky's normalisation and copies.
(The reference throws RangeError where the mirror raises ValueError.)"""

import math

import pytest

from raymond_gb300 import Material, Sky, Vec3


def close(a, b, tol=1e-9):
    return abs(a - b) <= tol


def vclose(a, b, tol=1e-9):
    return close(a.x, b.x, tol) and close(a.y, b.y, tol) and close(a.z, b.z, tol)


def test_factories_make_each_type():
    color = Vec3(0.5, 0.25, 1)
    assert Material.diffuse(color).type == "diffuse"
    assert Material.metal(color, 0.3).roughness == 0.3
    assert Material.plastic(color).type == "plastic"
    assert Material.glass(1.33).ior == 1.33
    lamp = Material.light(color, 4)
    assert lamp.emissive is True
    assert vclose(lamp.emission, Vec3(2, 1, 4))
    checker = Material.checkered(color, Vec3(0, 0, 0), 0.5)
    assert checker.checkerSize == 0.5
    assert Material.diffuse(color).checker is None


def test_materials_keep_values_in_range():
    assert Material.metal(Vec3(0, 0, 0), 3).roughness == 1
    assert Material.metal(Vec3(0, 0, 0), -1).roughness == 0
    assert Material.glass(0.5).ior == 1
    assert Material.light(Vec3(1, 1, 1), 0).emissive is False
    with pytest.raises(ValueError):
        Material(type="chrome")


@pytest.mark.parametrize("size", [0.01, 0.05, 0.3])
def test_sun_radiance_over_its_disc_adds_up_to_its_strength(size):
    sky = Sky(sunStrength=3, sunColor=Vec3(1, 0.5, 0.25), sunSize=size)
    # irradiance on a surface facing the sun: radiance × the disc's projected solid angle π sin²(size)
    irradiance = sky.sunRadiance.scale(math.pi * math.sin(size) ** 2)
    expected = 3 * (1 + math.cos(size)) / 2
    assert close(irradiance.x, expected)
    assert close(irradiance.y, expected * 0.5)


def test_sky_normalises_directions():
    sky = Sky(sunDirection=Vec3(0, 10, 0), sunStrength=2)
    assert vclose(sky.sunDirection, Vec3(0, 1, 0))
    black = Sky.black()
    assert vclose(black.horizon, Vec3(0, 0, 0))
    assert black.sunStrength == 0
