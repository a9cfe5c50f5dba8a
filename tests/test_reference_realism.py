"""tests/unit/realism.test.mjs of the reference, restated: normal maps made
from heights and sampled as plain numbers, materials gaining bumps, glow and
dispersion, volumes kept out of the BVH, the packed material words for
normal maps and emission textures, and — on the oracle's surface frames —
that a normal map leaning right tilts the normal towards increasing u and
one leaning up towards decreasing v, on every kind of primitive."""

import math

import numpy as np
import pytest

import oracle
from raymond_gb300 import NONE, Box, Mat4, Material, Mesh, Quad, Scene, Sphere, Texture, Vec2, Vec3
from fixtures import bump

WHITE = Vec3(1, 1, 1)


def constant_normal_map(n):
    """A 1×1 normal map tilting every normal the same way (realism.test.mjs:12)."""
    return Texture(1, 1, [int(math.floor((c * 0.5 + 0.5) * 255 + 0.5)) for c in (n.x, n.y, n.z)] + [255])


def raycast(scene, origin, direction):
    """Scene.raycast (src/Scene.mjs:255-283) from the oracle's pieces: the
    closest hit in double, its surface frame, the normal map's tilt, and the
    normal turned to face the ray."""
    packed = scene.pack()
    o = np.array(origin.tuple(), dtype=np.float64)
    d = np.array(direction.tuple(), dtype=np.float64)
    r = oracle.raycast(packed, np.concatenate([o, d]).astype(np.float32))
    p = int(r["prim"][0])
    if p == NONE:
        return None
    # The ray as the oracle took it (f32), so the frame is at its own hit.
    o32, d32 = o.astype(np.float32).astype(np.float64), d.astype(np.float32).astype(np.float64)
    t = float(r["t"][0])
    sf = oracle.surface_double(packed, p, o32, d32, t, r["uv"][0, 0], r["uv"][0, 1])
    m = packed.materialList[int(packed.primitives[p * 16 + 1])]
    shading = sf["shading"]
    if m.normalMap is not None:
        su, sv = sf["uv"][0] * m.textureScale.x, sf["uv"][1] * m.textureScale.y
        texel = m.normalMap.sample_many(np.array([su]), np.array([sv]), srgb=False)[0]
        shading = bump(sf["shading"], sf["geometric"], sf["tangent"], sf["up"], texel, m.normalScale)
    facing = shading if sf["geometric"] @ d32 < 0.0 else -shading
    return {"object": int(packed.objectIndex[p]), "point": o32 + d32 * t, "uv": sf["uv"], "normal": facing}


def test_normal_maps_from_heights_tilt_away_from_slopes():
    flat = Texture.normalMap(4, 4, lambda u, v: 0.25)
    assert list(flat.data[:4]) == [128, 128, 255, 255]  # straight out
    i = (32 * 64 + 32) * 4
    right = Texture.normalMap(64, 64, lambda u, v: 0.1 * u)  # rising to the right: leans left
    assert list(right.data[i:i + 3]) == [115, 128, 254]
    down = Texture.normalMap(64, 64, lambda u, v: 0.1 * v)  # rising downwards: leans up
    assert list(down.data[i:i + 3]) == [128, 140, 254]


def test_normal_maps_sample_and_resize_as_plain_numbers():
    t = Texture(1, 1, [64, 128, 255, 255])
    raw = t.sample(0.5, 0.5, False)
    assert abs(raw.x - 64 / 255) <= 1e-9 and abs(raw.y - 128 / 255) <= 1e-9
    assert t.sample(0.5, 0.5).x < 0.06  # as colour it is decoded from sRGB
    assert list(t.resized(2, 2, False).data[:4]) == [64, 128, 255, 255]


def test_materials_gain_bumps_glow_and_dispersion():
    bumps = Texture.normalMap(8, 8, lambda u, v: 0.0)
    pattern = Texture.procedural(2, 2, lambda u, v: WHITE)
    base = Material.plastic(Vec3(0.5, 0.2, 0.1), 0.3).withTexture(pattern, 3, Vec3(0.9, 0.9, 0.9))

    bumpy = base.withNormalMap(bumps, 2)
    assert bumpy.normalMap is bumps and bumpy.normalScale == 2
    assert bumpy.texture is pattern and bumpy.roughness == 0.3 and bumpy.type == "plastic"

    glowing = bumpy.withEmission(Vec3(1, 0.5, 0), 4, pattern)
    assert glowing.emission.tuple() == (4, 2, 0)
    assert glowing.emissionTexture is pattern and glowing.normalMap is bumps
    assert glowing.glows and not glowing.emissive  # glows, but is not a light to aim at
    assert Material.light(WHITE).emissive

    # Crown glass: n_d 1.5168, Abbe number 64.17, so n_F - n_C = 0.00805.
    crown = Material.glass(1.5168, WHITE, 64.17)
    assert abs(crown.iorAt(587.6) - 1.5168) <= 1e-9
    assert abs((crown.iorAt(486.1) - crown.iorAt(656.3)) - (1.5168 - 1) / 64.17) <= 1e-9
    assert crown.iorAt(400) > crown.iorAt(700)
    assert Material.glass(1.5).dispersion == 0


def test_volumes_stay_out_of_the_bvh_after_the_surfaces():
    fog = Material.volume(Vec3(0.9, 0.9, 0.9), 0.5, 0.3)
    floor = Quad(Vec3(-5, 0, 5), Vec3(10, 0, 0), Vec3(0, 0, -10), Material.diffuse(WHITE))
    ball = Sphere(Vec3(0, 1, 0), 1, Material.diffuse(WHITE))
    cloud = Sphere(Vec3(0, 3, 0), 2, fog)
    haze = Box.fromCorners(Vec3(-4, 0, -4), Vec3(4, 3, 4), fog)
    packed = Scene().add(cloud, floor, haze, ball).pack()

    assert packed.primitiveCount == 2  # two surfaces in the BVH
    assert packed.volumes == [2, 3]  # then the volumes
    assert packed.primitives.size == 4 * 16

    f = packed.materials.view(np.float32)
    m = packed.materialList.index(fog) * 24
    assert abs(f[m + 20] - 0.5) <= 1e-6 and abs(f[m + 21] - 0.3) <= 1e-6

    # Rays go through volumes: the raycast sees the ball inside the cloud.
    scene = Scene().add(cloud, ball)
    hit = raycast(scene, Vec3(0, 1, 6), Vec3(0, 0, -1))
    assert hit is not None and scene.objects[hit["object"]] is ball

    for bad in (Mesh.icosphere(fog, 1), Quad(Vec3(0, 0, 0), Vec3(1, 0, 0), Vec3(0, 1, 0), fog)):
        with pytest.raises(Exception, match="Sphere or a Box"):
            Scene().add(bad).pack()


def test_packed_materials_name_their_normal_map_and_emission_texture():
    bumps = Texture.normalMap(8, 8, lambda u, v: 0.0)
    pattern = Texture.procedural(2, 2, lambda u, v: WHITE)
    a = Material.diffuse(WHITE).withTexture(pattern).withNormalMap(bumps, 1.5)
    b = Material.light(WHITE).withEmission(WHITE, 2, pattern)
    packed = Scene().add(Sphere(Vec3(0, 0, 0), 1, a), Sphere(Vec3(3, 0, 0), 1, b)).pack()
    u = packed.materials
    f = u.view(np.float32)

    def at(m):
        return packed.materialList.index(m) * 24

    assert packed.textures == [pattern]  # colour and emission textures share a list
    assert packed.normalMaps == [bumps]
    assert u[at(a) + 16] == 0 and f[at(a) + 17] == np.float32(1.5) and u[at(a) + 18] == NONE
    assert u[at(b) + 16] == NONE and u[at(b) + 18] == 0


SHAPES = {
    "sphere": lambda m: Sphere(Vec3(0, 0, 0), 1, m, rotation=Mat4.rotateZ(0.5).multiplyMat4(Mat4.rotateY(0.8))),
    "quad": lambda m: Quad(Vec3(-1, -1, 0.2), Vec3(2, 0.3, 0), Vec3(-0.2, 2, 0.1), m),
    "box": lambda m: Box(Mat4.rotateY(0.7).multiplyMat4(Mat4.rotateX(0.5)).multiplyMat4(Mat4.scale(1, 0.8, 0.6)), m),
    "torus": lambda m: Mesh.torus(m, radius=0.7, tube=0.3).transformed(Mat4.rotateX(1.1)),
    # One triangle, without texture coordinates and with mirrored ones.
    "triangle": lambda m: Mesh([Vec3(-1.5, -1, 0), Vec3(1.5, -0.8, 0.3), Vec3(-0.2, 1.5, -0.2)], [0, 1, 2], m),
    "mirrored triangle": lambda m: Mesh([Vec3(-1.5, -1, 0), Vec3(1.5, -0.8, 0.3), Vec3(-0.2, 1.5, -0.2)], [0, 1, 2], m,
                                        uvs=[Vec2(1, 1), Vec2(0, 0.9), Vec2(0.6, 0)]),
}


@pytest.mark.parametrize("name", list(SHAPES))
def test_normal_maps_tilt_the_right_way(name):
    make = SHAPES[name]
    plain = Scene().add(make(Material.diffuse(WHITE)))
    right = Scene().add(make(Material.diffuse(WHITE).withNormalMap(constant_normal_map(Vec3(0.6, 0, 0.8)))))
    up = Scene().add(make(Material.diffuse(WHITE).withNormalMap(constant_normal_map(Vec3(0, 0.6, 0.8)))))

    def unit(v):
        return v / np.linalg.norm(v)

    checked = 0
    for ox, oy in ((0, 0), (0.31, 0.12), (-0.25, 0.3), (0.1, -0.35), (-0.4, -0.2), (0.45, 0.4)):
        for origin in (Vec3(0, 0, 5), Vec3(3, 3, 3), Vec3(-4, 1, 2), Vec3(1, -4, 2)):
            target = Vec3(ox, oy, 0)

            def ray(dx, dy):
                return raycast(plain, origin, target.add(Vec3(dx, dy, 0)).subtract(origin))

            h, h1, h2 = ray(0, 0), ray(1e-3, 0), ray(0, 1e-3)
            if not h or not h1 or not h2 or h1["object"] != h["object"] or h2["object"] != h["object"]:
                continue
            # How the point moves with u and v.
            e1, e2 = h1["point"] - h["point"], h2["point"] - h["point"]
            t1, t2 = h1["uv"] - h["uv"], h2["uv"] - h["uv"]
            det = t1[0] * t2[1] - t2[0] * t1[1]
            if abs(det) < 1e-9 or abs(t1[0]) > 0.1 or abs(t2[0]) > 0.1:
                continue  # on a seam
            dpdu = unit((e1 * t2[1] - e2 * t1[1]) / det)
            dpdv = unit((e2 * t1[0] - e1 * t2[0]) / det)

            n = h["normal"]
            lean_right = raycast(right, origin, target.subtract(origin))["normal"] - n
            lean_up = raycast(up, origin, target.subtract(origin))["normal"] - n
            assert np.linalg.norm(lean_right) > 0.3 and unit(lean_right) @ dpdu > 0.8, name
            assert np.linalg.norm(lean_up) > 0.3 and unit(lean_up) @ -dpdv > 0.8, name
            checked += 1
    assert checked >= 4, f"{checked} points checked"
