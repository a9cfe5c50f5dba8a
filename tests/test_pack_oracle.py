"""The product's packer and host tables against the oracle's independent
restatements of Scene.#pack (oracle/pack.py, src/Scene.mjs:294-539) and of
Renderer's lights buffer, deltaObjects, #writeEmitters and #writeParams
(oracle/host.py, src/Renderer.mjs:571-607, 670-717, 925-991, 1167-1254):
byte for byte on the config scenes, the reference's browser-test fixtures,
and scenes that reach every branch (volumes, rotated spheres, affine
boxes, flat, smooth and textured meshes, the empty scene)."""

import math

import numpy as np
import pytest

import fixtures
import oracle
from oracle import host as ohost
from oracle import pack as opack
from raymond_gb300 import Box, Camera, Mat4, Material, Mesh, Quad, Scene, Sky, Sphere, Texture, Vec2, Vec3, scenes
from raymond_gb300.renderer import delta_objects, emitters_block, light_table, params_block


def same_packed(a, b):
    assert a.primitiveCount == b.primitiveCount
    assert a.nodeCount == b.nodeCount
    for key in ("primitives", "nodes", "materials", "lights"):
        x, y = np.asarray(getattr(a, key)), np.asarray(getattr(b, key))
        assert x.dtype == y.dtype and np.array_equal(x, y), key
    # attributes compared as bits: a NaN-free f32 array either way
    assert np.array_equal(np.asarray(a.attributes, np.float32).view(np.uint32),
                          np.asarray(b.attributes, np.float32).view(np.uint32))
    assert list(a.volumes) == list(b.volumes)
    assert [id(t) for t in a.textures] == [id(t) for t in b.textures]
    assert [id(t) for t in a.normalMaps] == [id(t) for t in b.normalMaps]
    assert [id(m) for m in a.materialList] == [id(m) for m in b.materialList]
    assert [id(o) for o in a.objects] == [id(o) for o in b.objects]


def same_tables(scene, camera, size=(64, 48)):
    """Lights words, powers, delta objects, emitters and the uniform block."""
    packed = scene.pack()
    ref = opack.pack(scene.objects)
    words, powers = light_table(packed)
    owords, opowers = ohost.light_words(ref)
    assert np.array_equal(words, owords)
    assert [(p["prim"], p["power"]) for p in powers] == [(p["prim"], p["power"]) for p in opowers]
    deltas = delta_objects(scene)
    odeltas = ohost.delta_objects(scene.objects, ref)
    assert (deltas is None) == (odeltas is None)
    if deltas:
        assert deltas["centre"].tuple() == odeltas["centre"] and deltas["radius"] == odeltas["radius"]
        assert deltas["reach"] == odeltas["reach"]
        assert [(t["centre"].tuple(), t["radius"]) for t in deltas["targets"]] == \
               [(t["centre"], t["radius"]) for t in odeltas["targets"]]
    em = emitters_block(powers, len(powers), deltas, scene.sky)
    oem = ohost.emitters(opowers, odeltas, scene.sky, len(opowers))
    assert (em is None) == (oem is None)
    if em is not None:
        assert np.array_equal(em.view(np.uint32), oem.view(np.uint32))
    w, h = size
    for kw in (dict(), dict(samples=12, spp=4, view="depth", firefly_clamp=0.0, denoise=False, caustics=True),
               dict(samples=3, spp=1, max_bounces=3, exposure=2.5)):
        a = params_block(scene, camera, w, h, light_count=len(powers), volume_count=len(packed.volumes),
                         deltas=deltas, **kw)
        b = ohost.params(scene, camera, w, h, light_count=len(opowers), volume_count=len(ref.volumes),
                         deltas=odeltas, **kw)
        assert a == b, kw


def branch_scene():
    m = Material.diffuse(Vec3(0.5, 0.6, 0.7))
    tex = Texture.procedural(4, 4, lambda u, v: Vec3(u, v, 0.3))
    bumps = Texture.normalMap(4, 4, lambda u, v: 0.1 * u * v)
    textured = Material.plastic(Vec3(0.3, 0.2, 0.1), 0.4).withTexture(tex, 2.0).withNormalMap(bumps, 0.7)
    glowing = Material.diffuse(Vec3(0.2, 0.2, 0.2)).withEmission(Vec3(1, 0.5, 0.25), 3.0, tex)
    grid = Mesh.surface(lambda u, v: Vec3(u * 2 - 1, 0.1 * math.sin(u * 5) * math.cos(v * 3), v * 2 - 1), 7, 5,
                        textured)
    return Scene(sky=Sky(sunStrength=2.0, sunDirection=Vec3(0.2, 1, 0.3), sunSize=0.02)).add(
        Sphere(Vec3(0.1, 0.2, 0.3), 0.4, Material.glass(1.5, Vec3(1, 0.9, 0.8), 30.0),
               rotation=Mat4.rotateZ(0.3).multiplyMat4(Mat4.rotateX(-0.7))),
        Sphere(Vec3(2, 1, 0), 0.25, Material.light(Vec3(1, 1, 1), 8.0)),
        Quad(Vec3(-1, 2, -1), Vec3(0.5, 0, 0.1), Vec3(0, 0.1, 0.5), Material.light(Vec3(1, 0.8, 0.6), 5.0)),
        Quad(Vec3(-4, 0, 4), Vec3(8, 0, 0), Vec3(0, 0, -8), Material.checkered(Vec3(0.9, 0.9, 0.9),
                                                                             Vec3(0.1, 0.1, 0.1), 0.25)),
        Box(Mat4.translate(0.5, 0.3, -0.2).multiplyMat4(Mat4.rotateY(0.4)).multiplyMat4(Mat4.rotateX(0.2))
            .multiplyMat4(Mat4.scale(0.3, 0.2, 0.5)), Material.metal(Vec3(0.9, 0.8, 0.7), 0.005)),
        Sphere(Vec3(0, 0.5, 0), 1.5, Material.volume(Vec3(0.9, 0.9, 0.9), 0.3, 0.5)),
        Box.fromCorners(Vec3(-3, 0, -3), Vec3(3, 2, 3), Material.volume(Vec3(0.8, 0.8, 0.9), 0.1), 0.2),
        Mesh.icosphere(m, 2).transformed(Mat4.translate(-1.5, 0.6, 0.5)),
        Mesh.icosphere(glowing, 1, shading="flat").transformed(Mat4.translate(1.5, 0.6, 0.5)),
        grid,
        Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], dtype=np.float64), [0, 1, 2, 2, 1, 3], m,
             shading="flat", uvs=[Vec2(0, 0), Vec2(1, 0), Vec2(0, 1), Vec2(1, 1)]),
    ), Camera(position=Vec3(0, 2, 5), target=Vec3(0, 0.5, 0), fov=0.9, aperture=0.05, focusDistance=4.2)


def test_branch_scene_packs_identically():
    scene, camera = branch_scene()
    same_packed(scene.pack(), opack.pack(scene.objects))
    same_tables(scene, camera)


def test_empty_scene_packs_identically():
    scene = Scene()
    a, b = scene.pack(), opack.pack(scene.objects)
    same_packed(a, b)
    assert b.primitives[0] == opack.NONE and b.nodes[7] == 1
    same_tables(scene, Camera())


def test_cornell_packs_identically():
    scene, camera = scenes.cornell_scene()
    same_packed(scene.pack(), opack.pack(scene.objects))
    same_tables(scene, camera, (256, 256))


@pytest.mark.parametrize("name,arg", [(n, a) for n, a in (
    ("mixed", None), ("furnaceFog", None), ("furnaceDispersive", None), ("sphereLight", None), ("quadLight", None),
    ("sun", None), ("lightAsMesh", "metal"), ("room", None), ("blackSmoke", None), ("lampInFog", "light"),
    ("lampInFog", "mesh"), ("stripThroughGlass", "20"), ("causticLamp", None), ("causticSun", None),
    ("causticMirror", None), ("causticLampMany", None), ("causticSunMany", None), ("causticThroughGlass", None),
    ("textured", None), ("bumpy", None), ("patternedLamps", None), ("patternedLamp", "light"), ("patternedLamp", "dark"),
    ("environmentSky", None), ("environmentFloor", None))])
def test_browser_fixtures_pack_identically(name, arg):
    scene, cam = fixtures.SCENES[name](arg)
    same_packed(scene.pack(), opack.pack(scene.objects))
    same_tables(scene, Camera(**cam))


def test_water_caustics_packs_identically():
    scene, camera, _ = scenes.water_caustics()
    same_packed(scene.pack(), opack.pack(scene.objects))
    same_tables(scene, camera, (1024, 1024))


def test_sphere_field_packs_identically():
    """The headline scene: 509,281 primitives, 10,000 materials."""
    scene, camera, _ = scenes.sphere_field()
    same_packed(scene.pack(), opack.pack(scene.objects))
    same_tables(scene, camera, (1024, 1024))
