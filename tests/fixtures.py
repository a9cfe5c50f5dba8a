"""The reference's browser-test scenes (tests/browser/fixture.mjs:35-298)
restated, and trace(): renders one on the GPU through the Renderer and
returns its pixels beside what the oracle's Scene.raycast sees through each
pixel centre (fixture.mjs:311-364)."""

import math

import numpy as np

import oracle
from raymond_gb300 import (Box, Camera, Canvas, EnvironmentMap, Mat4, Material, Mesh, Quad, Renderer, Scene, Sky, Sphere,
                           Texture, Vec2, Vec3)

BLACK = Vec3(0, 0, 0)
WHITE = Vec3(1, 1, 1)
FLOOR_ALBEDO = 0.5


def white_sky():
    return Sky(zenith=Vec3(1, 1, 1), horizon=Vec3(1, 1, 1), ground=Vec3(1, 1, 1))


def floor(material=None):
    m = material or Material.diffuse(Vec3(FLOOR_ALBEDO, FLOOR_ALBEDO, FLOOR_ALBEDO))
    return Quad(Vec3(-20, 0, 20), Vec3(40, 0, 0), Vec3(0, 0, -40), m)


LOOK_DOWN = dict(position=Vec3(0, 4, 4), target=Vec3(0, 0, 0), fov=math.pi / 3)

MATERIALS = {
    "diffuse": Material.diffuse(Vec3(0.7, 0.7, 0.7)),
    "plastic": Material.plastic(Vec3(0.7, 0.2, 0.2), 0.3),
    "metal": Material.metal(Vec3(0.9, 0.8, 0.6), 0.4),
}


def _mixed():
    scene = Scene(sky=Sky.black()).add(
        floor(),
        Sphere(Vec3(-1.2, 0.6, 0), 0.6, Material.diffuse(Vec3(1, 0, 0))),
        Box.fromCorners(Vec3(0.2, 0, -1.4), Vec3(1.2, 1.4, -0.4), Material.metal(Vec3(1, 1, 1), 0.2), 0.6),
        Mesh.torus(Material.plastic(Vec3(0, 0, 1)), radius=0.5, tube=0.2, segments=32, sides=16)
        .transformed(Mat4.translate(0.9, 0.5, 1.0).multiplyMat4(Mat4.rotateX(1.2))),
        Mesh.icosphere(Material.glass(), 1, shading="flat")
        .transformed(Mat4.translate(-0.3, 0.4, 1.4).multiplyMat4(Mat4.scale(0.4, 0.4, 0.4))))
    return scene, dict(position=Vec3(1.5, 3, 4.5), target=Vec3(0, 0.4, 0), fov=math.pi / 3)


def _furnace(material):
    scene = Scene(sky=white_sky()).add(Sphere(Vec3(0, 0, 0), 1, material))
    return scene, dict(position=Vec3(0, 0, 3.2), target=Vec3(0, 0, 0), fov=math.pi / 3)


SCENES = {
    "mixed": lambda arg=None: _mixed(),
    "furnaceDiffuse": lambda arg=None: _furnace(Material.diffuse(Vec3(0.8, 0.8, 0.8))),
    "furnaceGlass": lambda arg=None: _furnace(Material.glass(1.5)),
    "furnaceDispersive": lambda arg=None: _furnace(Material.glass(1.5, WHITE, 20)),
    "furnaceFog": lambda arg=None: _furnace(Material.volume(WHITE, 2.0, 0.5)),
    "sphereLight": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(), Sphere(Vec3(0.5, 1.5, -1), 0.5, Material.light(Vec3(1, 1, 1), 6.0))), LOOK_DOWN),
    "quadLight": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(), Quad(Vec3(-0.5, 1.5, -1.5), Vec3(1.2, 0, 0), Vec3(0, 0, 0.8), Material.light(Vec3(1, 1, 1), 6.0))),
        LOOK_DOWN),
    "sun": lambda arg=None: (Scene(sky=Sky(zenith=BLACK, horizon=BLACK, ground=BLACK, sunStrength=2.0,
                                           sunDirection=Vec3(0, 1, 0), sunSize=0.05)).add(floor()), LOOK_DOWN),
    "lightAsSphere": lambda arg: (Scene(sky=Sky.black()).add(
        floor(MATERIALS[arg]), Sphere(Vec3(0, 1.6, -0.5), 1.0, Material.light(Vec3(1, 1, 1), 2.0))), LOOK_DOWN),
    "lightAsMesh": lambda arg: (Scene(sky=Sky.black()).add(
        floor(MATERIALS[arg]),
        Mesh.icosphere(Material.light(Vec3(1, 1, 1), 2.0), 5).transformed(Mat4.translate(0, 1.6, -0.5))), LOOK_DOWN),
    "room": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(Material.checkered(Vec3(0.8, 0.8, 0.8), Vec3(0.15, 0.15, 0.15), 0.5)),
        Quad(Vec3(-2, 0, -2), Vec3(4, 0, 0), Vec3(0, 3, 0), Material.diffuse(Vec3(0.7, 0.3, 0.2))),
        Sphere(Vec3(-0.6, 0.5, -0.4), 0.5, Material.diffuse(Vec3(0.3, 0.6, 0.9))),
        Box.fromCorners(Vec3(0.2, 0, -0.8), Vec3(1.0, 0.8, 0.0), Material.plastic(Vec3(0.9, 0.9, 0.9), 0.3), 0.4),
        Quad(Vec3(-0.6, 2.5, -0.6), Vec3(1.2, 0, 0), Vec3(0, 0, 1.2), Material.light(Vec3(1, 1, 1), 4.0))),
        dict(position=Vec3(0.5, 2.2, 3.2), target=Vec3(0, 0.4, -0.5), fov=math.pi / 3)),
    "blackSmoke": lambda arg=None: (Scene(sky=white_sky()).add(
        Sphere(Vec3(-0.7, 0, 0), 0.8, Material.volume(BLACK, 1.5)),
        Box(Mat4.translate(0.6, 0, 0).multiplyMat4(Mat4.rotateY(0.6)).multiplyMat4(Mat4.rotateX(0.4))
            .multiplyMat4(Mat4.scale(0.6, 0.5, 0.4)), Material.volume(BLACK, 1.5))),
        dict(position=Vec3(0, 0, 3.2), target=Vec3(0, 0, 0), fov=math.pi / 3)),
    "lampInFog": lambda arg: (Scene(sky=Sky.black()).add(
        floor(),
        Box.fromCorners(Vec3(-3, 0, -3), Vec3(3, 2.5, 2), Material.volume(Vec3(0.9, 0.9, 0.9), 0.5, 0.4)),
        Sphere(Vec3(0, 1.4, -0.5), 0.6, Material.light(WHITE, 3.0)) if arg == "light" else
        Mesh.icosphere(Material.light(WHITE, 3.0), 5).transformed(
            Mat4.translate(0, 1.4, -0.5).multiplyMat4(Mat4.scale(0.6, 0.6, 0.6)))), LOOK_DOWN),
    "stripThroughGlass": lambda arg: (Scene(sky=Sky.black()).add(
        Quad(Vec3(-0.3, -2, -3), Vec3(0.6, 0, 0), Vec3(0, 4, 0), Material.light(WHITE, 1.0)),
        Sphere(Vec3(0, 0, 0), 1, Material.glass(1.5, WHITE, float(arg)))),
        dict(position=Vec3(0, 0, 3.2), target=Vec3(0, 0, 0), fov=math.pi / 3)),
}

def _dark_sun(strength, direction, size):
    return Sky(zenith=BLACK, horizon=BLACK, ground=BLACK, sunStrength=strength, sunDirection=direction, sunSize=size)


CAUSTIC_SCENES = {
    "causticLamp": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(), Sphere(Vec3(0, 0.9, 0), 0.5, Material.glass(1.5)),
        Sphere(Vec3(0.3, 2.6, -0.2), 0.15, Material.light(WHITE, 60.0))), LOOK_DOWN),
    "causticSun": lambda arg=None: (Scene(sky=_dark_sun(2.0, Vec3(0.3, 1, 0.1), 0.03)).add(
        floor(), Sphere(Vec3(0, 0.9, 0), 0.5, Material.glass(1.5))), LOOK_DOWN),
    "causticMirror": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(), Quad(Vec3(-1, 0.2, -1.6), Vec3(2, 0, 0), Vec3(0, 1.2, 0.5), Material.metal(Vec3(0.9, 0.9, 0.9), 0)),
        Quad(Vec3(0.25, 1.4, 1.4), Vec3(-0.5, 0, 0), Vec3(0, 0.5, 0.2), Material.light(WHITE, 30.0))), LOOK_DOWN),
    "causticLampMany": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(), Sphere(Vec3(0, 0.6, 0), 0.4, Material.glass(1.5)),
        Box.fromCorners(Vec3(-0.5, 1.5, -0.5), Vec3(0.5, 1.52, 0.5), Material.glass(1.5)),
        Sphere(Vec3(1.0, 0.35, 0.4), 0.35, Material.glass(1.5)),
        Sphere(Vec3(0.05, 2.6, 0), 0.3, Material.light(WHITE, 15.0))), LOOK_DOWN),
    "causticSunMany": lambda arg=None: (Scene(sky=_dark_sun(1.0, Vec3(0.2, 1, 0.1), 0.2)).add(
        floor(),
        *[Quad(Vec3(x0, 1.6, z0), Vec3(x1 - x0, 0, 0), Vec3(0, 0, z1 - z0), Material.diffuse(BLACK))
          for x0, x1, z0, z1 in ((-20, -1, -20, 20), (1.1, 20, -20, 20), (-1, 1.1, -20, -0.5), (-1, 1.1, 0.5, 20))],
        Box.fromCorners(Vec3(-1, 1.59, -0.5), Vec3(0.05, 1.61, 0.5), Material.glass(1.5)),
        Box.fromCorners(Vec3(0.05, 1.59, -0.5), Vec3(1.1, 1.61, 0.5), Material.glass(1.5)),
        Sphere(Vec3(0.2, 0.5, 0), 0.35, Material.glass(1.5))),
        dict(position=Vec3(0, 1.4, 2.0), target=Vec3(0.1, 0, -0.2), fov=math.pi / 2.5)),
    "causticThroughGlass": lambda arg=None: (Scene(sky=Sky.black()).add(
        floor(), Sphere(Vec3(0, 0.9, 0), 0.5, Material.glass(1.5)),
        Sphere(Vec3(0.3, 2.6, -0.2), 0.3, Material.light(WHITE, 20.0)),
        Box.fromCorners(Vec3(-3, 0, 1.6), Vec3(3, 3.5, 1.62), Material.glass(1.5))),
        dict(position=Vec3(0, 2.4, 2.4), target=Vec3(0, 0, 0), fov=math.pi / 4)),
}
SCENES.update(CAUSTIC_SCENES)

# Textures and the environment of tests/browser/fixture.mjs:13-25 and environment.mjs:7-17.
GRADIENT = Texture.procedural(64, 64, lambda u, v: Vec3(u, v, 0.5 + 0.5 * math.sin(u * 6.28)))
GRID = Texture.procedural(64, 64, lambda u, v: Vec3((math.floor(u * 4) + 1) / 4, (math.floor(v * 4) + 1) / 4,
                                                   ((math.floor(u * 4) + math.floor(v * 4)) % 2) * 0.8 + 0.1))
BUMPS = Texture.normalMap(64, 64, lambda u, v: 0.03 * math.sin(u * math.pi * 4) * math.cos(v * math.pi * 6))
PATTERN = Texture.procedural(64, 64, lambda u, v: Vec3(1 - 0.9 * u, 0.3 + 0.4 * v, 0.1 + 0.9 * u * v))
ENV_SUN = Vec3(0.45, 0.6, -0.66).normalized()


def _env_radiance(d):
    near = d.dot(ENV_SUN)
    c18 = math.cos(0.18)
    sun = 40 * (near - c18) / (1 - c18) + 10 if near > c18 else 0
    sky = 0.2 + 0.6 * max(d.y, 0)
    return Vec3(sky * 0.6 + sun, sky * 0.8 + sun * 0.9, sky + sun * 0.7)


ENVIRONMENT = EnvironmentMap.procedural(128, 64, _env_radiance)
ENV_STRENGTH, ENV_ROTATION = 1.5, 0.7
TEX_CAMERA = dict(position=Vec3(0.8, 2.6, 3.8), target=Vec3(0, 0.4, 0), fov=math.pi / 3)

TEXTURE_SCENES = {
    "textured": lambda arg=None: (Scene(sky=Sky.black()).add(
        Quad(Vec3(-10, 0, 10), Vec3(20, 0, 0), Vec3(0, 0, -20), Material.diffuse(Vec3(1, 1, 1)).withTexture(GRID, 6)),
        Sphere(Vec3(-1.0, 0.7, 0), 0.7, Material.diffuse(Vec3(1, 1, 1)).withTexture(GRADIENT),
               rotation=Mat4.rotateZ(0.4).multiplyMat4(Mat4.rotateY(1.0))),
        Box.fromCorners(Vec3(0.3, 0, -0.9), Vec3(1.3, 1.0, 0.1),
                        Material.plastic(Vec3(1, 0.8, 0.8)).withTexture(GRID, Vec2(1, 2), Vec3(1, 0.8, 0.8)), 0.5),
        Mesh.torus(Material.diffuse(Vec3(1, 1, 1)).withTexture(GRADIENT, 3), radius=0.4, tube=0.18, segments=32,
                   sides=16).transformed(Mat4.translate(0.6, 0.35, 1.0).multiplyMat4(Mat4.rotateX(1.1)))), TEX_CAMERA),
    "bumpy": lambda arg=None: (Scene(sky=Sky.black()).add(
        Quad(Vec3(-10, 0, 10), Vec3(20, 0, 0), Vec3(0, 0, -20),
             Material.diffuse(WHITE).withTexture(GRID, 6).withNormalMap(BUMPS, 1.5)),
        Sphere(Vec3(-1.0, 0.7, 0), 0.7, Material.diffuse(WHITE).withNormalMap(BUMPS, 2),
               rotation=Mat4.rotateZ(0.4).multiplyMat4(Mat4.rotateY(1.0))),
        Box.fromCorners(Vec3(0.3, 0, -0.9), Vec3(1.3, 1.0, 0.1),
                        Material.plastic(WHITE).withTexture(GRID, Vec2(1, 2)).withNormalMap(BUMPS, 2), 0.5),
        Mesh.torus(Material.diffuse(WHITE).withTexture(GRADIENT, 3).withNormalMap(BUMPS, 2), radius=0.4, tube=0.18,
                   segments=32, sides=16).transformed(Mat4.translate(0.6, 0.35, 1.0).multiplyMat4(Mat4.rotateX(1.1)))),
        TEX_CAMERA),
    "patternedLamps": lambda arg=None: (Scene(sky=Sky.black()).add(
        Quad(Vec3(-1.5, -1, 0), Vec3(1.4, 0, 0), Vec3(0, 2, 0), Material.light(WHITE).withEmission(WHITE, 1, PATTERN)),
        Sphere(Vec3(0.8, 0, 0), 0.8, Material.light(WHITE).withEmission(WHITE, 1, PATTERN), rotation=Mat4.rotateY(0.7))),
        dict(position=Vec3(0, 0, 2.6), target=Vec3(0, 0, 0), fov=math.pi / 3)),
    "patternedLamp": lambda arg: (Scene(sky=Sky.black()).add(
        floor(), Quad(Vec3(-1.0, 1.2, -1.5), Vec3(2.0, 0, 0), Vec3(0, 0, 1.4),
                      (Material.light(WHITE) if arg == "light" else Material.diffuse(BLACK)).withEmission(WHITE, 4, PATTERN))),
        LOOK_DOWN),
    "environmentSky": lambda arg=None: (Scene(sky=Sky.environment_sky(ENVIRONMENT, ENV_STRENGTH, ENV_ROTATION)),
                                        dict(position=Vec3(0, 0, 0), target=Vec3(0.3, 0.25, -1), fov=2.2)),
    "environmentFloor": lambda arg=None: (Scene(sky=Sky.environment_sky(ENVIRONMENT, ENV_STRENGTH, ENV_ROTATION)).add(
        floor()), LOOK_DOWN),
}
SCENES.update(TEXTURE_SCENES)


def bump(n, ng, tangent, up, t, strength):
    """Scene.mjs bump(): the shading normal tilted by a normal-map texel."""
    right = tangent - n * (n @ tangent)
    if np.linalg.norm(right) < 1e-9:
        return n
    right = right / np.linalg.norm(right)
    above = np.cross(n, right)
    if above @ up < 0.0:
        above = -above
    tilted = right * ((t[0] * 2 - 1) * strength) + above * ((t[1] * 2 - 1) * strength) + n * (t[2] * 2 - 1)
    tilted = tilted / np.linalg.norm(tilted)
    return tilted if tilted @ ng > 0.0 else n


_renderer = None


def renderer():
    global _renderer
    if _renderer is None:
        _renderer = Renderer.create(Canvas(48, 48))
    return _renderer


def pixel_rays(camera, size):
    rays = np.zeros((size * size, 6), dtype=np.float32)
    for y in range(size):
        for x in range(size):
            r = camera.pixelRay(x, y, size, size)
            rays[y * size + x] = [*r["origin"].tuple(), *r["direction"].tuple()]
    return rays


def pixel_hits(scene, camera, size):
    """The pixel-centre rays and what the oracle's Scene.raycast sees through
    each (fixture.mjs:311-364): per pixel the object index, distance, facing
    normal (normal-mapped), albedo and point, or None."""
    rays = pixel_rays(camera, size)
    packed = scene.pack()
    # Scene.raycast in double on the pixel-centre rays (the rays as doubles, not f32).
    ref = oracle.raycast(packed, rays)
    hits = []
    for i in range(size * size):
        p = int(ref["prim"][i])
        if p == oracle.NONE:
            hits.append(None)
            continue
        m = packed.materialList[int(packed.primitives[p * 16 + 1])]
        normal = ref["normal"][i]
        albedo_ = None
        if m.texture is not None or m.normalMap is not None or m.emissionTexture is not None:
            o, d = rays[i, :3].astype(np.float64), rays[i, 3:].astype(np.float64)
            sf = oracle.surface_double(packed, p, o, d, ref["t"][i], ref["uv"][i, 0], ref["uv"][i, 1])
            su, sv = sf["uv"][0] * m.textureScale.x, sf["uv"][1] * m.textureScale.y
            if m.normalMap is not None:
                t = m.normalMap.sample_many(np.array([su]), np.array([sv]), srgb=False)[0]
                shading = bump(sf["shading"], sf["geometric"], sf["tangent"], sf["up"], t, m.normalScale)
                normal = shading if sf["geometric"] @ d < 0 else -shading
            if m.type == "light":
                e = np.array(m.emission.tuple())
                albedo_ = e * (m.emissionTexture.sample_many(np.array([su]), np.array([sv]))[0]
                               if m.emissionTexture is not None else 1.0)
            elif m.texture is not None:
                albedo_ = np.array(m.color.tuple()) * m.texture.sample_many(np.array([su]), np.array([sv]))[0]
        if albedo_ is None:
            albedo_ = np.array((m.emission if m.type == "light" else m.color).tuple())
        hits.append({"object": int(packed.objectIndex[p]), "distance": float(ref["t"][i]), "normal": normal,
                     "albedo": albedo_, "point": rays[i, :3] + rays[i, 3:] * ref["t"][i]})
    return rays, hits


def oracle_trace(name, arg=None, spp=16, bounces=8, view="color", size=48, denoise=False, caustics=True, seed=0):
    """trace() with the oracle (the trace shader restated, on the CPU) making
    the image instead of the GPU, frame by frame as the renderer does (up
    to 16 samples a frame, no firefly clamp): path tracing (with the
    texture arrays and environment map as uploaded), and when the
    scene has mirrors or glass for light to be focused by and `caustics`
    is on, the same frame's light tracing with its splats and the photon
    map's gather through mirrors and glass (photon radius shrinking frame
    by frame); then the oracle's à-trous denoiser on the guides if asked."""
    from raymond_gb300.renderer import (PHOTON_CAPACITY, delta_objects, emitters_block, environment_arrays,
                                        light_table, params_block, texture_array)

    scene, cam_opts = SCENES[name](arg)
    camera = Camera(**cam_opts)
    packed = scene.pack()
    textures = texture_array(packed.textures, True) if packed.textures else None
    normal_maps = texture_array(packed.normalMaps, False) if packed.normalMaps else None
    env = scene.sky.environment
    environment = None
    if env is not None:
        rgba, table = environment_arrays(env)
        environment = (rgba, env.width, env.height, table)
    words, powers = light_table(packed)
    deltas = delta_objects(scene) if caustics and view == "color" else None
    emitters = emitters_block(powers, len(powers), deltas, scene.sky) if deltas else None
    # The oracle's light tracer and photon map take no textures.
    assert emitters is None or (textures is None and normal_maps is None), name
    acc = np.zeros((size, size, 4), np.float32)
    alb = np.zeros((size, size, 4), np.float32)
    nrm = np.zeros((size, size, 4), np.float32)
    spf = min(spp, 16)
    done = 0
    while done < spp:
        params = params_block(scene, camera, size, size, light_count=len(powers), volume_count=len(packed.volumes),
                              max_bounces=bounces, view=view, firefly_clamp=0.0, samples=done, spp=spf,
                              denoise=False, caustics=emitters is not None, deltas=deltas)
        o = oracle.render(packed, words, params, seed_hash=seed, environment=environment, textures=textures,
                          normal_maps=normal_maps)
        acc += o["accum"]
        alb += o["albedo"]
        nrm += o["normal"]
        if emitters is not None:
            lt = oracle.light_trace(packed, words, params, emitters, min(size * size * spf, PHOTON_CAPACITY),
                                    seed_hash=seed)
            light = lt["splats"][..., :3].astype(np.float32) / np.float32(65536.0)
            lum = light[..., 0] * np.float32(0.2126) + light[..., 1] * np.float32(0.7152) + light[..., 2] * np.float32(0.0722)
            acc[..., :3] += light * np.float32(spf)
            acc[..., 3] += lum * lum * np.float32(spf)
            acc += oracle.photon_gather(packed, words, params, lt["photons"], seed_hash=seed)
        done += spf
    pixels = (acc / done).reshape(-1).astype(np.float32)
    den = oracle.denoise(acc, alb, nrm, size, size, done).reshape(-1) if denoise else None
    rays, hits = pixel_hits(scene, camera, size)
    return {"pixels": pixels, "denoised": den, "hits": hits, "rays": rays, "samples": done, "scene": scene}


def trace(name, arg=None, spp=16, bounces=8, view="color", size=48, denoise=False, caustics=True, seed=0):
    """Renders scene `name` and returns pixels (size²×4), denoised (or None),
    hits (per pixel: object index, distance, normal — or None) and rays."""
    r = renderer()
    r.canvas.width = size
    r.canvas.height = size
    scene, cam_opts = SCENES[name](arg)
    camera = Camera(**cam_opts)
    r.scene = scene
    r.camera = camera
    r.view = view
    r.maxBounces = bounces
    r.fireflyClamp = 0
    r.samplesPerFrame = min(spp, 16)
    r.denoise = denoise
    r.caustics = caustics
    r.reset()
    while r.samples < spp:
        r.render()
    r.device.queue.onSubmittedWorkDone()
    pixels = r.readPixels()
    den = r.readPixels(denoised=True) if denoise else None
    rays, hits = pixel_hits(scene, camera, size)
    return {"pixels": pixels, "denoised": den, "hits": hits, "rays": rays, "samples": r.samples, "scene": scene}


def rgb(pixels, i):
    return pixels[i * 4:i * 4 + 3].astype(np.float64)


def interior(hits, size, obj=None):
    """Pixels whose centre and 4 neighbours see the same object (app.test.mjs:109-124)."""
    keep = []
    for y in range(1, size - 1):
        for x in range(1, size - 1):
            i = y * size + x
            h = hits[i]
            if h is None or (obj is not None and h["object"] != obj):
                continue
            if all(hits[j] is not None and hits[j]["object"] == h["object"] for j in (i - 1, i + 1, i - size, i + size)):
                keep.append(i)
    return keep
