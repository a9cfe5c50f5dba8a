"""Seeded synthetic scenes for the render path's workloads:

* cornell_primary — the unit-cube Cornell box (8 primitives) with one
  jittered primary ray per pixel;
* sphere_field — 10,000 spheres on a 40×40 ground around a displaced,
  smooth-shaded geodesic sphere of 499,280 triangles, under the gradient
  sky and a 0.27° sun.

Random numbers come from mulberry32 (the generator the reference's demo
scenes use, scenes/helpers.mjs:11-20) with the seed recorded."""

from __future__ import annotations

import math

import numpy as np

from .geometry import Box, Mesh, Quad, Sphere
from .material import Material
from .sky import Camera, Sky
from .scene import Scene
from .vec import Vec3


def mulberry32(seed: int):
    """mulberry32: a 32-bit state stepped by 0x6d2b79f5 and mixed; floats in [0, 1)."""
    a = seed & 0xFFFFFFFF

    def imul(x, y):
        return (x * y) & 0xFFFFFFFF

    def nxt():
        nonlocal a
        a = (a + 0x6D2B79F5) & 0xFFFFFFFF
        t = a
        t = imul(t ^ (t >> 15), t | 1)
        t ^= (t + imul(t ^ (t >> 7), t | 61)) & 0xFFFFFFFF
        return ((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296.0

    return nxt


def mulberry32_array(seed: int, n: int) -> np.ndarray:
    """n successive mulberry32 draws, vectorized (same sequence as mulberry32)."""
    a = (np.uint64(seed & 0xFFFFFFFF) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x6D2B79F5)) & np.uint64(0xFFFFFFFF)
    t = a.astype(np.uint32)
    with np.errstate(over="ignore"):
        t = (t ^ (t >> np.uint32(15))) * (t | np.uint32(1))
        t = t ^ (t + (t ^ (t >> np.uint32(7))) * (t | np.uint32(61)))
        t = t ^ (t >> np.uint32(14))
    return t.astype(np.float64) / 4294967296.0


# ---------------------------------------------------------------- C1 ----

def cornell_scene():
    """The unit-cube Cornell room, open at z = 0, lit by a 0.25² lamp (8 primitives)."""
    grey = Material.diffuse(Vec3(0.73, 0.73, 0.73))
    red = Material.diffuse(Vec3(0.65, 0.05, 0.05))
    green = Material.diffuse(Vec3(0.12, 0.45, 0.15))
    lamp = Material.light(Vec3(17.0, 12.0, 4.0))
    scene = Scene(sky=Sky.black())
    scene.add(
        Quad(Vec3(0, 0, 0), Vec3(0, 0, 1), Vec3(1, 0, 0), grey),       # floor, facing up
        Quad(Vec3(0, 1, 0), Vec3(1, 0, 0), Vec3(0, 0, 1), grey),       # ceiling, facing down
        Quad(Vec3(0, 0, 1), Vec3(0, 1, 0), Vec3(1, 0, 0), grey),       # back, facing the camera
        Quad(Vec3(1, 0, 0), Vec3(0, 0, 1), Vec3(0, 1, 0), red),        # left of the image (x = 1)
        Quad(Vec3(0, 0, 0), Vec3(0, 1, 0), Vec3(0, 0, 1), green),      # right of the image (x = 0)
        Quad(Vec3(0.375, 0.999, 0.375), Vec3(0.25, 0, 0), Vec3(0, 0, 0.25), lamp),
        Box.fromCorners(Vec3(0.2, 0.0, 0.5), Vec3(0.5, 0.3, 0.8), grey, math.radians(18.0)),
        Box.fromCorners(Vec3(0.5, 0.0, 0.25), Vec3(0.8, 0.6, 0.55), grey, math.radians(-15.0)),
    )
    camera = Camera(position=Vec3(0.5, 0.5, -1.4), target=Vec3(0.5, 0.5, 0.0), fov=math.radians(40.0))
    return scene, camera


def camera_rays_f32(camera: Camera, width: int, height: int, px: np.ndarray, py: np.ndarray) -> np.ndarray:
    """Pinhole rays through film positions (px, py), in f32 as the trace
    shader's camera_ray computes them (src/shaders.mjs:1148-1157): 6 floats each."""
    b = camera.basis()
    f32 = np.float32
    fwd = np.array(b["forward"].tuple(), dtype=f32)
    right = np.array(b["right"].tuple(), dtype=f32)
    up = np.array(b["up"].tuple(), dtype=f32)
    tan = f32(math.tan(camera.fov / 2.0))
    aspect = f32(width / height)
    ndcx = f32(2.0) * px.astype(f32) / f32(width) - f32(1.0)
    ndcy = f32(1.0) - f32(2.0) * py.astype(f32) / f32(height)
    d = (fwd[None, :] + right[None, :] * (ndcx * tan * aspect)[:, None] + up[None, :] * (ndcy * tan)[:, None])
    d = d.astype(f32)
    d = d / np.sqrt((d * d).sum(axis=1, dtype=f32)).astype(f32)[:, None]
    o = np.broadcast_to(np.array(camera.position.tuple(), dtype=f32), d.shape)
    return np.ascontiguousarray(np.concatenate([o, d], axis=1), dtype=f32)


def cornell_primary(size: int = 256, seed: int = 1):
    """The Cornell scene and one seeded-jitter ray per pixel, row-major,
    jitter (ξ1, ξ2) drawn in that order per pixel from mulberry32(seed)."""
    scene, camera = cornell_scene()
    xi = mulberry32_array(seed, 2 * size * size).reshape(-1, 2)
    ys, xs = np.meshgrid(np.arange(size), np.arange(size), indexing="ij")
    px = xs.reshape(-1) + xi[:, 0]
    py = ys.reshape(-1) + xi[:, 1]
    return scene, camera, camera_rays_f32(camera, size, size, px, py)


# ---------------------------------------------------------------- C2 ----

def _value_noise(points: np.ndarray, seed: int, octaves: int = 4, frequency: float = 2.0) -> np.ndarray:
    """Fractal value noise in [-1, 1]: random lattice values (from mulberry32),
    smoothstep-trilinear interpolation, octaves doubling in frequency and
    halving in amplitude."""
    table = mulberry32_array(seed, 512) * 2.0 - 1.0
    perm = np.argsort(mulberry32_array(seed + 1, 256))

    def lattice(ix, iy, iz):
        h = perm[(perm[(perm[ix & 255] + iy) & 255] + iz) & 255]
        return table[h]

    total = np.zeros(len(points))
    amp, norm, f = 1.0, 0.0, frequency
    for _ in range(octaves):
        p = points * f
        i0 = np.floor(p).astype(np.int64)
        t = p - i0
        s = t * t * (3.0 - 2.0 * t)
        acc = np.zeros(len(points))
        for dx in (0, 1):
            wx = s[:, 0] if dx else 1.0 - s[:, 0]
            for dy in (0, 1):
                wy = s[:, 1] if dy else 1.0 - s[:, 1]
                for dz in (0, 1):
                    wz = s[:, 2] if dz else 1.0 - s[:, 2]
                    acc += wx * wy * wz * lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
        total += amp * acc
        norm += amp
        amp *= 0.5
        f *= 2.0
    return total / norm


def geodesic_sphere(frequency: int):
    """Unit sphere from the icosahedron (the base of Mesh.icosphere,
    src/Mesh.mjs:190-212) with each face split into frequency² triangles,
    vertices projected to the sphere and welded: 20·frequency² triangles."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    base = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
                     (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], dtype=np.float64)
    base /= np.linalg.norm(base, axis=1)[:, None]
    faces = np.array([0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1,
                      8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8,
                      1]).reshape(-1, 3)
    n = frequency
    # Barycentric lattice per face: (i, j) with i + j <= n.
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = (ii + jj) <= n
    ii, jj = ii[keep], jj[keep]
    local = {(int(a), int(b)): k for k, (a, b) in enumerate(zip(ii, jj))}
    tri_local = []
    for i in range(n):
        for j in range(n - i):
            tri_local.append((local[(i, j)], local[(i + 1, j)], local[(i, j + 1)]))
            if i + j + 1 < n:
                tri_local.append((local[(i + 1, j)], local[(i + 1, j + 1)], local[(i, j + 1)]))
    tri_local = np.array(tri_local, dtype=np.int64)
    npts = len(ii)
    pts, tris = [], []
    for f, (a, b, c) in enumerate(faces):
        A, B, C = base[a], base[b], base[c]
        p = A[None, :] + (B - A)[None, :] * (ii / n)[:, None] + (C - A)[None, :] * (jj / n)[:, None]
        p /= np.linalg.norm(p, axis=1)[:, None]
        pts.append(p)
        tris.append(tri_local + f * npts)
    pts = np.concatenate(pts)
    tris = np.concatenate(tris)
    # Weld the copies along shared edges.
    key = np.round(pts * 1e9).astype(np.int64)
    _, first, inverse = np.unique(key, axis=0, return_index=True, return_inverse=True)
    welded = pts[first]
    return welded, inverse.reshape(-1)[tris]


def sphere_field(seed: int = 2, spheres: int = 10000, frequency: int = 158):
    """The sphere-field scene: returns (scene, camera, info). The centre
    mesh has 20·frequency² triangles (499,280 at 158)."""
    rnd = mulberry32(seed)
    scene = Scene(sky=Sky(sunStrength=3.0, sunSize=0.0047124))
    scene.add(Quad(Vec3(-20, 0, 20), Vec3(40, 0, 0), Vec3(0, 0, -40), Material.diffuse(Vec3(0.5, 0.5, 0.5))))
    kinds = {"diffuse": 0, "metal": 0, "glass": 0}
    objs = []
    for _ in range(spheres):
        r = 0.05 + 0.25 * rnd()
        x = -20.0 + 40.0 * rnd()
        z = -20.0 + 40.0 * rnd()
        pick = rnd()
        if pick < 0.60:
            m = Material.diffuse(Vec3(0.1 + 0.8 * rnd(), 0.1 + 0.8 * rnd(), 0.1 + 0.8 * rnd()))
            kinds["diffuse"] += 1
        elif pick < 0.85:
            m = Material.metal(Vec3(0.5 + 0.5 * rnd(), 0.5 + 0.5 * rnd(), 0.5 + 0.5 * rnd()), 0.5 * rnd())
            kinds["metal"] += 1
        else:
            m = Material.glass(1.5)
            kinds["glass"] += 1
        objs.append(Sphere(Vec3(x, r, z), r, m))
    scene.add(*objs)
    pos, idx = geodesic_sphere(frequency)
    disp = 1.0 + 0.1 * _value_noise(pos, seed + 1000)
    radius = 2.0
    centre = np.array([0.0, 2.2, 0.0])
    pos = pos * (disp * radius)[:, None] + centre[None, :]
    mesh = Mesh(pos, idx, Material.plastic(Vec3(0.8, 0.35, 0.2), 0.3))
    scene.add(mesh)
    camera = Camera(position=Vec3(0.0, 4.0, 12.0), target=Vec3(0.0, 1.5, 0.0), fov=math.radians(40.0))
    info = {"seed": seed, "spheres": spheres, "triangles": int(mesh.triangleCount), "materials": kinds,
            "frequency": frequency}
    return scene, camera, info


# ---------------------------------------------------------------- C4 ----

BATCH_RESOLUTIONS = ((256, 256), (512, 512), (960, 540), (1920, 1080))


def batch_instances(count: int = 64, seed: int = 4, spheres: int = 10000):
    """`count` seeded sphere-field instances: triangles log-uniform in
    1k–2M (as 20·f² of a geodesic sphere), a resolution from
    {256², 512², 960×540, 1920×1080} and 1–64 samples per frame each.
    Returns a list of (scene, camera, width, height, spp, info)."""
    rnd = mulberry32(seed)
    out = []
    for i in range(count):
        tris = math.exp(math.log(1000) + rnd() * (math.log(2_000_000) - math.log(1000)))
        freq = max(2, int(round(math.sqrt(tris / 20))))
        w, h = BATCH_RESOLUTIONS[min(3, int(rnd() * 4))]
        spp = 1 + min(63, int(rnd() * 64))
        scene, camera, info = sphere_field(seed=1000 + i, spheres=spheres, frequency=freq)
        info["spp"] = spp
        out.append((scene, camera, w, h, spp, info))
    return out


# ---------------------------------------------------------------- C3 ----

def water_caustics(seed: int = 3, segments: int = 255):
    """The caustics scene: a 2×2 water surface (Mesh.surface with
    segments² cells, 130,050 triangles at 255; ior 1.33) whose height is a
    sum of 8 seeded sinusoids (wavelength U[0.2, 2], amplitude
    U[0.002, 0.02]), a checkered diffuse floor one unit below it, a glass
    sphere (ior 1.5, r = 0.3) on the rim, and one spherical light of
    r = 0.1 above, under a dim sky. Returns (scene, camera, info)."""
    rnd = mulberry32(seed)
    waves = []
    for _ in range(8):
        a = 2.0 * math.pi * rnd()
        lam = 0.2 + 1.8 * rnd()
        amp = 0.002 + 0.018 * rnd()
        phase = 2.0 * math.pi * rnd()
        waves.append((math.cos(a), math.sin(a), 2.0 * math.pi / lam, amp, phase))

    def height(x, z):
        return sum(amp * math.sin(k * (dx * x + dz * z) + ph) for dx, dz, k, amp, ph in waves)

    dim = Vec3(0.02, 0.025, 0.035)
    scene = Scene(sky=Sky(zenith=dim, horizon=dim.scale(1.5), ground=dim.scale(0.5)))
    water = Mesh.surface(lambda u, v: Vec3(-1.0 + 2.0 * u, height(-1.0 + 2.0 * u, -1.0 + 2.0 * v), -1.0 + 2.0 * v),
                         segments, segments, Material.glass(1.33))
    floor = Quad(Vec3(-3.0, -1.0, 3.0), Vec3(6.0, 0.0, 0.0), Vec3(0.0, 0.0, -6.0),
                 Material.checkered(Vec3(0.8, 0.8, 0.75), Vec3(0.25, 0.3, 0.4), 0.25))
    ball = Sphere(Vec3(1.0, 0.3, -0.2), 0.3, Material.glass(1.5))
    lamp = Sphere(Vec3(0.4, 2.5, 0.6), 0.1, Material.light(Vec3(1.0, 0.95, 0.85), 300.0))
    scene.add(floor, water, ball, lamp)
    camera = Camera(position=Vec3(0.0, 2.6, 3.4), target=Vec3(0.0, -0.6, 0.0), fov=math.radians(45.0))
    info = {"seed": seed, "triangles": int(water.triangleCount), "waves": len(waves)}
    return scene, camera, info


# ------------------------------------------------- denoiser training views ----

def training_views(count: int, seed: int = 7, spheres=(300, 3000), frequency=(10, 55)):
    """`count` seeded views for the learned denoiser, alternating
    sphere-field variants (C2's generator with spheres[0]–spheres[1]
    spheres and a centre mesh of frequency[0]–frequency[1], 20·f²
    triangles, seen from a random orbit) and water caustics variants (C3's
    generator with a random camera). Returns a list of (scene, camera,
    info)."""
    rnd = mulberry32(seed)
    out = []
    for i in range(count):
        scene_seed = int(rnd() * 2147483647.0)
        if i % 2 == 0:
            n_spheres = int(spheres[0] + (spheres[1] - spheres[0]) * rnd())
            freq = int(frequency[0] + (frequency[1] - frequency[0]) * rnd())
            scene, camera, info = sphere_field(seed=scene_seed, spheres=n_spheres, frequency=freq)
            az = 2.0 * math.pi * rnd()
            dist = 6.0 + 10.0 * rnd()
            elev = 0.5 + 5.0 * rnd()
            tx, tz = -3.0 + 6.0 * rnd(), -3.0 + 6.0 * rnd()
            camera = Camera(position=Vec3(tx + dist * math.sin(az), elev, tz + dist * math.cos(az)),
                            target=Vec3(tx, 0.3 + 1.5 * rnd(), tz), fov=math.radians(30.0 + 30.0 * rnd()))
        else:
            scene, camera, info = water_caustics(seed=scene_seed, segments=int(40 + 60 * rnd()))
            az = 2.0 * math.pi * rnd()
            dist = 2.5 + 2.0 * rnd()
            camera = Camera(position=Vec3(dist * math.sin(az), 1.2 + 2.0 * rnd(), dist * math.cos(az)),
                            target=Vec3(0.4 * rnd() - 0.2, -0.7, 0.4 * rnd() - 0.2), fov=math.radians(40.0 + 20.0 * rnd()))
        info["view"] = i
        out.append((scene, camera, info))
    return out
