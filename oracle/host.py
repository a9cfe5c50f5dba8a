"""The renderer's host tables restated (src/Renderer.mjs) — TEST
INFRASTRUCTURE ONLY.

What Renderer computes on the host from a packed scene before the shaders
run, restated independently of the product so that its tables are checked
and the bench's reference arm needs nothing of the product:

* the lights buffer: light primitives, volume primitives, then each
  light's running next-event chance as f32 bits, the last forced to 1
  (src/Renderer.mjs:571-607), with the chances of `lightChances`
  (:1167-1179) and each light's power (luminance · π · area, :588-594);
* `deltaObjects`: the mirrors and glass light tracing aims at, split into
  at most 16 target spheres (:1187-1254, `boxAround` and `radius` :1258-1273);
* `#writeEmitters`: the light-tracing sources and targets (:670-717);
* `#writeParams`: the 208-byte uniform block (:925-991), with the camera's
  basis from `Mat4.lookAt` (src/Camera.mjs:115-123, src/Mat4.mjs:307-318)
  and the sun's radiance (src/Sky.mjs:132-136).

Scene objects, camera and sky are read by their fields, as in pack.py."""

from __future__ import annotations

import math

import numpy as np

from .pack import NONE, box_corners

VIEWS = {"color": 0, "albedo": 1, "normal": 2, "depth": 3}
UNIFORM_SHARE = 0.25
MAX_TARGETS = 16


def _v(p):
    return (float(p.x), float(p.y), float(p.z))


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _length(a):
    return math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])


def _normalized(a):
    n = _length(a)
    return (a[0] / n, a[1] / n, a[2] / n)


def light_chances(powers):
    total = 0.0
    for p in powers:
        total += p
    n = len(powers)
    if not (total > 0) or not math.isfinite(total):
        return [1 / n for _ in powers]
    return [UNIFORM_SHARE / n + (1 - UNIFORM_SHARE) * p / total for p in powers]


def light_powers(packed):
    """Each light's primitive and power: luminance of its emission × π × its area."""
    lights = [] if int(packed.lights[0]) == NONE else [int(x) for x in packed.lights]
    pu = np.asarray(packed.primitives, dtype=np.uint32)
    pf = pu.view(np.float32)
    mf = np.asarray(packed.materials, dtype=np.uint32).view(np.float32)
    out = []
    for prim in lights:
        b, m = prim * 16, int(pu[prim * 16 + 1]) * 24
        lum = 0.2126 * float(mf[m + 4]) + 0.7152 * float(mf[m + 5]) + 0.0722 * float(mf[m + 6])
        if int(pu[b]) == 1:  # a quad: |u × v|
            u = (float(pf[b + 8]), float(pf[b + 9]), float(pf[b + 10]))
            v = (float(pf[b + 12]), float(pf[b + 13]), float(pf[b + 14]))
            area = _length(_cross(u, v))
        else:
            area = 4 * math.pi * float(pf[b + 7]) ** 2
        out.append({"prim": prim, "power": lum * math.pi * area})
    return out


def light_words(packed):
    """The lights-and-volumes buffer's u32 words, and the lights' powers."""
    powers = light_powers(packed)
    chances = light_chances([p["power"] for p in powers])
    running, cumulative = 0.0, []
    for c in chances:
        running += c
        cumulative.append(running)
    cum = np.array(cumulative, dtype=np.float32)
    if cum.size:
        cum[-1] = 1.0
    words = [p["prim"] for p in powers] + [int(v) for v in packed.volumes] + [int(w) for w in cum.view(np.uint32)]
    return np.array(words if words else [NONE], dtype=np.uint32), powers


def _box_around(points):
    mn = [math.inf] * 3
    mx = [-math.inf] * 3
    for p in points:
        for a in range(3):
            mn[a] = min(mn[a], p[a])
            mx[a] = max(mx[a], p[a])
    return {"min": mn, "max": mx}


def _radius(box):
    return math.hypot(box["max"][0] - box["min"][0], box["max"][1] - box["min"][1], box["max"][2] - box["min"][2]) / 2


def _sphere_around(box):
    return {"centre": ((box["min"][0] + box["max"][0]) / 2, (box["min"][1] + box["max"][1]) / 2,
                       (box["min"][2] + box["max"][2]) / 2),
            "radius": max(_radius(box), 1e-3) * 1.001}


def delta_objects(objects, packed):
    """deltaObjects (src/Renderer.mjs:1187-1254), or None with no mirror or glass."""
    boxes = []
    for obj in objects:
        m = obj.material
        if not (m.type == "glass" or (m.type == "metal" and m.roughness < 0.01)):
            continue
        if hasattr(obj, "indices"):
            pts = [tuple(float(c) for c in p) for p in np.asarray(obj.positions, dtype=np.float64).reshape(-1, 3)]
        elif hasattr(obj, "transform"):
            pts = box_corners(obj.transform)
        elif hasattr(obj, "corner"):
            c, u, v = _v(obj.corner), _v(obj.u), _v(obj.v)
            cu = (c[0] + u[0], c[1] + u[1], c[2] + u[2])
            pts = [c, cu, (c[0] + v[0], c[1] + v[1], c[2] + v[2]), (cu[0] + v[0], cu[1] + v[1], cu[2] + v[2])]
        else:
            c, r = _v(obj.center), float(obj.radius)
            pts = [(c[0] - r, c[1] - r, c[2] - r), (c[0] + r, c[1] + r, c[2] + r)]
        box = _box_around(pts)
        box["centre"] = [(box["min"][a] + box["max"][a]) / 2 for a in range(3)]
        boxes.append(box)
    if not boxes:
        return None
    groups = [boxes]
    while len(groups) < MAX_TARGETS:
        biggest, size = -1, 0
        for i, g in enumerate(groups):
            s = _radius(_box_around([x for b in g for x in (b["min"], b["max"])])) if len(g) > 1 else 0
            if s > size:
                biggest, size = i, s
        if biggest < 0:
            break
        group = groups[biggest]
        spread = _box_around([b["centre"] for b in group])
        extent = [spread["max"][a] - spread["min"][a] for a in range(3)]
        axis = extent.index(max(extent))
        group = sorted(group, key=lambda b: b["centre"][axis])
        half = len(group) >> 1
        groups[biggest:biggest + 1] = [group[:half], group[half:]]
    targets = [_sphere_around(_box_around([x for b in g for x in (b["min"], b["max"])])) for g in groups]
    everything = _sphere_around(_box_around([x for b in boxes for x in (b["min"], b["max"])]))
    if packed.primitiveCount > 0:
        f = np.asarray(packed.nodes[:8], dtype=np.uint32).view(np.float32)
        lo = (float(f[0]), float(f[1]), float(f[2]))
        hi = (float(f[4]), float(f[5]), float(f[6]))
        middle = ((lo[0] + hi[0]) * 0.5, (lo[1] + hi[1]) * 0.5, (lo[2] + hi[2]) * 0.5)
        reach = max(_length(_sub(t["centre"], middle)) for t in targets) + _length(_sub(hi, lo)) / 2 + 1
    else:
        reach = 1
    return {"centre": everything["centre"], "radius": everything["radius"], "reach": reach, "targets": targets}


def sun_radiance(sky):
    solid_angle = 2.0 * math.pi * (1.0 - math.cos(sky.sunSize))
    s = sky.sunStrength / solid_angle
    return (sky.sunColor.x * s, sky.sunColor.y * s, sky.sunColor.z * s)


def emitters(powers, deltas, sky, light_count):
    """#writeEmitters' vec4s (f32, u32 words where the reference writes
    them), or None when light tracing has nothing to do."""
    if not deltas:
        return None
    circles = 0.0
    for t in deltas["targets"]:
        circles += math.pi * t["radius"] ** 2
    sources = [dict(p) for p in powers]
    if sky.sunStrength > 0:
        omc = 2.0 * math.sin(sky.sunSize / 2.0) ** 2
        r = sun_radiance(sky)
        lum = 0.2126 * r[0] + 0.7152 * r[1] + 0.0722 * r[2]
        sources.append({"prim": NONE, "power": lum * 2 * math.pi * omc * circles})
    total = 0.0
    for s in sources:
        total += s["power"]
    if not (total > 0):
        return None
    data = np.zeros((2 + light_count + MAX_TARGETS) * 4, dtype=np.float32)
    u = data.view(np.uint32)
    u[0], u[1] = len(sources), len(deltas["targets"])
    data[2], data[3] = deltas["reach"], circles
    running = 0.0
    for k, s in enumerate(sources):
        running += s["power"] / total
        data[4 + 4 * k] = 1.0 if k == len(sources) - 1 else running
        u[4 + 4 * k + 1] = s["prim"]
        data[4 + 4 * k + 2] = s["power"] / total
    for j, t in enumerate(deltas["targets"]):
        o = 4 + (len(sources) + j) * 4
        data[o:o + 4] = [*t["centre"], t["radius"]]
    return data


def camera_basis(camera):
    """right, up and forward of Mat4.lookAt(position, target, up)."""
    eye, target, up = _v(camera.position), _v(camera.target), _v(camera.up)
    look = _normalized(_sub(target, eye))
    right = _normalized(_cross(look, up))
    true_up = _cross(right, look)
    return right, true_up, look


def params(scene, camera, width, height, light_count=0, volume_count=0, max_bounces=8, view="color",
           firefly_clamp=20.0, samples=0, spp=1, exposure=1.0, denoise=True, caustics=False, deltas=None) -> bytes:
    """The 208-byte uniform block of #writeParams for one frame."""
    buf = bytearray(208)
    f = np.frombuffer(buf, dtype=np.float32)
    u = np.frombuffer(buf, dtype=np.uint32)
    right, up, forward = camera_basis(camera)
    sky = scene.sky
    focus = camera.focusDistance if camera.focusDistance > 0.0 else _length(_sub(_v(camera.target),
                                                                                 _v(camera.position)))
    f[0:3] = _v(camera.position)
    f[3] = camera.aperture
    f[4:7] = right
    f[7] = math.tan(camera.fov / 2.0)
    f[8:11] = up
    f[11] = focus
    f[12:15] = forward
    f[15] = width / height
    f[16:19] = _v(sky.zenith)
    f[19] = 2.0 * math.sin(sky.sunSize / 2.0) ** 2
    f[20:23] = _v(sky.horizon)
    u[23] = 1 if sky.sunStrength > 0.0 else 0
    f[24:27] = _v(sky.ground)
    f[27] = firefly_clamp
    f[28:31] = _v(sky.sunDirection)
    u[31] = light_count
    f[32:35] = sun_radiance(sky)
    u[35] = max_bounces
    u[36] = VIEWS[view]
    u[37] = volume_count
    f[38] = sky.environmentStrength if sky.environment is not None else 0.0
    f[39] = sky.environmentRotation
    u[40], u[41] = width, height
    u[42], u[43], u[44] = samples, spp, samples + spp
    f[45] = exposure
    u[46] = 1 if denoise else 0
    u[47] = 1 if caustics else 0
    distance = (max(_length(_sub(_v(camera.position), deltas["centre"])), deltas["radius"]) if deltas else 1)
    start = max(3 * 2 * math.tan(camera.fov / 2) * distance / height, 1e-5)
    frame = math.floor(samples / max(spp, 1)) + 1
    f[48] = start * frame ** (-1 / 6)
    f[49] = 2 * f[48]
    return bytes(buf)
