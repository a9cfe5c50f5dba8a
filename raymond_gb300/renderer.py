"""Renderer (src/Renderer.mjs) over libraymond_cuda.so: the same properties,
restart rules, uniform block and packed uploads as the WebGPU renderer, with
the GPU work done by the sm_103a kernels behind the C ABI."""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _native
from ._native import check, lib, ptr
from .geometry import Box, Mesh, Quad
from .scene import NONE, PRIMITIVE_KINDS, Scene
from .vec import Vec3

VIEWS = {"color": 0, "albedo": 1, "normal": 2, "depth": 3}
PARAMS_BYTES = 208
IMAGE_KEY_BYTES = 168
PHOTON_CAPACITY = 524288
MAX_TARGETS = 16
UNIFORM_SHARE = 0.25


def light_chances(powers):
    """NEE's chance per light: 3/4 by power, 1/4 spread evenly (src/Renderer.mjs:1173-1179)."""
    total = sum(powers)
    n = len(powers)
    if not (total > 0) or not math.isfinite(total):
        return [1 / n for _ in powers]
    return [UNIFORM_SHARE / n + (1 - UNIFORM_SHARE) * p / total for p in powers]


def to_half(x: float) -> int:
    """Nearest half float's bits, saturating at 65504 (src/Renderer.mjs:1143-1160)."""
    if not (x > 0.0):
        return 0
    if x >= 65504.0:
        return 0x7BFF
    if x < 6.1035e-5:
        return int(_js_round(x / 5.9605e-8))
    exponent = math.floor(math.log2(x))
    mantissa = int(_js_round((x / 2 ** exponent - 1.0) * 1024))
    e = exponent + 15
    if mantissa == 1024:
        mantissa = 0
        e += 1
    return (e << 10) | mantissa


def _js_round(x: float) -> float:
    return math.floor(x + 0.5)


def to_half_array(x) -> np.ndarray:
    """to_half over an array at once (the environment upload's millions of
    values): the same steps in float64; the exponent comes from frexp, which
    gives floor(log2(x)) exactly, and a value that rounds up to the next
    power of two lands on it either way through the mantissa carry."""
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros(x.shape, dtype=np.uint16)
    pos = x > 0.0
    sat = pos & (x >= 65504.0)
    sub = pos & ~sat & (x < 6.1035e-5)
    norm = pos & ~sat & ~sub
    out[sat] = 0x7BFF
    out[sub] = np.floor(x[sub] / 5.9605e-8 + 0.5).astype(np.uint16)
    xn = x[norm]
    _, e2 = np.frexp(xn)
    exponent = e2.astype(np.int64) - 1
    mantissa = np.floor((xn / np.ldexp(1.0, exponent) - 1.0) * 1024 + 0.5).astype(np.int64)
    e = exponent + 15
    carry = mantissa == 1024
    mantissa[carry] = 0
    e[carry] += 1
    out[norm] = ((e << 10) | mantissa).astype(np.uint16)
    return out


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


def delta_objects(scene: Scene):
    """Mirrors and glass for light tracing to aim at (src/Renderer.mjs:1187-1254)."""
    boxes = []
    for obj in scene.objects:
        m = obj.material
        if not (m.type == "glass" or (m.type == "metal" and m.roughness < 0.01)):
            continue
        if isinstance(obj, Mesh):
            pts = [tuple(p) for p in obj.positions]
        elif isinstance(obj, Box):
            pts = [p.tuple() for p in obj.corners()]
        elif isinstance(obj, Quad):
            c, u, v = obj.corner, obj.u, obj.v
            pts = [c.tuple(), c.add(u).tuple(), c.add(v).tuple(), c.add(u).add(v).tuple()]
        else:
            r = Vec3(obj.radius, obj.radius, obj.radius)
            pts = [obj.center.subtract(r).tuple(), obj.center.add(r).tuple()]
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

    def sphere_around(box):
        return {"centre": Vec3((box["min"][0] + box["max"][0]) / 2, (box["min"][1] + box["max"][1]) / 2,
                               (box["min"][2] + box["max"][2]) / 2),
                "radius": max(_radius(box), 1e-3) * 1.001}

    targets = [sphere_around(_box_around([x for b in g for x in (b["min"], b["max"])])) for g in groups]
    allb = sphere_around(_box_around([x for b in boxes for x in (b["min"], b["max"])]))
    bounds = scene.bounds()
    if bounds:
        middle = bounds["min"].add(bounds["max"]).scale(0.5)
        reach = (max(t["centre"].subtract(middle).length() for t in targets)
                 + bounds["max"].subtract(bounds["min"]).length() / 2 + 1)
    else:
        reach = 1
    return {"centre": allb["centre"], "radius": allb["radius"], "reach": reach, "targets": targets}


def _gpu_name() -> str:
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:
        return "gpu"


def texture_array(textures, srgb):
    """A texture array as Renderer uploads one (src/Renderer.mjs:637-661):
    every texture resized to the largest width and height (at most 2048),
    as colour (sRGB) or as plain numbers; (RGBA bytes, width, height)."""
    w = min(2048, max(t.width for t in textures))
    h = min(2048, max(t.height for t in textures))
    return np.concatenate([t.resized(w, h, srgb).data.reshape(-1) for t in textures]), w, h


def byte_decoding(srgb):
    """What each byte value of a texture stands for when sampled
    (src/Texture.mjs fromSrgbByte, fromByte): linear light, or byte/255."""
    from .texture import _PLAIN, _SRGB_TO_LINEAR

    return _SRGB_TO_LINEAR if srgb else _PLAIN


def table_row_sines(width, height):
    """sin((y + 0.5) / rows · π) for each row of the environment's importance
    table (src/EnvironmentMap.mjs:208-213)."""
    cw = min(width, 512)
    rows = min(height, 256, cw)
    return [math.sin((y + 0.5) / rows * math.pi) for y in range(rows)]


def environment_arrays(env):
    """What Renderer uploads for an environment map (src/Renderer.mjs:723-760):
    its pixels as RGBA half floats (alpha 1) and its importance table."""
    rgba = np.empty(env.width * env.height * 4, dtype=np.uint16)
    rgba.reshape(-1, 4)[:, :3] = to_half_array(env.data.reshape(-1)).reshape(-1, 3)
    rgba.reshape(-1, 4)[:, 3] = to_half(1.0)
    return rgba, env.importance()


def emitters_block(light_powers, light_count, deltas, sky):
    """Renderer.#writeEmitters (src/Renderer.mjs:670-717): a header (sources,
    targets, the sun's start distance, the targets' circles' total area),
    then per source its running chance, primitive (NONE for the sun) and
    chance, chosen by power (the sun's is what falls on the targets'
    circles), then the target spheres (centre, radius). float32 vec4s, or
    None if there is nothing for light tracing to do."""
    if not deltas:
        return None
    circles = sum(math.pi * t["radius"] ** 2 for t in deltas["targets"])
    sources = list(light_powers)
    if sky.sunStrength > 0:
        omc = 2.0 * math.sin(sky.sunSize / 2.0) ** 2
        r = sky.sunRadiance
        lum = 0.2126 * r.x + 0.7152 * r.y + 0.0722 * r.z
        sources.append({"prim": NONE, "power": lum * 2 * math.pi * omc * circles})
    total = sum(src["power"] for src in sources)
    if not (total > 0):
        return None
    data = np.zeros((2 + light_count + MAX_TARGETS) * 4, dtype=np.float32)
    u = data.view(np.uint32)
    u[0] = len(sources)
    u[1] = len(deltas["targets"])
    data[2] = deltas["reach"]
    data[3] = circles
    running = 0.0
    for k, src in enumerate(sources):
        running += src["power"] / total
        data[4 + k * 4] = 1.0 if k == len(sources) - 1 else running
        u[4 + k * 4 + 1] = src["prim"]
        data[4 + k * 4 + 2] = src["power"] / total
    for j, t in enumerate(deltas["targets"]):
        c = t["centre"]
        data[4 + (len(sources) + j) * 4: 8 + (len(sources) + j) * 4] = [c.x, c.y, c.z, t["radius"]]
    return data


def light_table(packed):
    """The lights buffer of Renderer.#upload (src/Renderer.mjs:571-607): the
    light primitives, the volumes, then each light's running total chance
    as f32 bits (last forced to 1); and each light's power (luminance ·
    π · area), which light tracing chooses by. Returns (u32 words, powers)."""
    lights = [] if packed.lights[0] == NONE else [int(x) for x in packed.lights]
    pf = packed.primitives.view(np.float32)
    mf = packed.materials.view(np.float32)
    powers = []
    for p in lights:
        b, m = p * 16, int(packed.primitives[p * 16 + 1]) * 24
        lum = 0.2126 * float(mf[m + 4]) + 0.7152 * float(mf[m + 5]) + 0.0722 * float(mf[m + 6])
        if packed.primitives[b] == PRIMITIVE_KINDS["quad"]:
            u = Vec3(float(pf[b + 8]), float(pf[b + 9]), float(pf[b + 10]))
            v = Vec3(float(pf[b + 12]), float(pf[b + 13]), float(pf[b + 14]))
            area = u.cross(v).length()
        else:
            area = 4 * math.pi * float(pf[b + 7]) ** 2
        powers.append({"prim": p, "power": lum * math.pi * area})
    chances = light_chances([l["power"] for l in powers])
    total = 0.0
    cumulative = []
    for c in chances:
        total += c
        cumulative.append(total)
    cum = np.array(cumulative, dtype=np.float32)
    if cum.size:
        cum[-1] = 1.0
    words = np.concatenate([np.array(lights, dtype=np.uint32), np.array(packed.volumes, dtype=np.uint32),
                            cum.view(np.uint32)]).astype(np.uint32)
    if words.size == 0:
        words = np.array([NONE], dtype=np.uint32)
    return words, powers


def params_block(scene, camera, width, height, light_count=0, volume_count=0, max_bounces=8, view="color",
                 firefly_clamp=20.0, samples=0, spp=1, exposure=1.0, denoise=True, caustics=False,
                 deltas=None) -> bytes:
    """The 208-byte uniform block as Renderer.#writeParams lays it out
    (src/Renderer.mjs:925-991; offsets src/shaders.mjs:9-24)."""
    buf = bytearray(PARAMS_BYTES)
    f = np.frombuffer(buf, dtype=np.float32)
    u = np.frombuffer(buf, dtype=np.uint32)
    b = camera.basis()
    sky = scene.sky

    def row(r, v):
        f[r * 4: r * 4 + 3] = [v.x, v.y, v.z]

    row(0, camera.position)
    f[3] = camera.aperture
    row(1, b["right"])
    f[7] = math.tan(camera.fov / 2.0)
    row(2, b["up"])
    f[11] = camera.effectiveFocusDistance
    row(3, b["forward"])
    f[15] = width / height
    row(4, sky.zenith)
    f[19] = 2.0 * math.sin(sky.sunSize / 2.0) ** 2
    row(5, sky.horizon)
    u[23] = 1 if sky.sunStrength > 0.0 else 0
    row(6, sky.ground)
    f[27] = firefly_clamp
    row(7, sky.sunDirection)
    u[31] = light_count
    row(8, sky.sunRadiance)
    u[35] = max_bounces
    u[36] = VIEWS[view]
    u[37] = volume_count
    f[38] = sky.environmentStrength if sky.environment is not None else 0.0
    f[39] = sky.environmentRotation
    u[40] = width
    u[41] = height
    u[42] = samples
    u[43] = spp
    u[44] = samples + spp
    f[45] = exposure
    u[46] = 1 if denoise else 0
    u[47] = 1 if caustics else 0
    # Photon mapping's radius: ~3 pixels where the camera sees the mirrors
    # and glass, shrinking as frames^(-1/6); cells twice the radius.
    distance = max(camera.position.subtract(deltas["centre"]).length(), deltas["radius"]) if deltas else 1
    start = max(3 * 2 * math.tan(camera.fov / 2) * distance / height, 1e-5)
    frame = math.floor(samples / max(spp, 1)) + 1
    f[48] = start * frame ** (-1 / 6)
    f[49] = 2 * f[48]
    return bytes(buf)


class _Queue:
    def __init__(self, renderer):
        self._r = renderer

    def onSubmittedWorkDone(self):
        """Blocks until the frame's GPU work is done (the Promise's resolution)."""
        self._r._sync()


class _Device:
    def __init__(self, renderer):
        self.queue = _Queue(renderer)


class Canvas:
    """A headless canvas: only its size matters."""

    def __init__(self, width: int, height: int):
        self.width = width
        self.height = height


class Renderer:
    """Progressive path tracer (src/Renderer.mjs:84-1137) on one GPU."""

    def __init__(self, handle, canvas, device_index=0, seed=0):
        self._h = handle
        self._canvas = canvas
        self._device = _Device(self)
        self._scene = None
        self._camera = None
        self._max_bounces = 8
        self._spp = 1
        self._exposure = 1.0
        self._firefly = 20.0
        self._view = "color"
        self._denoise = True
        self._caustics = True
        self._caustics_active = False
        self._samples = 0
        self._params = bytearray(PARAMS_BYTES)
        self._image_key = bytes(IMAGE_KEY_BYTES)
        self._uploaded_scene = None
        self._uploaded_version = -1
        self._uploaded_environment = False  # nothing uploaded yet (the reference's undefined)
        self._light_count = 0
        self._volume_count = 0
        self._textured = False
        self._dispersive = False
        self._light_powers = []
        self._deltas = None
        self._width = 0
        self._height = 0
        self._resized = False
        self._disposed = False
        self._batch = None  # the BatchRenderer that rendered its last frame, if any
        self.flags = 0  # extra raymond_render flags (path choice)
        # A Denoiser (raymond_gb300.denoiser) to filter the displayed image
        # instead of the à-trous filter; None keeps the à-trous filter.
        self.learnedDenoiser = None

    @staticmethod
    def create(canvas, powerPreference="high-performance", device=0, seed=0, pathCapacity=0) -> "Renderer":
        """Renderer.create (src/Renderer.mjs:247-279); raises RuntimeError if no GPU can be used.
        seed: XORed into the sample hashes (0 keeps the reference's streams);
        pathCapacity: wavefront paths in flight (0: sized automatically)."""
        cfg = _native.Config(device=device, seed=seed, path_capacity=pathCapacity)
        h = ctypes.c_void_p()
        rc = lib().raymond_create(ctypes.byref(h), ctypes.byref(cfg))
        if rc != _native.OK:
            msg = lib().raymond_last_error(None)
            raise RuntimeError(f"CUDA isn't available: {msg.decode() if msg else rc}")
        return Renderer(h, canvas, device, seed)

    # ---- properties (src/Renderer.mjs:281-395) ----
    @property
    def device(self):
        return self._device

    @property
    def canvas(self):
        return self._canvas

    @property
    def scene(self):
        return self._scene

    @scene.setter
    def scene(self, value):
        self._scene = value

    @property
    def camera(self):
        return self._camera

    @camera.setter
    def camera(self, value):
        self._camera = value

    @property
    def maxBounces(self):
        return self._max_bounces

    @maxBounces.setter
    def maxBounces(self, value):
        self._max_bounces = max(1, min(64, math.floor(value)))

    @property
    def samplesPerFrame(self):
        return self._spp

    @samplesPerFrame.setter
    def samplesPerFrame(self, value):
        self._spp = max(1, min(64, math.floor(value)))

    @property
    def exposure(self):
        return self._exposure

    @exposure.setter
    def exposure(self, value):
        self._exposure = max(float(value), 0.0)

    @property
    def fireflyClamp(self):
        return self._firefly

    @fireflyClamp.setter
    def fireflyClamp(self, value):
        self._firefly = max(float(value), 0.0)

    @property
    def view(self):
        return self._view

    @view.setter
    def view(self, value):
        if value not in VIEWS:
            raise ValueError(f'Unknown view "{value}".')
        self._view = value

    @property
    def denoise(self):
        return self._denoise

    @denoise.setter
    def denoise(self, value):
        self._denoise = bool(value)

    @property
    def caustics(self):
        return self._caustics

    @caustics.setter
    def caustics(self, value):
        self._caustics = bool(value)

    @property
    def samples(self):
        return self._samples

    def reset(self):
        self._samples = 0

    # ---- frames ----
    def _prepare(self):
        """Everything render() does before launching: uploads, resize,
        caustics gate, uniforms. Returns the feature bits."""
        scene, camera = self._scene, self._camera
        width = max(1, int(self._canvas.width))
        height = max(1, int(self._canvas.height))
        if scene is not self._uploaded_scene or scene.version != self._uploaded_version:
            self._upload(scene)
        env = scene.sky.environment
        if self._uploaded_environment is False or env is not self._uploaded_environment:
            self._upload_environment(env)
        if not self._resized or width != self._width or height != self._height:
            self._resize(width, height)
        caustics = False
        if self._caustics and camera.aperture == 0 and self._view == "color" and self._volume_count == 0:
            caustics = self._caustics_enabled(scene)
        if caustics != self._caustics_active:
            self._caustics_active = caustics
            self._samples = 0
        self._write_params(scene, camera, width, height)
        return ((_native.FEATURE_VOLUMES if self._volume_count > 0 else 0)
                | (_native.FEATURE_TEXTURES if self._textured else 0)
                | (_native.FEATURE_ENVIRONMENT if env is not None else 0)
                | (_native.FEATURE_DISPERSION if self._dispersive else 0))

    def render(self):
        """Adds samplesPerFrame paths per pixel (src/Renderer.mjs:406-491)."""
        if self._scene is None or self._camera is None:
            return
        features = self._prepare()
        buf = (ctypes.c_char * PARAMS_BYTES).from_buffer(self._params)
        check(lib().raymond_render(self._h, ctypes.addressof(buf), features, self.flags), self._h)
        self._samples += self._spp
        self._denoise_learned()

    def autotune(self, trials: int = 2, cache: str | None = None):
        """Picks the launch shape for this scene and image by timing
        candidates (the one-kernel path; wavefront traversal steps and
        blocks per SM; the binary or the 4-wide tree) and keeps the fastest; remembered in a JSON cache
        keyed by GPU, features, scene-size bucket, resolution, samples per
        frame and bounces. Starts the image over. Returns the tuning."""
        import json
        import os

        if self._scene is None or self._camera is None:
            raise RuntimeError("Set a scene and camera before tuning.")
        features = self._prepare()
        packed = self._scene.pack()
        key = "|".join(str(x) for x in (
            _gpu_name(), features, int(math.log2(max(packed.primitiveCount, 1))), self._width, self._height,
            self._spp, self._max_bounces))
        path = cache or os.path.join(os.path.expanduser("~"), ".cache", "raymond_gb300", "tuning.json")
        table = {}
        try:
            with open(path) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
        t = _native.Tuning()
        if key in table:
            for k, v in table[key].items():
                setattr(t, k, v)
            check(lib().raymond_set_tuning(self._h, ctypes.byref(t)), self._h)
        else:
            buf = (ctypes.c_char * PARAMS_BYTES).from_buffer(self._params)
            check(lib().raymond_autotune(self._h, ctypes.addressof(buf), features, trials, ctypes.byref(t)), self._h)
            table[key] = {f: getattr(t, f) for f, _ in _native.Tuning._fields_}
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                with open(path, "w") as f:
                    json.dump(table, f, indent=1)
            except OSError:
                pass
        self._samples = 0
        return {f: getattr(t, f) for f, _ in _native.Tuning._fields_}

    @property
    def tuning(self):
        t = _native.Tuning()
        check(lib().raymond_get_tuning(self._h, ctypes.byref(t)), self._h)
        return {f: getattr(t, f) for f, _ in _native.Tuning._fields_}

    def _caustics_enabled(self, scene) -> bool:
        """Uploads the emitters light tracing starts from; False if there is
        nothing for light tracing to do."""
        data = emitters_block(self._light_powers, self._light_count, self._deltas, scene.sky)
        if data is None:
            return False
        check(lib().raymond_set_emitters(self._h, ptr(data), data.size // 4), self._h)
        return True

    def setPhotons(self, photonsPerFrame=0, capacity=0, radius=0.0):
        """Light paths per frame, photon-map capacity and a fixed gathering
        radius beyond the reference's sizes (0: the reference's)."""
        check(lib().raymond_set_photons(self._h, int(photonsPerFrame), int(capacity), float(radius)), self._h)

    def readPixels(self, denoised=False, out=None) -> np.ndarray:
        """The average so far, w×h×4 float32 from the top left (src/Renderer.mjs:502-528).
        `out`, if given, is a C-contiguous float32 array of w·h·4 elements that
        is filled and returned (one buffer, say page-locked, reused across
        frames instead of a new one each time)."""
        if self._batch is not None:
            self._batch.sync()
        if not self._resized or self._samples == 0:
            raise RuntimeError("Nothing has been rendered yet.")
        if denoised and not self._denoising():
            raise RuntimeError("Only the color view is denoised, with denoise on.")
        n = self._width * self._height * 4
        if out is None:
            out = np.empty(n, dtype=np.float32)
        elif not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.size == n and out.flags.c_contiguous):
            raise ValueError(f"readPixels(out=...) needs a C-contiguous float32 array of {n} elements.")
        check(lib().raymond_read_pixels(self._h, ptr(out), out.nbytes, 1 if denoised else 0, self._samples), self._h)
        return out

    def readGuides(self):
        """The raw per-pixel sums: accum, guide albedo, guide normal (each h×w×4 float32)."""
        if self._batch is not None:
            self._batch.sync()
        shape = (self._height, self._width, 4)
        a, g, n = (np.empty(shape, dtype=np.float32) for _ in range(3))
        check(lib().raymond_read_guides(self._h, ptr(a), ptr(g), ptr(n), a.nbytes), self._h)
        return a, g, n

    def readDisplay(self) -> np.ndarray:
        """The tone-mapped display image as h×w×4 uint8 (the canvas's pixels)."""
        out = np.empty((self._height, self._width, 4), dtype=np.uint8)
        check(lib().raymond_read_display(self._h, ptr(out), out.nbytes), self._h)
        return out

    def dispose(self):
        if not self._disposed and self._h:
            lib().raymond_destroy(self._h)
            self._h = None
            self._disposed = True

    def __del__(self):
        try:
            self.dispose()
        except Exception:
            pass

    def _sync(self):
        check(lib().raymond_sync(self._h), self._h)

    def _denoising(self):
        return self._denoise and self._view == "color"

    def _atrous(self):
        """The à-trous filter runs inside the frame unless the network replaces it."""
        return self._denoising() and self.learnedDenoiser is None

    def _denoise_learned(self):
        """The network over this frame's sums (display only), on this renderer's stream."""
        if self.learnedDenoiser is not None and self._denoising():
            check(lib().raymond_denoise_learned(self._h, self.learnedDenoiser.handle, self._samples, None), self._h)

    # ---- uploads (src/Renderer.mjs:550-799) ----
    def _upload(self, scene: Scene):
        packed = scene.pack()
        words, powers = light_table(packed)
        lights = [p["prim"] for p in powers]
        self._light_count = len(lights)
        self._volume_count = len(packed.volumes)
        self._textured = len(packed.textures) + len(packed.normalMaps) > 0
        self._dispersive = any(m.dispersion > 0 for m in packed.materialList)
        self._light_powers = powers
        self._words = words
        self._deltas = delta_objects(scene)
        attrs = packed.attributes.astype(np.float32)
        check(lib().raymond_upload_scene(
            self._h, ptr(packed.primitives), packed.primitives.size // 16, packed.primitiveCount,
            ptr(packed.nodes), packed.nodeCount, ptr(packed.materials), max(packed.materialCount, 1),
            ptr(attrs), attrs.size // 4, ptr(words), words.size, len(lights), len(packed.volumes)), self._h)
        self._upload_textures(packed)
        self._uploaded_scene = scene
        self._uploaded_version = scene.version
        self._samples = 0

    def _upload_textures(self, packed):
        """The texture arrays, each texture resized into its layer on the GPU
        (raymond_upload_texture_images; the same bytes as texture_array)."""
        for which, textures, srgb in ((0, packed.textures, True), (1, packed.normalMaps, False)):
            if not textures:
                continue
            images = [np.ascontiguousarray(t.data, dtype=np.uint8) for t in textures]
            ptrs = (ctypes.c_void_p * len(images))(*[ptr(a) for a in images])
            widths = np.array([t.width for t in textures], dtype=np.uint32)
            heights = np.array([t.height for t in textures], dtype=np.uint32)
            decode = np.ascontiguousarray(byte_decoding(srgb), dtype=np.float64)
            check(lib().raymond_upload_texture_images(self._h, which, ptrs, ptr(widths), ptr(heights), len(images),
                                                      1 if srgb else 0, ptr(decode)), self._h)

    def _upload_environment(self, env):
        """The environment's half floats and importance table, built on the GPU
        (raymond_upload_environment_rgb; the same as environment_arrays)."""
        if env is not None:
            rgb = np.ascontiguousarray(env.data, dtype=np.float32)
            sines = np.ascontiguousarray(table_row_sines(env.width, env.height), dtype=np.float64)
            check(lib().raymond_upload_environment_rgb(self._h, ptr(rgb), env.width, env.height, ptr(sines),
                                                       len(sines)), self._h)
        self._uploaded_environment = env
        self._samples = 0

    def _resize(self, width, height):
        check(lib().raymond_resize(self._h, width, height), self._h)
        self._width, self._height = width, height
        self._resized = True
        self._samples = 0

    def _write_params(self, scene, camera, width, height):
        """Renderer.#writeParams (src/Renderer.mjs:925-991) with its restart rule."""
        block = params_block(scene, camera, width, height, light_count=self._light_count,
                             volume_count=self._volume_count, max_bounces=self._max_bounces, view=self._view,
                             firefly_clamp=self._firefly, samples=self._samples, spp=self._spp,
                             exposure=self._exposure, denoise=self._atrous(), caustics=self._caustics_active,
                             deltas=self._deltas)
        key = bytes(block[:IMAGE_KEY_BYTES])
        if key != self._image_key:
            self._image_key = key
            self._samples = 0
            block = params_block(scene, camera, width, height, light_count=self._light_count,
                                 volume_count=self._volume_count, max_bounces=self._max_bounces, view=self._view,
                                 firefly_clamp=self._firefly, samples=0, spp=self._spp, exposure=self._exposure,
                                 denoise=self._atrous(), caustics=self._caustics_active, deltas=self._deltas)
        self._params[:] = block

    def tracePrimary(self, rays: np.ndarray, scene: Scene | None = None):
        """Closest hits of rays (n×6 float32: origin, direction) on the
        scene (uploaded first if it changed): leaf-order primitive indices
        (NONE for a miss) and distances, via raymond_trace_primary."""
        scene = scene if scene is not None else self._scene
        if scene is not self._uploaded_scene or scene.version != self._uploaded_version:
            self._upload(scene)
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        prim = np.empty(len(rays), dtype=np.uint32)
        t = np.empty(len(rays), dtype=np.float32)
        check(lib().raymond_trace_primary(self._h, ptr(rays), len(rays), ptr(prim), ptr(t)), self._h)
        return prim, t

    @property
    def params(self) -> bytes:
        """The last uniform block written (208 bytes)."""
        return bytes(self._params)

    @property
    def handle(self):
        return self._h


class BatchRenderer:
    """Renders a frame of many renderers in one pass (raymond_render_batch):
    their paths share one wavefront pool and the frame replays as one CUDA
    graph while the set of images, sample counts and bounces stays the same.
    Each renderer keeps its own scene, image and progressive average."""

    def __init__(self, device=0, graph=True, pathCapacity=0):
        self._exec = Renderer.create(Canvas(1, 1), device=device, pathCapacity=pathCapacity)
        self.graph = graph

    def render(self, renderers):
        n = len(renderers)
        jobs = (_native.Job * n)()
        keep = []
        for i, r in enumerate(renderers):
            if r.scene is None or r.camera is None:
                raise ValueError("Every renderer in a batch needs a scene and a camera.")
            r.caustics = False
            features = r._prepare()
            buf = (ctypes.c_char * PARAMS_BYTES).from_buffer(r._params)
            keep.append(buf)
            jobs[i] = _native.Job(r.handle, ctypes.addressof(buf), features)
        check(lib().raymond_render_batch(self._exec.handle, jobs, n, _native.BATCH_GRAPH if self.graph else 0),
              self._exec.handle)
        for r in renderers:
            r._samples += r._spp
            r._batch = self
            r._denoise_learned()

    def sync(self):
        check(lib().raymond_sync(self._exec.handle), self._exec.handle)

    @property
    def handle(self):
        return self._exec.handle

    def stats(self):
        st = _native.Stats()
        check(lib().raymond_get_stats(self._exec.handle, ctypes.byref(st)), self._exec.handle)
        return st

    def dispose(self):
        self._exec.dispose()
