"""CUDA against the oracle on the same inputs, with every disagreement
classified (tests/parity.py): per-pixel images of both render paths on the
Cornell room (pinhole and thin lens), the reference's fixture scenes (GGX
metal and plastic, dielectric and dispersive glass, fog, textures, normal
maps, the environment map) and crops of the 1024² sphere field (10,000
spheres of diffuse, metal and glass, the smooth 499,280-triangle mesh, the
sun); one frame's light tracing (splat sums and photons, matched by light
path) and the photon map's gather on identical photon lists, on the
reference's caustic fixtures and on the water-caustics scene at 1M light
paths, a 4M-photon map and r = 0.01; and the 16-seed unbiasedness test on
a small scene of the sphere field's kind; and the jobs of one batched
frame, each against the oracle. No unexplained difference is allowed
anywhere.

Reference: src/shaders.mjs:133-212 (streams), 714-871 (BSDFs),
1148-1166 (camera_ray), 1436-1831 (splat, photon map, light_trace,
resolve); tests/browser/app.test.mjs:127-156, 512-569."""

import ctypes

import numpy as np
import pytest

import fixtures
import oracle
from oracle import host, pack
from parity import classify_light_paths, classify_pixels, perturbation_runs
from raymond_gb300 import Camera, Canvas, Renderer, _native, scenes
from raymond_gb300.renderer import environment_arrays, texture_array

pytestmark = pytest.mark.gpu

WF, MK = _native.FLAG_WAVEFRONT, _native.FLAG_MEGAKERNEL


def gpu_frame(scene, camera, w, h, spp, flags, bounces=8, seed=0):
    r = Renderer.create(Canvas(w, h), seed=seed)
    r.scene, r.camera = scene, camera
    r.maxBounces, r.samplesPerFrame, r.fireflyClamp, r.denoise = bounces, spp, 0, False
    r.caustics = False
    r.flags = flags
    r.render()
    r.device.queue.onSubmittedWorkDone()
    params, accum = r.params, r.readGuides()[0]
    r.dispose()
    return params, accum


def oracle_frame(scene, params, region=None, seed=0):
    """The oracle's frame and its perturbation runs, on the uploaded arrays."""
    packed = pack.pack(scene.objects)
    words, _ = host.light_words(packed)
    kw = {}
    if packed.textures:
        kw["textures"] = texture_array(packed.textures, True)
    if packed.normalMaps:
        kw["normal_maps"] = texture_array(packed.normalMaps, False)
    env = scene.sky.environment
    if env is not None:
        rgba, table = environment_arrays(env)
        kw["environment"] = (rgba, env.width, env.height, table)

    def run():
        return oracle.render(packed, words, params, region=region, seed_hash=seed, **kw)["accum"]

    return run(), perturbation_runs(run)


def fixture(name, arg=None):
    scene, cam = fixtures.SCENES[name](arg)
    return scene, Camera(**cam)


def cornell_lens():
    scene, camera = scenes.cornell_scene()
    return scene, Camera(position=camera.position, target=camera.target, up=camera.up, fov=camera.fov,
                         aperture=0.04, focusDistance=1.6)


IMAGE_CASES = {
    # name: (scene and camera, size, spp, share of pixels allowed to differ at all (classified))
    "cornell": (scenes.cornell_scene, 64, 8, 0.01),
    "cornell_thin_lens": (cornell_lens, 64, 8, 0.01),
    "room": (lambda: fixture("room"), 48, 8, 0.01),
    "mixed_metal_plastic_glass": (lambda: fixture("mixed"), 48, 8, 0.01),
    "glass_furnace": (lambda: fixture("furnaceGlass"), 48, 8, 0.01),
    "dispersive_glass": (lambda: fixture("stripThroughGlass", "20"), 48, 8, 0.01),
    "fog_lamp": (lambda: fixture("lampInFog", "light"), 48, 8, 0.01),
    "textured": (lambda: fixture("textured"), 48, 4, 0.01),
    "normal_maps": (lambda: fixture("bumpy"), 48, 4, 0.01),
    "environment": (lambda: fixture("environmentFloor"), 48, 4, 0.01),
}


@pytest.mark.parametrize("flags", [WF, MK], ids=["wavefront", "one_kernel"])
@pytest.mark.parametrize("name", list(IMAGE_CASES))
def test_image_matches_oracle_per_pixel(gpu, name, flags):
    make, size, spp, share = IMAGE_CASES[name]
    scene, camera = make()
    params, got = gpu_frame(scene, camera, size, size, spp, flags)
    ref, runs = oracle_frame(scene, params)
    c = classify_pixels(got, ref, runs)
    assert c["unexplained"] == 0, (name, c)
    assert c["agree"] >= (1.0 - share) * c["n"], (name, c)
    if c["decision"] == 0:  # the luminance² sums (the variance the denoiser reads) follow the colour
        assert np.allclose(got[..., 3], ref[..., 3], rtol=1e-3, atol=1e-6)


# 64² crops of the 1024² frame and the share of their pixels that must agree
# outright: most of the mesh crop, all of the sky and ground by the horizon,
# half of a crop full of glass spheres (chains of refractions there turn
# rounding into visibly different paths, every one a classified decision).
FIELD_CROPS = {"mesh": ((480, 480), 0.85), "horizon": ((200, 300), 0.99), "glass_and_metal": ((700, 560), 0.45)}


@pytest.mark.parametrize("flags", [WF, MK], ids=["wavefront", "one_kernel"])
@pytest.mark.parametrize("crop", list(FIELD_CROPS))
def test_sphere_field_crop_matches_oracle_per_pixel(gpu, sphere_field, crop, flags):
    """Crops of the headline frame at 4 spp: GGX metal and glass spheres, the
    smooth mesh, the sun, roulette from bounce 3."""
    scene, camera = sphere_field
    params, got = gpu_frame(scene, camera, 1024, 1024, 4, flags)
    (x0, y0), share = FIELD_CROPS[crop]
    ref, runs = oracle_frame(scene, params, region=(x0, y0, 64, 64))
    c = classify_pixels(got[y0:y0 + 64, x0:x0 + 64], ref, runs)
    assert c["unexplained"] == 0, (crop, c["unexplained_idx"], c)
    assert c["agree"] >= share * c["n"], (crop, c)


@pytest.fixture(scope="module")
def sphere_field():
    scene, camera, _ = scenes.sphere_field()
    return scene, camera


# Jobs of one batched frame: (case, size, spp, crop or None, share that must agree outright).
BATCH_CASES = [("cornell", 64, 8, None, 0.99), ("mixed_metal_plastic_glass", 48, 8, None, 0.99),
               ("dispersive_glass", 48, 8, None, 0.99), ("environment", 48, 4, None, 0.99),
               ("sphere_field", 1024, 4, (480, 480), 0.85)]


def test_batched_jobs_match_oracle_per_pixel(gpu, sphere_field):
    """One batched frame of several scenes (raymond_render_batch: one path
    pool in groups, one CUDA graph), each job's image against the oracle on
    its own parameters, every difference classified: the batch is checked
    against the oracle itself, not only against single frames."""
    from raymond_gb300 import BatchRenderer

    jobs = []
    for name, size, spp, crop, share in BATCH_CASES:
        scene, camera = sphere_field if name == "sphere_field" else IMAGE_CASES[name][0]()
        r = Renderer.create(Canvas(size, size), seed=0)
        r.scene, r.camera = scene, camera
        r.maxBounces, r.samplesPerFrame, r.fireflyClamp, r.denoise = 8, spp, 0, False
        r.flags = WF
        jobs.append((name, scene, r, crop, share))
    batch = BatchRenderer(graph=True)
    batch.render([j[2] for j in jobs])
    batch.sync()
    for name, scene, r, crop, share in jobs:
        got = r.readGuides()[0]
        if crop is None:
            ref, runs = oracle_frame(scene, r.params)
        else:
            x0, y0 = crop
            ref, runs = oracle_frame(scene, r.params, region=(x0, y0, 64, 64))
            got = got[y0:y0 + 64, x0:x0 + 64]
        c = classify_pixels(got, ref, runs)
        assert c["unexplained"] == 0, (name, c)
        assert c["agree"] >= share * c["n"], (name, c)
    for j in jobs:
        j[2].dispose()
    batch.dispose()


# ---- light transport ----

def light_trace_both(scene, camera, size, spp=4, photons=0, capacity=0, radius=0.0):
    """One frame's light tracing on the GPU (raymond_light_trace) and in the
    oracle with its perturbation runs, on the same uniform block."""
    r = Renderer.create(Canvas(size, size))
    r.scene, r.camera = scene, camera
    r.samplesPerFrame, r.denoise, r.caustics = spp, False, True
    if photons or capacity or radius:
        r.setPhotons(photons, capacity, radius)
    r.render()
    r.device.queue.onSubmittedWorkDone()
    features = r._prepare()
    block = bytearray(r.params)
    assert int(np.frombuffer(block, np.uint32)[47]) == 1, "caustics are on for this scene"
    if radius:
        f = np.frombuffer(block, dtype=np.float32)
        f[48], f[49] = radius, 2 * radius  # the radius the renderer applies
    params = bytes(block)
    cap = capacity or 524288
    splats = np.zeros(size * size * 4, np.uint32)
    photons_out = np.zeros(cap * 11, np.float32)
    count = ctypes.c_uint32()
    pbuf = (ctypes.c_char * 208).from_buffer_copy(params)
    lib = _native.lib()
    _native.check(lib.raymond_light_trace(r.handle, ctypes.addressof(pbuf), features, _native.ptr(splats),
                                          splats.nbytes, _native.ptr(photons_out), photons_out.size,
                                          ctypes.byref(count)), r.handle)
    n = count.value
    gpu = {"splats": splats.reshape(size, size, 4), "photons": photons_out[: n * 11].reshape(n, 11)}

    packed = pack.pack(scene.objects)
    words, powers = host.light_words(packed)
    deltas = host.delta_objects(scene.objects, packed)
    emitters = host.emitters(powers, deltas, scene.sky, len(powers))
    light_paths = photons or min(size * size * spp, cap)

    def run():
        return oracle.light_trace(packed, words, params, emitters, light_paths)

    ref = oracle.light_trace(packed, words, params, emitters, light_paths, margins=True)

    def gather(photon_list, rows):
        out = np.zeros(size * size * 4, np.float32)
        plist = np.ascontiguousarray(photon_list, np.float32)
        _native.check(lib.raymond_photon_gather(r.handle, ctypes.addressof(pbuf), features, _native.ptr(plist),
                                                len(plist), _native.ptr(out), out.nbytes), r.handle)
        return out.reshape(size, size, 4)

    ctx = {"packed": packed, "words": words, "params": params, "gpu_gather": gather, "renderer": r}
    return gpu, ref, perturbation_runs(run), ctx


CAUSTIC_FIXTURES = ["causticLamp", "causticSun", "causticMirror", "causticLampMany", "causticSunMany",
                    "causticThroughGlass"]


@pytest.mark.parametrize("name", CAUSTIC_FIXTURES)
def test_light_tracing_matches_oracle(gpu, name):
    """Photons and splats matched by light path, and the splat sums per
    pixel, 96² at 4 spp (36,864 light paths)."""
    scene, camera = fixture(name)
    got, ref, runs, ctx = light_trace_both(scene, camera, 96)
    try:
        c = classify_light_paths(got["photons"], got["splats"], ref, runs, ctx["params"])
        assert c["unexplained"] == 0 and c["splat_unexplained"] == 0 and c["pixel_unexplained"] == 0, (name, c)
        assert c["agree"] >= 0.5 * c["paths"], (name, c)
    finally:
        ctx["renderer"].dispose()


@pytest.mark.parametrize("name", CAUSTIC_FIXTURES)
def test_photon_gather_matches_oracle_on_the_same_photons(gpu, name):
    """The gather over the oracle's own photon list on both sides; pixels
    whose 8 cells hold more than the 4,096 photons a gather visits depend on
    list order (the GPU's follows its atomics) and are counted apart."""
    scene, camera = fixture(name)
    _, ref, _, ctx = light_trace_both(scene, camera, 96)
    try:
        got = ctx["gpu_gather"](ref["photons"], None)

        def run():
            return oracle.photon_gather(ctx["packed"], ctx["words"], ctx["params"], ref["photons"])

        base, visits = oracle.photon_gather(ctx["packed"], ctx["words"], ctx["params"], ref["photons"], visits=True)
        c = classify_pixels(got, base, perturbation_runs(run))
        capped = int((visits >= 4096).sum())
        assert c["unexplained"] <= capped, (name, c, capped)
        assert c["agree"] + c["decision"] + c["continuous"] + capped >= c["n"]
    finally:
        ctx["renderer"].dispose()


def test_water_caustics_at_full_parameters(gpu):
    """The water-caustics scene at 1024²: 1,000,000 light paths splatted and
    deposited into a 4,194,304-photon map, gathered at r = 0.01 (cell
    0.02), on a band of 64 rows through the pool."""
    scene, camera, _ = scenes.water_caustics()
    got, ref, runs, ctx = light_trace_both(scene, camera, 1024, photons=1_000_000, capacity=4_194_304, radius=0.01)
    try:
        assert len(ref["photons"]) > 100_000
        c = classify_light_paths(got["photons"], got["splats"], ref, runs, ctx["params"])
        assert c["unexplained"] == 0 and c["splat_unexplained"] == 0 and c["pixel_unexplained"] == 0, c
        assert c["agree"] >= 0.99 * c["paths"], c
        rows = (448, 64)
        g = ctx["gpu_gather"](ref["photons"], rows)[448:512]

        def run():
            return oracle.photon_gather(ctx["packed"], ctx["words"], ctx["params"], ref["photons"], rows=rows)[448:512]

        base, visits = oracle.photon_gather(ctx["packed"], ctx["words"], ctx["params"], ref["photons"], rows=rows,
                                            visits=True)
        c = classify_pixels(g, base[448:512], perturbation_runs(run))
        capped = int((visits[448:512] >= 4096).sum())
        assert c["unexplained"] <= capped, (c, capped)
        assert (np.abs(base[448:512, :, :3]).max(axis=-1) > 0).sum() > 1000  # the band sees caustics
    finally:
        ctx["renderer"].dispose()


# ---- unbiasedness on a scene of the sphere field's kind ----

def test_sixteen_seeds_are_unbiased_on_a_small_sphere_field(gpu):
    """16 seeds × 64 spp on a 32² frame of a small sphere field (300
    spheres: diffuse, GGX metal, glass; a smooth 2,000-triangle mesh; the
    sun; 8 bounces with roulette): the per-pixel mean lies within 3σ of the
    oracle's 4,096-spp render, save the 0.27% tail plus a 1.5% margin."""
    scene, camera, _ = scenes.sphere_field(seed=5, spheres=300, frequency=10)
    camera = Camera(position=camera.position, target=camera.target, fov=camera.fov)
    size, spp = 32, 64
    lums = []
    for seed in range(1, 17):
        _, acc = gpu_frame(scene, camera, size, size, spp, WF, seed=seed)
        lums.append((acc[..., 0] * 0.2126 + acc[..., 1] * 0.7152 + acc[..., 2] * 0.0722) / spp)
    lums = np.array(lums)
    mean = lums.mean(axis=0)
    sigma_mean = lums.std(axis=0, ddof=1) / 4.0
    packed = pack.pack(scene.objects)
    words, powers = host.light_words(packed)
    ref_spp = 4096
    params = host.params(scene, camera, size, size, light_count=len(powers), max_bounces=8, spp=ref_spp,
                         firefly_clamp=0.0)
    acc = oracle.render(packed, words, params)["accum"]
    ref = (acc[..., 0] * 0.2126 + acc[..., 1] * 0.7152 + acc[..., 2] * 0.0722) / ref_spp
    ref_var = np.maximum(acc[..., 3] / ref_spp - ref * ref, 0) / ref_spp
    z = (mean - ref) / np.sqrt(sigma_mean ** 2 + ref_var + 1e-12)
    outside = (np.abs(z) > 3).mean()
    assert outside <= 0.0027 + 0.015, outside
