"""CPU oracle of Raymond's render path — TEST INFRASTRUCTURE ONLY.

A restatement of the reference's algorithms (BVH.build, Scene.raycast,
the trace shader's traversal and, in oracle/pathtrace.cpp, its path
tracer and denoiser; in oracle/pack.py, Scene.#pack; in oracle/host.py,
the Renderer's host tables and uniform block) used only to check the
product, by tests/, __graft_entry__.smoke() and the cpu_baseline and
reference legs of bench.py. Nothing in raymond_gb300 imports it. Parity
status: pinned against the known answers of the reference's own unit
tests; not against executed reference output (no JavaScript engine exists
on either machine)."""

from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB, build

_lib = None
NONE = 0xFFFFFFFF


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        P, U32, I, D, F = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_double, ctypes.c_float
        _lib.ro_bvh_build.restype = U32
        _lib.ro_bvh_build.argtypes = [P, P, U32, U32, P, P]
        _lib.ro_raycast_batch.restype = None
        _lib.ro_raycast_batch.argtypes = [P, U32, P, P, P, U32, D, P, P, P, P, P, I]
        _lib.ro_intersect_double.restype = I
        _lib.ro_intersect_double.argtypes = [P, U32, P, P, D, P]
        _lib.ro_trace32_batch.restype = None
        _lib.ro_trace32_batch.argtypes = [P, P, P, U32, F, I, P, P, P, P, I]
        _lib.ro_surface_double.restype = None
        _lib.ro_surface_double.argtypes = [P, P, U32, P, P, D, D, D, P]
        _lib.ro_render.restype = None
        _lib.ro_render.argtypes = [P, P, P, P, P, P, U32, U32, U32, U32, U32, P, P, P, P, I]
        _lib.ro_render_scene.restype = None
        _lib.ro_render_scene.argtypes = [P, P, P, P, P, P, U32, U32, U32, U32, U32, P, P, P, P, I, P, U32, U32, P, U32,
                                         U32, P, U32, U32, P, U32, U32]
        _lib.ro_light_trace.restype = U32
        _lib.ro_light_trace.argtypes = [P, P, P, P, P, P, P, U32, U32, U32, U32, P, P, P, P, P, P, I]
        _lib.ro_photon_gather.restype = None
        _lib.ro_photon_gather.argtypes = [P, P, P, P, P, P, P, U32, U32, U32, U32, P, P, I]
        _lib.ro_set_jitter.restype = None
        _lib.ro_set_jitter.argtypes = [U32, F]
        _lib.ro_sample_streams.restype = None
        _lib.ro_sample_streams.argtypes = [P, U32, P, U32, U32, U32, P]
        _lib.ro_denoise.restype = None
        _lib.ro_denoise.argtypes = [P, P, P, U32, U32, U32, P, I]
        _lib.ro_display.restype = None
        _lib.ro_display.argtypes = [P, P, P, P]
        _lib.ro_net_param_count.restype = ctypes.c_uint64
        _lib.ro_net_param_count.argtypes = []
        _lib.ro_net_layout.restype = None
        _lib.ro_net_layout.argtypes = [P, P, P, P]
        _lib.ro_net_loss_grad.restype = D
        _lib.ro_net_loss_grad.argtypes = [P, P, P, P, P, P, U32, U32, U32, I, D, D, D, P, P]
        _lib.ro_conv3x3.restype = None
        _lib.ro_conv3x3.argtypes = [I, U32, U32, U32, P, U32, U32, P, U32, U32, P, P, P, P, I, P, P, P]
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def threads() -> int:
    return os.cpu_count() or 1


def bvh_build(mins, maxs, max_leaf=4):
    """BVH.build (src/BVH.mjs:57-234): returns (nodes u32 (n*8,), order u32)."""
    mins = np.ascontiguousarray(mins, dtype=np.float64).reshape(-1)
    maxs = np.ascontiguousarray(maxs, dtype=np.float64).reshape(-1)
    count = mins.size // 3
    nodes = np.zeros(max(1, 2 * count - 1) * 8, dtype=np.uint32)
    order = np.zeros(count, dtype=np.uint32)
    n = lib().ro_bvh_build(_p(mins), _p(maxs), count, max_leaf, _p(nodes), _p(order))
    return nodes[: n * 8].copy(), order


def raycast(packed, rays, t_max=np.inf, nthreads=None):
    """Scene.raycast in double on the packed scene: dict of prim, t, uv, normal, front."""
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
    n = len(rays)
    prim = np.empty(n, dtype=np.uint32)
    t = np.empty(n, dtype=np.float64)
    uv = np.empty(2 * n, dtype=np.float64)
    normal = np.empty(3 * n, dtype=np.float64)
    front = np.empty(n, dtype=np.uint8)
    attrs = np.ascontiguousarray(packed.attributes, dtype=np.float32)
    lib().ro_raycast_batch(_p(packed.primitives), packed.primitiveCount, _p(packed.nodes), _p(attrs), _p(rays), n,
                           float(t_max), _p(prim), _p(t), _p(uv), _p(normal), _p(front), nthreads or threads())
    return {"prim": prim, "t": t, "uv": uv.reshape(-1, 2), "normal": normal.reshape(-1, 3), "front": front}


def intersect_double(packed, p, o, d, t_max=np.inf):
    o = np.ascontiguousarray(o, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.zeros(3, dtype=np.float64)
    hit = lib().ro_intersect_double(_p(packed.primitives), int(p), _p(o), _p(d), float(t_max), _p(out))
    return out if hit else None


def trace32(packed, rays, t_max=1e30, any_hit=False, nthreads=None):
    """The trace shader's traversal in f32, with counters: dict prim, t, inner, tested."""
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
    n = len(rays)
    prim = np.empty(n, dtype=np.uint32)
    t = np.empty(n, dtype=np.float32)
    inner = np.empty(n, dtype=np.uint32)
    tested = np.empty(n, dtype=np.uint32)
    lib().ro_trace32_batch(_p(packed.primitives), _p(packed.nodes), _p(rays), n, float(t_max), 1 if any_hit else 0,
                           _p(prim), _p(t), _p(inner), _p(tested), nthreads or threads())
    return {"prim": prim, "t": t, "inner": inner, "tested": tested}


def bytes_per_ray(inner: np.ndarray, tested: np.ndarray) -> np.ndarray:
    """Algorithmic bytes of one traversal: the root box, both child boxes of
    every inner node visited, and every primitive record tested:
    32·(1 + 2·inner) + 64·tested."""
    return 32 * (1 + 2 * inner.astype(np.int64)) + 64 * tested.astype(np.int64)


def render(packed, lights_words, params: bytes, region=None, seed_hash=0, nthreads=None, environment=None,
           textures=None, normal_maps=None):
    """One frame of the trace shader's main() restated in f32 over a region
    (x0, y0, w, h) of the image: dict accum/albedo/normal (h×w×4 sums) and
    counters (algorithmic bytes, rays, surface hits, paths). As the renderer
    uploads them, or None: `environment` (RGBA half floats, width, height,
    importance table dict), `textures` and `normal_maps` (RGBA bytes of
    every layer, width, height)."""
    import struct
    width, height = struct.unpack_from("<2I", params, 160)
    x0, y0, rw, rh = region if region else (0, 0, width, height)
    accum = np.zeros(rw * rh * 4, dtype=np.float32)
    alb = np.zeros(rw * rh * 4, dtype=np.float32)
    nrm = np.zeros(rw * rh * 4, dtype=np.float32)
    counters = np.zeros(8, dtype=np.uint64)
    pbuf = np.frombuffer(bytes(params), dtype=np.uint8).copy()
    words = np.ascontiguousarray(lights_words, dtype=np.uint32)
    attrs = np.ascontiguousarray(packed.attributes, dtype=np.float32)
    args = (_p(packed.primitives), _p(packed.nodes), _p(packed.materials), _p(attrs), _p(words), _p(pbuf),
            seed_hash, x0, y0, rw, rh, _p(accum), _p(alb), _p(nrm), _p(counters), nthreads or threads())
    if environment is None and textures is None and normal_maps is None:
        lib().ro_render(*args)
    else:
        keep = []  # the arrays the call reads, alive until it returns

        def arr(a, dtype):
            keep.append(np.ascontiguousarray(a, dtype=dtype))
            return _p(keep[-1])

        env = (None, 0, 0, None, 0, 0)
        if environment is not None:
            rgba, ew, eh, table = environment
            env = (arr(rgba, np.uint16), ew, eh, arr(table["data"], np.float32), table["width"], table["height"])
        tex = (None, 0, 0) if textures is None else (arr(textures[0], np.uint8), textures[1], textures[2])
        nmaps = (None, 0, 0) if normal_maps is None else (arr(normal_maps[0], np.uint8), normal_maps[1],
                                                          normal_maps[2])
        lib().ro_render_scene(*args, *env, *tex, *nmaps)
    return {"accum": accum.reshape(rh, rw, 4), "albedo": alb.reshape(rh, rw, 4), "normal": nrm.reshape(rh, rw, 4),
            "bytes": int(counters[0]), "rays": int(counters[1]), "hits": int(counters[2]), "paths": int(counters[3]),
            "trav_closest": int(counters[4]), "trav_shadow": int(counters[5]), "rays_closest": int(counters[6]),
            "rays_shadow": int(counters[7])}


def light_trace(packed, lights_words, params: bytes, emitters, photons, seed_hash=0, nthreads=None, ids=None,
                margins=False):
    """One frame of light_trace (src/shaders.mjs:1628-1814) for its photons
    0..photons-1, or the range ids = (first, count) of them: dict splats
    (h×w×4 u32 fixed-point sums, 1/65536 units), photons (n×9 float32:
    where each landed, its power, the direction it came from), in photon
    order, photon_ids (each one's light path), photon_splats (n×4 u32: the
    pixel each splatted into, or NONE, and the fixed-point amounts) and
    with margins, photon_margins (the smallest edge margin of the
    primitives each photon's path hit, 0 where a hit tied with another
    primitive's) and path_margins (that margin for every path
    id0..id0+count-1, 1 where a path hit nothing); margins cost a second
    traversal per hit."""
    import struct
    width, height = struct.unpack_from("<2I", params, 160)
    splats = np.zeros(width * height * 4, dtype=np.uint32)
    id0, count = ids if ids is not None else (0, int(photons))
    out = np.zeros(max(int(count), 1) * 9, dtype=np.float32)
    ids_out = np.zeros(max(int(count), 1), dtype=np.uint32)
    splat_out = np.zeros(max(int(count), 1) * 4, dtype=np.uint32)
    margin_out = np.zeros(max(int(count), 1), dtype=np.float32) if margins else None
    path_margins = np.ones(max(int(count), 1), dtype=np.float32) if margins else None
    pbuf = np.frombuffer(bytes(params), dtype=np.uint8).copy()
    words = np.ascontiguousarray(lights_words, dtype=np.uint32)
    attrs = np.ascontiguousarray(packed.attributes, dtype=np.float32)
    em = np.ascontiguousarray(emitters, dtype=np.float32)
    n = lib().ro_light_trace(_p(packed.primitives), _p(packed.nodes), _p(packed.materials), _p(attrs), _p(words),
                             _p(pbuf), _p(em), int(photons), int(id0), int(count), seed_hash, _p(splats), _p(out),
                             _p(ids_out), _p(splat_out), _p(margin_out), _p(path_margins), nthreads or threads())
    return {"splats": splats.reshape(height, width, 4), "photons": out[: n * 9].reshape(n, 9),
            "photon_ids": ids_out[:n], "photon_splats": splat_out[: n * 4].reshape(n, 4),
            "photon_margins": margin_out[:n] if margins else None,
            "path_margins": path_margins[: int(count)] if margins else None, "first_id": int(id0)}


def photon_gather(packed, lights_words, params: bytes, photons, seed_hash=0, nthreads=None, rows=None, visits=False):
    """One frame of photon_gather (src/shaders.mjs:1585-1626), on every row
    or rows = (first, count): the caustic light the photon map adds to each
    pixel (h×w×4 float32 sums); with visits, also each pixel's count of
    photons visited (h×w; the gather stops at 4096), as (light, visits)."""
    import struct
    width, height = struct.unpack_from("<2I", params, 160)
    accum = np.zeros(width * height * 4, dtype=np.float32)
    ph = np.ascontiguousarray(photons, dtype=np.float32).reshape(-1)
    if ph.size == 0:
        ph = np.zeros(9, np.float32)  # a valid address; the count passed is 0
        count = 0
    else:
        count = ph.size // 9
    pbuf = np.frombuffer(bytes(params), dtype=np.uint8).copy()
    words = np.ascontiguousarray(lights_words, dtype=np.uint32)
    attrs = np.ascontiguousarray(packed.attributes, dtype=np.float32)
    vis = np.zeros(width * height, dtype=np.uint32) if visits else None
    lib().ro_photon_gather(_p(packed.primitives), _p(packed.nodes), _p(packed.materials), _p(attrs), _p(words),
                           _p(pbuf), _p(ph), count,
                           *(rows if rows is not None else (0, height)), seed_hash, _p(accum), _p(vis),
                           nthreads or threads())
    if visits:
        return accum.reshape(height, width, 4), vis.reshape(height, width)
    return accum.reshape(height, width, 4)


class jitter:
    """Perturbation runs (oracle/pathtrace.cpp, nudge): inside the block
    every ray the oracle traces has its origin and direction scaled
    componentwise by 1 ± size, signs hashed from the ray and `seed`; seeds
    2k and 2k + 1 nudge each ray opposite ways. Results that move under it
    rest on a near-tie decision, where rounding may send the GPU the other
    way. Not thread-safe across concurrent oracle calls."""

    def __init__(self, seed: int, size: float):
        self.seed, self.size = int(seed), float(size)

    def __enter__(self):
        lib().ro_set_jitter(self.seed, self.size)
        return self

    def __exit__(self, *exc):
        lib().ro_set_jitter(0, 0.0)
        return False


def sample_streams(pairs, dim_ids, chain, seed_hash=0):
    """The oracle's sample streams (src/shaders.mjs:135-212 and the seedings
    at :1585, :1638, :1852-1859) in raymond_sample_streams's layout: per
    (pixel index, sample index) pair, rand2() and rand() at each dimension
    id, the spectrum position, `chain` light-path draws, `chain` gather draws."""
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
    dims = np.ascontiguousarray(dim_ids, dtype=np.uint32).reshape(-1)
    per = 3 * dims.size + 1 + 2 * int(chain)
    out = np.zeros((len(pairs), per), dtype=np.float32)
    lib().ro_sample_streams(_p(pairs), len(pairs), _p(dims) if dims.size else None, dims.size, int(chain), int(seed_hash),
                            _p(out))
    return out


def denoise(accum, guide_albedo, guide_normal, width, height, total_samples, nthreads=None):
    """prepare, five à-trous passes and compose (src/shaders.mjs:1974-2097): h×w×4."""
    out = np.zeros(width * height * 4, dtype=np.float32)
    a = np.ascontiguousarray(accum, dtype=np.float32)
    g = np.ascontiguousarray(guide_albedo, dtype=np.float32)
    n = np.ascontiguousarray(guide_normal, dtype=np.float32)
    lib().ro_denoise(_p(a), _p(g), _p(n), width, height, total_samples, _p(out), nthreads or threads())
    return out.reshape(height, width, 4)


def display(accum, denoised, params: bytes):
    """The display pass (src/shaders.mjs:2124-2152) into RGBA8."""
    import struct
    width, height = struct.unpack_from("<2I", params, 160)
    out = np.zeros(width * height * 4, dtype=np.uint8)
    a = np.ascontiguousarray(accum, dtype=np.float32)
    d = np.ascontiguousarray(denoised if denoised is not None else accum, dtype=np.float32)
    pbuf = np.frombuffer(bytes(params), dtype=np.uint8).copy()
    lib().ro_display(_p(a), _p(d), _p(pbuf), _p(out))
    return out.reshape(height, width, 4)


def surface_double(packed, p, o, d, t, u, v):
    """Scene.raycast's surface frame at a hit: dict geometric, shading (unflipped), uv, tangent, up."""
    out = np.zeros(14)
    o = np.ascontiguousarray(o, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    attrs = np.ascontiguousarray(packed.attributes, dtype=np.float32)
    lib().ro_surface_double(_p(packed.primitives), _p(attrs), int(p), _p(o), _p(d), float(t), float(u), float(v),
                            _p(out))
    return {"geometric": out[0:3], "shading": out[3:6], "uv": out[6:8], "tangent": out[8:11], "up": out[11:14]}


# ---- the learned denoiser's network (oracle/net.cpp) ----

def net_layout():
    """Per layer (weight offset, bias offset, cin, cout) of the flat parameter vector."""
    L = lib()
    wo = np.zeros(19, np.uint64)
    bo = np.zeros(19, np.uint64)
    ci = np.zeros(19, np.uint32)
    co = np.zeros(19, np.uint32)
    L.ro_net_layout(_p(wo), _p(bo), _p(ci), _p(co))
    return int(L.ro_net_param_count()), [(int(wo[i]), int(bo[i]), int(ci[i]), int(co[i])) for i in range(19)]


def net_loss_grad(params, accum, albedo, normal, target, samples, bf16=False, grads=True, out=False, w_log=1.0,
                  w_rel=0.0, rel_eps=0.01):
    """Loss, gradients (float64, or None) and the network output ([n,h,w,16] float32, or None)
    for n images of h×w (float4 arrays [n,h,w,4] as a renderer accumulates them)."""
    L = lib()
    params = np.ascontiguousarray(params, dtype=np.float64)
    accum = np.ascontiguousarray(accum, dtype=np.float32)
    n, h, w = accum.shape[:3]
    albedo = np.ascontiguousarray(albedo, dtype=np.float32)
    normal = np.ascontiguousarray(normal, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    samples = np.ascontiguousarray(np.broadcast_to(np.asarray(samples, np.float32), (n,)))
    g = np.zeros(params.size, np.float64) if grads else None
    o = np.zeros((n, h, w, 16), np.float32) if out else None
    loss = L.ro_net_loss_grad(_p(params), _p(accum), _p(albedo), _p(normal), _p(target), _p(samples), n, h, w,
                              1 if bf16 else 0, float(w_log), float(w_rel), float(rel_eps), _p(g), _p(o))
    return loss, g, o


def conv3x3(mode, src0, weight, bias=None, src1=None, shift0=0, dy=None, mask=None, act=0):
    """One 3×3 convolution in double: mode 0 forward, 1 input gradient, 2 weight/bias gradient.
    src0 [n,h0,w0,c0] (h0 = h/2 when shift0), src1 [n,h,w,c1], weight [cout,9,cin]."""
    L = lib()
    src0 = np.ascontiguousarray(src0, dtype=np.float32)
    n = src0.shape[0]
    c0 = src0.shape[3]
    if src1 is not None:
        src1 = np.ascontiguousarray(src1, dtype=np.float32)
        h, w, c1 = src1.shape[1], src1.shape[2], src1.shape[3]
    else:
        h, w, c1 = src0.shape[1] << shift0, src0.shape[2] << shift0, 0
    weight = np.ascontiguousarray(weight, dtype=np.float32)
    cout = weight.shape[0]
    cin = c0 + c1
    bias = None if bias is None else np.ascontiguousarray(bias, dtype=np.float32)
    dy = None if dy is None else np.ascontiguousarray(dy, dtype=np.float32)
    mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    out = dw = db = None
    if mode == 0:
        out = np.zeros((n, h, w, cout), np.float32)
    elif mode == 1:
        out = np.zeros((n, h, w, cin), np.float32)
    else:
        dw = np.zeros((cout, 9, cin), np.float64)
        db = np.zeros(cout, np.float64)
    L.ro_conv3x3(mode, n, h, w, _p(src0), c0, shift0, _p(src1), c1, cout, _p(weight), _p(bias), _p(dy), _p(mask),
                 act, _p(out), _p(dw), _p(db))
    return out if mode != 2 else (dw, db)
