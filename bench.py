#!/usr/bin/env python
"""Benchmark of the render path on the sphere-field workload: 1024×1024,
8 bounces, NEE+MIS, Russian roulette from bounce 3, FP32 accumulation, the
à-trous denoiser on (the renderer's default), 10,000 spheres on a 40×40
ground around a 499,280-triangle displaced geodesic sphere, gradient sky and
a 0.27° sun. A step is one frame, Renderer.render(): the trace, the
denoiser and the tone map. Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--spp S] [--impl ours|reference]

The default line also carries "learned_denoiser": the learned denoiser's
inference on a 1920×1080 frame of the same scene against the tensor peak;
and "time_to_rmse": the wall time to RMSE ≤ 0.01 against a 16,384-spp
render of the scene, for the one-kernel path with the à-trous filter, the
wavefront path's raw running average, and the wavefront path with the
learned denoiser on the display (about 45 s; --no-rmse skips it).
Other workloads (--workload):
  caustics the water-caustics scene at 1024² with light tracing (1M light paths
           splatted) and photon mapping (up to 4M photons, r = 0.01) every frame
  batch    64 seeded sphere-field instances as one graph-replayed batched frame
  denoise  the learned denoiser's 1080p inference as its own line
  primary  closest hits of the Cornell room's 256² jittered primary rays, one
           traversal launch per step (--size sets the image side)
  bvh      the scene producer: BVH.build over the sphere field's primitive
           boxes on the host cores (no GPU), against the oracle's build
  rmse     the time-to-RMSE measurement alone, as its own line

Under torchrun each rank renders its own copy of the frame (replicas; the
scene does not shard across GPUs here): value = paths of all ranks ÷ the
slowest rank's time.
"""

from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpaths/s"
WORKLOAD = "sphere field 1024x1024, 8 bounces, NEE+MIS, RR from bounce 3, a-trous on"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_throughput(units_per_step, steps, seconds, world, device):
    """Whole-job rate of `world` independent replicas, each doing the same
    fixed work per step: all ranks' units over the slowest rank's time (the
    job ends when its last replica does). Returns (units per second, the
    time used)."""
    if world > 1:
        import torch

        t = torch.tensor([seconds], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        seconds = float(t.item())
    return units_per_step * steps * world / seconds, seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": max(maxes) if maxes else None,
                "reasons": sorted(reasons), "samples": len(sms)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# k_wf_extend's measured traffic per path on the sphere field (ncu, 512²
# frame, 4-wide tree): DRAM read + write, bytes through L2, and the mean
# share of active lanes per executed instruction.
EXTEND_DRAM_BYTES_PER_PATH = (227_195_392 + 53_279_232) / 1_048_576
EXTEND_L2_BYTES_PER_PATH = 5_481_172_960 / 1_048_576
EXTEND_LANES_PER_INSTRUCTION = 11.7

CAUSTICS_WORKLOAD = ("water caustics 1024x1024 (130,050-triangle water surface, glass sphere, r=0.1 lamp), "
                     "8 bounces, 1M light paths splatted + photon map of up to 4M photons gathered at r=0.01")
CAUSTICS_LIGHT_PATHS = 1_000_000
CAUSTICS_PHOTONS = 4_194_304
CAUSTICS_RADIUS = 0.01


def build_workload(size, spp, bounces, workload="field"):
    import raymond_gb300 as rg
    from raymond_gb300 import scenes

    if workload == "caustics":
        return scenes.water_caustics()
    scene, camera, info = scenes.sphere_field()
    return scene, camera, info


class OracleScene:
    """A workload scene as the oracle packs it (oracle/pack.py: Scene.#pack
    restated) with its lights table, delta objects and emitters
    (oracle/host.py: Renderer's host tables restated). Nothing here touches
    the product's library, so the reference arm maps only the oracle's."""

    def __init__(self, scene):
        from oracle import host, pack

        self.scene = scene
        self.packed = pack.pack(scene.objects)
        self.words, self.powers = host.light_words(self.packed)
        self.deltas = host.delta_objects(scene.objects, self.packed)

    def params(self, camera, width, height, spp, bounces, **kw) -> bytes:
        from oracle import host

        return host.params(self.scene, camera, width, height, light_count=len(self.powers),
                           volume_count=len(self.packed.volumes), max_bounces=bounces, spp=spp, **kw)

    def emitters(self):
        from oracle import host

        return host.emitters(self.powers, self.deltas, self.scene.sky, len(self.powers))


def band_starts(height, bands, rows):
    """First rows of `bands` bands of `rows` rows centred at the middles of
    equal slices of the image, so a sample is not biased towards its top
    rows (sky, where paths end after one bounce)."""
    return [max(0, min(height - rows, ((2 * k + 1) * height) // (2 * bands) - rows // 2)) for k in range(bands)]


def oracle_sample(osc, params: bytes, width, height, rows_per_band, bands, threads, detail=False):
    """The oracle's f32 path tracer on `bands` bands spread down the image:
    returns (paths, seconds, algorithmic bytes per path, rays per path), and
    with detail the per-path closest-hit and shadow traversal bytes too."""
    import oracle

    tot = {"paths": 0, "bytes": 0, "rays": 0, "trav_closest": 0, "trav_shadow": 0, "rays_closest": 0,
           "rays_shadow": 0}
    t0 = time.perf_counter()
    for y0 in band_starts(height, bands, rows_per_band):
        r = oracle.render(osc.packed, osc.words, params, region=(0, y0, width, rows_per_band), nthreads=threads)
        for key in tot:
            tot[key] += r[key]
    secs = time.perf_counter() - t0
    p = max(tot["paths"], 1)
    out = (tot["paths"], secs, tot["bytes"] / p, tot["rays"] / p)
    if detail:
        return out + ({k: tot[k] / p for k in ("trav_closest", "trav_shadow", "rays_closest", "rays_shadow")},)
    return out


def caustics_cpu_sample(osc, camera, size, spp, bounces, threads, strips=16, rows=2):
    """The oracle's frame of the caustics workload on a bounded sample: the
    camera paths (leaving caustic paths to light tracing) on `strips` bands
    of `rows` rows, the same fraction of the frame's light paths (splatted
    and deposited), and the photon map's gather on the bands. Returns
    (camera paths, light paths, seconds)."""
    import numpy as np

    import oracle

    emitters = osc.emitters()
    block = bytearray(osc.params(camera, size, size, spp, bounces, caustics=emitters is not None, deltas=osc.deltas))
    f = np.frombuffer(block, dtype=np.float32)
    f[48], f[49] = CAUSTICS_RADIUS, 2 * CAUSTICS_RADIUS  # the fixed radius the GPU run sets
    params = bytes(block)
    light_paths = CAUSTICS_LIGHT_PATHS * strips * rows // size
    paths = 0
    starts = band_starts(size, strips, rows)
    t0 = time.perf_counter()
    for y0 in starts:
        r = oracle.render(osc.packed, osc.words, params, region=(0, y0, size, rows), nthreads=threads)
        paths += r["paths"]
    if emitters is not None:
        lt = oracle.light_trace(osc.packed, osc.words, params, emitters, CAUSTICS_LIGHT_PATHS, ids=(0, light_paths),
                                nthreads=threads)
        for y0 in starts:
            oracle.photon_gather(osc.packed, osc.words, params, lt["photons"], rows=(y0, rows), nthreads=threads)
    return paths, light_paths, time.perf_counter() - t0


def device_view(torch, ptr, shape, device):
    """A device float32 buffer of the library's (a renderer's) as a torch tensor, without a copy."""

    class _View:
        pass

    v = _View()
    v.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False), "version": 3,
                                  "strides": None}
    return torch.as_tensor(v, device=f"cuda:{device}")


def measured_peak_tensor():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured (burst)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def measured_peak_tensor_sustained():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops_sustained"]), "measured (sustained)"
    except (OSError, KeyError, ValueError):
        return 1700.0, "fallback"


def denoiser_flops(width, height):
    """Algorithmic FLOPs of one learned-denoiser frame: Σ over the 19 convolutions
    of 2·H_l·W_l·C_in·C_out·9, with the 12 real input and 3 real output channels."""
    from raymond_gb300.denoiser import Denoiser  # noqa: F401  (layer table lives in the library)
    import oracle

    _, layout = oracle.net_layout()
    levels = [0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0]
    total = 0.0
    for li, (_, _, cin, cout) in enumerate(layout):
        cin = 12 if li == 0 else cin
        cout = 3 if li == 18 else cout
        px = (width / 2 ** levels[li]) * (height / 2 ** levels[li])
        total += 2.0 * px * cin * cout * 9
    return total


def measure_denoiser(scene, camera, local, steps, warmup, width=1920, height=1080, spp=4):
    """The learned denoiser's inference on a width×height frame of the scene,
    inputs resident in HBM: mean ms per frame (CUDA events on the network's
    stream, L2 flushed between steps), TFLOP/s against the tensor peak, the
    end-to-end time with host buffers, and the CPU oracle's rate."""
    import numpy as np
    import torch

    import raymond_gb300 as rg
    from raymond_gb300 import _native
    from raymond_gb300.denoiser import DEFAULT_WEIGHTS, Denoiser, make_batch

    r = rg.Renderer.create(rg.Canvas(width, height), device=local)
    r.scene, r.camera = scene, camera
    r.caustics = False
    r.denoise = False
    r.samplesPerFrame = spp
    r.render()
    r.device.queue.onSubmittedWorkDone()
    bufs = _native.Buffers()
    _native.check(_native.lib().raymond_get_buffers(r.handle, bufs), r.handle)
    shape = (1, height, width, 4)
    acc, alb, nrm = (device_view(torch, p, shape, local) for p in (bufs.accum, bufs.guide_albedo, bufs.guide_normal))
    net = Denoiser(device=local, weights=DEFAULT_WEIGHTS)
    out = torch.empty(shape, dtype=torch.float32, device=f"cuda:{local}")
    batch = make_batch(acc, alb, nrm, samples_all=float(r.samples))
    # The network runs on a torch-owned stream, so torch's allocators never
    # hold on to a stream that the library destroys.
    stream = torch.cuda.Stream(device=local)
    torch.cuda.synchronize()
    net.use_stream(stream.cuda_stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    for _ in range(max(warmup, 3)):
        net.infer(batch, out)
    net.sync()
    ms = []
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        net.infer(batch, out)
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    flops = denoiser_flops(width, height)
    peak, peak_kind = measured_peak_tensor()
    sustained, _ = measured_peak_tensor_sustained()
    frame_s = statistics.mean(ms) / 1e3
    achieved = flops / frame_s / 1e12

    # End to end: host (pinned) buffers in, the denoised image out.
    host = [x.cpu().pin_memory() for x in (acc, alb, nrm)]
    dev = [torch.empty(shape, dtype=torch.float32, device=f"cuda:{local}") for _ in range(3)]
    res = torch.empty(shape, dtype=torch.float32).pin_memory()
    e2e_steps = max(3, steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        with torch.cuda.stream(stream):
            for d, h in zip(dev, host):
                d.copy_(h, non_blocking=True)
        net.infer(make_batch(*dev, samples_all=float(r.samples)), out)
        with torch.cuda.stream(stream):
            res.copy_(out, non_blocking=True)
        stream.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps

    # CPU: the oracle's network forward (double, one thread) on a 32×32 crop.
    import oracle

    crop = [np.ascontiguousarray(x[0, :32, :32].cpu().numpy()) for x in (acc, alb, nrm)]
    params = net.get_params().astype(np.float64)
    t0 = time.perf_counter()
    oracle.net_loss_grad(params, crop[0][None], crop[1][None], crop[2][None], crop[0][None], float(r.samples),
                         grads=False)
    cpu_s = (time.perf_counter() - t0) * (width * height) / (32 * 32)
    torch.cuda.synchronize()
    del host, dev, res, out, flush, acc, alb, nrm
    net.use_stream(None)
    net.dispose()
    r.dispose()
    return {
        "workload": f"learned denoiser, {width}x{height} frame of the sphere field at {spp} spp",
        "ms_per_frame": statistics.mean(ms), "frames_per_s": 1.0 / frame_s,
        "launches_per_frame": 25,
        "roofline": {"bound": "tensor", "kernel": "k_conv_halo (19 launches, whole inference)", "achieved": achieved,
                     "peak": peak, "peak_kind": peak_kind, "unit": "TFLOP/s", "frac": achieved / peak,
                     "frac_of_sustained": achieved / sustained, "peak_sustained": sustained,
                     "flops_per_frame": flops, "traffic": None},
        "e2e": {"value": 1.0 / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": 3 * width * height * 16,
                "d2h_bytes_per_step": width * height * 16},
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "frames/s", "cores": 1, "kind": "port",
                         "sample": "oracle network forward on a 32x32 crop, scaled by pixels"},
        "l2": "flushed between steps (512 MB write)",
        "training": training_note(),
    }


def training_note():
    """How the shipped weights were trained, against the configured data set
    (2,000 crops of 256² rendered at 1–8 spp with 16,384-spp targets): read
    from the training report that sits beside the weights."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "raymond_gb300", "weights", "denoiser_unet.json")
    try:
        with open(path) as f:
            rep = json.load(f)
    except (OSError, ValueError):
        return None
    views, size, target = int(rep["views"]), int(rep["size"]), int(rep["target_spp"])
    noisy = [int(s) for s in rep["noisy_spp"]]
    return {
        "views": views, "crop_px": size, "target_spp": target, "input_spp": noisy, "adam_steps": int(rep["steps"]),
        "field_spheres": rep.get("field_spheres"), "field_mesh_frequency": rep.get("field_frequency"),
        "paths": views * size * size * (target + sum(noisy)),
        "configured": "2,000 crops of 256x256 at 1-8 spp with 16,384-spp targets",
        "configured_paths": 2000 * 256 * 256 * (16384 + 8),
        "note": "a reduced data set (about 1/7 of the configured paths), with inputs up to 512 spp",
    }


def run_denoise(args, local):
    """The learned denoiser's 1080p inference as its own bench line."""
    scene, camera, info = build_workload(args.size, args.spp, args.bounces)
    clocks = ClockSampler(local)
    clocks.start()
    d = measure_denoiser(scene, camera, local, args.steps, args.warmup)
    clock_info = clocks.stop()
    return {
        "metric": "learned-denoiser frames/s at 1920x1080", "value": d["frames_per_s"], "unit": "frames/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": d["ms_per_frame"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded mulberry32 scene, rendered at 4 spp)",
        "config": {"workload": d["workload"], "l2": d["l2"], "weights": "raymond_gb300/weights/denoiser_unet.npz",
                   "training": d["training"]},
        "e2e": d["e2e"], "gpu_launches": d["launches_per_frame"] * args.steps, "roofline": d["roofline"],
        "cpu_baseline": d["cpu_baseline"], "clocks": clock_info,
    }


PRIMARY_WORKLOAD = "Cornell room 256x256, one jittered primary ray per pixel (mulberry32 seed 1), closest hit"


L2_NOTE = "GPU arm: flushed between steps (512 MB write); CPU arm: not applicable"


def primary_config(rays):
    return {"workload": PRIMARY_WORKLOAD, "rays": rays, "l2": L2_NOTE}


def primary_case(size):
    """The Cornell primary-ray case: the room, its f32 camera rays, the
    oracle's packing of the room, and the algorithmic bytes of tracing the
    rays counted by the oracle's f32 traversal: 32·(1 + 2·inner nodes
    visited) + 64·primitives tested per ray."""
    import oracle
    from oracle import pack
    from raymond_gb300 import scenes

    scene, camera, rays = scenes.cornell_primary(size, seed=1)
    packed = pack.pack(scene.objects)
    counts = oracle.trace32(packed, rays)
    return scene, packed, rays, counts, int(oracle.bytes_per_ray(counts["inner"], counts["tested"]).sum())


def primary_cpu(packed, rays, seconds=1.0):
    """Scene.raycast restated in double (oracle/raycast.cpp) on all host
    cores, repeated over the whole ray set for about `seconds`: Mrays/s."""
    import oracle

    threads = os.cpu_count() or 1
    oracle.raycast(packed, rays[:1024], nthreads=threads)
    done, t0 = 0, time.perf_counter()
    while True:
        oracle.raycast(packed, rays, nthreads=threads)
        done += len(rays)
        dt = time.perf_counter() - t0
        if dt >= seconds:
            return done / dt / 1e6, threads, dt


def run_primary(args, local):
    """Closest hits of the Cornell room's 65,536 primary rays: one traversal
    launch per step, rays resident in HBM and L2 flushed between steps
    (device time by CUDA events on the renderer's stream); end to end
    through Renderer.tracePrimary with host arrays."""
    import numpy as np
    import torch

    import oracle
    import raymond_gb300 as rg
    from raymond_gb300 import _native

    size = 256 if args.size == 1024 else args.size
    scene, packed, rays, counts, algo_bytes = primary_case(size)
    n = len(rays)
    r = rg.Renderer.create(rg.Canvas(1, 1), device=local)
    r.tracePrimary(rays[:32], scene)  # uploads the scene
    lib = _native.lib()
    stream = torch.cuda.ExternalStream(lib.raymond_get_stream(r.handle), device=f"cuda:{local}")
    d_rays = torch.from_numpy(rays).to(f"cuda:{local}")
    d_prim = torch.empty(n, dtype=torch.int32, device=f"cuda:{local}")
    d_t = torch.empty(n, dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def launch():
        _native.check(lib.raymond_trace_primary_device(r.handle, d_rays.data_ptr(), n, d_prim.data_ptr(),
                                                       d_t.data_ptr()), r.handle)

    for _ in range(max(args.warmup, 3)):
        launch()
    _native.check(lib.raymond_sync(r.handle), r.handle)
    clocks = ClockSampler(local)
    clocks.start()
    ms = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        launch()
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    clock_info = clocks.stop()
    prim = d_prim.cpu().numpy().view(np.uint32)
    agree = float(np.mean(prim == counts["prim"]))

    # End to end: numpy rays in, numpy hits out, through the public call.
    e2e_steps = max(args.steps, 10)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        r.tracePrimary(rays, scene)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    del d_rays, d_prim, d_t, flush
    r.dispose()

    launch_s = statistics.mean(ms) / 1e3
    peak, peak_kind = measured_peak_hbm()
    achieved = algo_bytes / launch_s / 1e9
    cpu_value, cores, cpu_s = primary_cpu(packed, rays)
    return {
        "metric": "Mrays/s (primary, closest hit)", "value": n / launch_s / 1e6, "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32 jitter)",
        "config": primary_config(n),
        "hits_equal_to_oracle_f32": agree,
        "e2e": {"value": n / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 24 * n,
                "d2h_bytes_per_step": 8 * n},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_trace_primary", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "algorithmic_bytes_per_launch": algo_bytes,
                     "note": "algorithmic bytes are node and primitive reads that the 8-primitive room serves "
                             "from L1; the launch is latency-bound"},
        "cpu_baseline": {"value": cpu_value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"oracle Scene.raycast (double) over all {n} rays, repeated for {cpu_s:.1f} s"},
        "clocks": clock_info,
    }


def run_primary_reference(args, rank, world):
    if rank != 0:
        return None
    size = 256 if args.size == 1024 else args.size
    scene, packed, rays, _, _ = primary_case(size)
    times = []
    value = 0.0
    for _ in range(args.steps):
        value, cores, dt = primary_cpu(packed, rays, seconds=0.5)
        times.append(dt)
    return {
        "metric": "Mrays/s (primary, closest hit)", "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mulberry32 jitter)", "impl": "reference",
        "config": primary_config(len(rays)),
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"oracle Scene.raycast (double) over all {len(rays)} rays for 0.5 s per step"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def field_boxes():
    """The sphere field's primitive boxes as Scene.#pack hands them to
    BVH.build (the oracle's packing, oracle/pack.py): (mins, maxs), f64."""
    import numpy as np

    import oracle
    from oracle import pack
    from raymond_gb300 import scenes

    captured = {}

    def capture(mins, maxs):
        captured["mins"], captured["maxs"] = np.array(mins, dtype=np.float64), np.array(maxs, dtype=np.float64)
        return oracle.bvh_build(mins, maxs)

    scene, _, _ = scenes.sphere_field()
    pack.pack(scene.objects, bvh_build=capture)
    return captured["mins"], captured["maxs"]


def bvh_config(count):
    return {"workload": f"binned-SAH BVH of the sphere field's {count} primitive boxes, leaves of at most 4"}


def run_bvh(args):
    """The scene producer beside the path: BVH.build's binned SAH over the
    sphere field's 509,281 primitive boxes, natively on all host cores and on
    one, against the oracle's single-threaded restatement of the same build
    (src/BVH.mjs:57-234), whose nodes and leaf order must come out identical."""
    import numpy as np

    import oracle
    from raymond_gb300 import scene as scene_mod

    mins, maxs = field_boxes()
    count = len(mins)
    threads = os.cpu_count() or 1

    def timed(fn, reps):
        best = math.inf
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            best = min(best, time.perf_counter() - t0)
        return best, out

    for _ in range(max(args.warmup, 1)):
        scene_mod.BVH.build(mins, maxs, threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        b = scene_mod.BVH.build(mins, maxs, threads=threads)
        times.append(time.perf_counter() - t0)
    one_s, _ = timed(lambda: scene_mod.BVH.build(mins, maxs, threads=1), 2)
    ref_s, (nodes, order) = timed(lambda: oracle.bvh_build(mins, maxs), 1)
    same = bool(np.array_equal(nodes, b.nodes) and np.array_equal(order, b.order))
    value = count / statistics.median(times) / 1e6
    return {
        "metric": "Mprims/s (BVH build)", "value": value, "unit": "Mprims/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(times), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64 build, f32 nodes",
        "data": "synthetic (seeded mulberry32 scene)",
        "config": bvh_config(count), "threads": threads, "nodes": int(b.nodeCount), "identical_to_oracle": same,
        "single_thread": {"value": count / one_s / 1e6, "unit": "Mprims/s", "ms": 1e3 * one_s},
        "e2e": {"value": value, "unit": "Mprims/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        "cpu_baseline": {"value": count / ref_s / 1e6, "unit": "Mprims/s", "cores": 1, "kind": "port",
                         "sample": f"oracle BVH.build restatement over all {count} boxes, once"},
    }


def run_bvh_reference(args):
    """The reference arm of the BVH line: the oracle's restatement of
    BVH.build (src/BVH.mjs:57-234), single-threaded as the reference's is,
    over the same 509,281 boxes."""
    import oracle

    mins, maxs = field_boxes()
    count = len(mins)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.bvh_build(mins, maxs)
        times.append(time.perf_counter() - t0)
    value = count / statistics.median(times) / 1e6
    return {
        "metric": "Mprims/s (BVH build)", "value": value, "unit": "Mprims/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(times), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64 build, f32 nodes",
        "data": "synthetic (seeded mulberry32 scene)", "impl": "reference",
        "config": bvh_config(count), "threads": 1,
        "cpu_baseline": {"value": value, "unit": "Mprims/s", "cores": 1, "kind": "port",
                         "sample": f"oracle BVH.build restatement over all {count} boxes, each step"},
        "e2e": {"value": value, "unit": "Mprims/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def batch_config(inst, bounces):
    """The batch line's workload, the same on both arms."""
    return {"workload": f"batch of {len(inst)} seeded sphere-field instances",
            "paths_per_frame": sum(w * h * spp for _, _, w, h, spp, _ in inst),
            "triangles": [i[5]["triangles"] for i in inst], "resolutions": [f"{i[2]}x{i[3]}" for i in inst],
            "spp": [i[4] for i in inst], "bounces": bounces,
            "l2": "inputs larger than L2 (the 64 scenes' records and images)"}


def run_batch_reference(args):
    """The reference arm of the batch line: the oracle's f32 path tracer on
    every instance of the batch in turn (the reference renders one scene
    at a time), on a bounded sample of each frame — `rows` single rows at
    the middles of equal slices of each image, on all host cores. Scenes
    are packed by the oracle (oracle/pack.py, oracle/host.py)."""
    import oracle
    from raymond_gb300 import scenes

    inst = scenes.batch_instances(args.batch, spheres=args.batch_spheres)
    threads = os.cpu_count() or 1
    rows = 2
    prepared = []
    for scene, camera, w, h, spp, info in inst:
        osc = OracleScene(scene)
        prepared.append((osc, osc.params(camera, w, h, spp, args.bounces), w, h))
    times, paths, rays = [], 0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for osc, params, w, h in prepared:
            for y0 in band_starts(h, rows, 1):
                r = oracle.render(osc.packed, osc.words, params, region=(0, y0, w, 1), nthreads=threads)
                paths += r["paths"]
                rays += r["rays"]
        times.append(time.perf_counter() - t0)
    value = paths / sum(times) / 1e6
    sample = (f"{rows} single rows at the middles of the halves of each of the {len(inst)} instances' frames per "
              "step, one instance after another")
    return {
        "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32 scenes)",
        "impl": "reference", "config": batch_config(inst, args.bounces),
        "rays_per_path_in_sample": rays / max(paths, 1),
        "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


REFERENCE_UNAVAILABLE = {
    "denoise": "the reference has no learned denoiser",
    "rmse": "the reference's CPU path to RMSE 0.01 at 1024x1024 would take hours on the host cores",
}


def time_to_rmse(scene, camera, local, size, spp, bounces, threshold=0.01, reference_spp=16384, max_spp=4096):
    """Time to RMSE ≤ threshold against a reference_spp render of the scene
    (RMSE over linear RGB as tests/browser/app.test.mjs:574-580 computes it),
    displaying after every frame of `spp` samples, for three ways of
    showing the image:
      plain_atrous    the one-kernel path, the display the à-trous filter's
      raw_average     the wavefront path, the display the running average
      learned         the wavefront path with the learned denoiser on the
                      display (the running average is left as it is)
    Frame times are wall-clock, each frame waited for; the RMSE check after
    a frame is not timed."""
    import torch

    import raymond_gb300 as rg
    from raymond_gb300 import _native
    from raymond_gb300.denoiser import DEFAULT_WEIGHTS, Denoiser

    dev = f"cuda:{local}"

    def renderer(seed, flags):
        r = rg.Renderer.create(rg.Canvas(size, size), device=local, seed=seed)
        r.scene, r.camera = scene, camera
        r.maxBounces = bounces
        r.caustics = False
        r.flags = flags
        return r

    t0 = time.perf_counter()
    ref = renderer(0x2545F491, _native.FLAG_WAVEFRONT)
    ref.denoise = False
    ref.samplesPerFrame = 64
    for _ in range(reference_spp // 64):
        ref.render()
    target = torch.from_numpy(ref.readPixels().reshape(size, size, 4)).to(dev)
    ref.dispose()
    ref_s = time.perf_counter() - t0

    def view(r, which):
        b = _native.Buffers()
        _native.check(_native.lib().raymond_get_buffers(r.handle, b), r.handle)
        return device_view(torch, b.denoised if which == "denoised" else b.accum, (size, size, 4), local)

    def rmse(img):
        d = img[..., :3] - target[..., :3]
        return float(torch.sqrt(torch.mean(d * d)).item())

    def run(r, display):
        """Frames until the displayed image (and the running average) reach
        the threshold: (first (spp, seconds) for the display, the same for
        the running average, the curve)."""
        views, elapsed, curve = None, 0.0, []
        shown = raw = None
        gc.collect()
        gc.disable()  # no collector pause inside a timed frame
        try:
            while r.samples < max_spp and (shown is None or raw is None):
                torch.cuda.synchronize()
                t = time.perf_counter()
                r.render()
                r._sync()
                elapsed += time.perf_counter() - t
                if views is None:
                    views = (view(r, display), view(r, "accum"))
                e_raw = rmse(views[1] / r.samples)
                e = e_raw if display == "accum" else rmse(views[0])
                curve.append((r.samples, round(elapsed, 4), round(e, 5), round(e_raw, 5)))
                if shown is None and e <= threshold:
                    shown = (r.samples, elapsed)
                if raw is None and e_raw <= threshold:
                    raw = (r.samples, elapsed)
        finally:
            gc.enable()
        return shown, raw, curve

    def summary(reached, curve):
        return {"reached": reached is not None, "seconds": reached[1] if reached else None,
                "spp": reached[0] if reached else None, "ms_per_frame": 1e3 * curve[-1][1] / len(curve),
                "curve_spp_seconds_rmse_rawrmse": curve[:: max(1, len(curve) // 24)]}

    plain = renderer(0, _native.FLAG_MEGAKERNEL)
    plain.denoise = True
    plain.samplesPerFrame = spp
    p_shown, _, p_curve = run(plain, "denoised")
    plain.dispose()

    raw = renderer(0, _native.FLAG_WAVEFRONT)
    raw.denoise = False
    raw.samplesPerFrame = spp
    r_shown, _, r_curve = run(raw, "accum")
    raw.dispose()

    net = Denoiser(device=local, weights=DEFAULT_WEIGHTS)
    ours = renderer(0, _native.FLAG_WAVEFRONT)
    ours.denoise = True
    ours.learnedDenoiser = net
    ours.samplesPerFrame = spp
    o_shown, _, o_curve = run(ours, "denoised")
    ours.dispose()
    net.dispose()

    p, a, o = summary(p_shown, p_curve), summary(r_shown, r_curve), summary(o_shown, o_curve)
    ok = p["reached"] and o["reached"]
    return {
        "workload": f"sphere field {size}x{size}, {spp} spp per displayed frame, {bounces} bounces",
        "threshold": threshold, "reference_spp": reference_spp, "reference_seconds": ref_s, "max_spp": max_spp,
        "plain_atrous": p, "raw_average": a, "learned": o,
        "speedup_vs_plain_atrous": p["seconds"] / o["seconds"] if ok else None,
        "speedup_vs_raw_average": a["seconds"] / o["seconds"] if (a["reached"] and o["reached"]) else None,
    }


def frame_traversal(split, paths, trace_ms, peak):
    """All closest-hit and shadow traversal bytes of a frame over the frame's
    trace time. The wavefront frame runs its extension, shading and shadow
    kernels on several streams at once, so one launch's event-timed
    duration is GPU time shared with the others: the per-launch figure
    understates the traversal's rate, the frame's does not."""
    algo = (split["trav_closest"] + split["trav_shadow"]) * paths
    gbps = algo / (trace_ms / 1e3) / 1e9
    return {"bytes": algo, "trace_ms": trace_ms, "achieved": gbps, "frac": gbps / peak, "unit": "GB/s",
            "note": "extension and shadow traversal bytes of the frame (the oracle's count) over the frame's "
                    "trace time, which also holds shading"}


def run_rmse(args, local):
    """Time to RMSE ≤ 0.01 against a 16,384-spp render as its own line."""
    scene, camera, info = build_workload(args.size, args.spp, args.bounces)
    clocks = ClockSampler(local)
    clocks.start()
    t = time_to_rmse(scene, camera, local, args.size, args.spp, args.bounces, args.threshold, args.reference_spp,
                     args.max_spp)
    clock_info = clocks.stop()
    return {
        "metric": "time-to-RMSE 0.01 (wavefront + learned denoiser)", "value": t["learned"]["seconds"], "unit": "s",
        "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 trace, bf16 network", "data": "synthetic (seeded mulberry32 scene)",
        "config": {"workload": t["workload"], "threshold": args.threshold, "reference_spp": args.reference_spp,
                   "max_spp": args.max_spp, "l2": L2_NOTE},
        "time_to_rmse": t, "clocks": clock_info,
    }


def frame_config(args, info, primitives, world, caustics):
    """The field and caustics lines' workload, the same on both arms."""
    return {"workload": CAUSTICS_WORKLOAD if caustics else WORKLOAD, "width": args.size, "height": args.size,
            "spp": args.spp, "bounces": args.bounces, "triangles": info["triangles"], "spheres": info.get("spheres"),
            "primitives": primitives, "parallelism": f"replicas x{world}", "l2": L2_NOTE}


def run_reference(args, rank, world):
    """The reference's CPU path (the shader's path tracer restated, on all
    host cores; for caustics with its light tracer and photon map too), on
    the oracle's packing of the scene."""
    if rank != 0:
        return None
    caustics = args.workload == "caustics"
    scene, camera, info = build_workload(args.size, args.spp, args.bounces, "caustics" if caustics else "field")
    osc = OracleScene(scene)
    params = osc.params(camera, args.size, args.size, args.spp, args.bounces)
    threads = os.cpu_count() or 1
    strips = 16
    rows = 2
    for _ in range(max(args.warmup, 0) and 1):
        oracle_sample(osc, params, args.size, args.size, 1, 1, threads)
    times, paths, light, rays = [], 0, 0, 0.0
    for _ in range(args.steps):
        if caustics:
            p, light, dt = caustics_cpu_sample(osc, camera, args.size, args.spp, args.bounces, threads, strips, rows)
        else:
            p, dt, _, rpp = oracle_sample(osc, params, args.size, args.size, rows, strips, threads)
            rays += rpp * p
        times.append(dt)
        paths += p
    value = paths / sum(times) / 1e6
    sample = (f"{strips} bands of {rows} rows x {args.size} px centred in equal slices of the image, {args.spp} spp "
              f"per step (1/{args.size // (strips * rows)} of a frame)")
    if caustics:
        sample += (f", with {light} of the frame's light paths splatted and deposited and the photon map "
                   "(those photons only) gathered on the bands")
    out = {
        "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32 scene)",
        "impl": "reference", "config": frame_config(args, info, osc.packed.primitiveCount, world, caustics),
        "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not caustics:
        out["rays_per_path_in_sample"] = rays / max(paths, 1)
    return out


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    import raymond_gb300 as rg
    from raymond_gb300 import _native

    torch.cuda.set_device(local)
    caustics = args.workload == "caustics"
    scene, camera, info = build_workload(args.size, args.spp, args.bounces, args.workload)
    r = rg.Renderer.create(rg.Canvas(args.size, args.size), device=local)
    r.scene, r.camera = scene, camera
    r.maxBounces = args.bounces
    r.samplesPerFrame = args.spp
    # The sphere field is plain path tracing; light tracing and photon mapping are the caustics workload's.
    r.caustics = caustics
    if caustics:
        r.setPhotons(CAUSTICS_LIGHT_PATHS, CAUSTICS_PHOTONS, CAUSTICS_RADIUS)
    r.flags = {"auto": 0, "megakernel": _native.FLAG_MEGAKERNEL, "wavefront": _native.FLAG_WAVEFRONT}[args.path]
    lib = _native.lib()
    stream = torch.cuda.ExternalStream(lib.raymond_get_stream(r.handle), device=local)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    tuning = None
    if args.path == "auto":
        tuning = r.autotune(trials=2)  # cached per GPU and workload in ~/.cache/raymond_gb300
    if args.bvh_width:
        import ctypes

        t = _native.Tuning()
        _native.check(_native.lib().raymond_get_tuning(r.handle, ctypes.byref(t)), r.handle)
        t.bvh_width = args.bvh_width
        _native.check(_native.lib().raymond_set_tuning(r.handle, ctypes.byref(t)), r.handle)
        tuning = r.tuning
    for _ in range(args.warmup):
        r.render()
    r.device.queue.onSubmittedWorkDone()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    stats = _native.Stats()
    step_ms, trace_ms, launches = [], [], 0
    ext_ms, ext_launches, shade_ms, shadow_ms, caustics_ms, denoise_ms, display_ms = [], [], [], [], [], [], []
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(len(step_ms)))  # 512 MB written: evicts the 129 MB L2 between steps
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        r.render()
        end.record(stream)
        end.synchronize()
        step_ms.append(start.elapsed_time(end))
        lib.raymond_get_stats(r.handle, stats)
        trace_ms.append(stats.ms_trace)
        launches += int(stats.launches)
        ext_ms.append(stats.ms_extend)
        ext_launches.append(stats.launches_extend)
        shade_ms.append(stats.ms_shade)
        shadow_ms.append(stats.ms_shadow)
        caustics_ms.append(stats.ms_caustics)
        denoise_ms.append(stats.ms_denoise)
        display_ms.append(stats.ms_display)
    torch.cuda.synchronize()
    barrier()
    clock_info = clocks.stop()

    paths_per_step = args.size * args.size * args.spp
    value, total_s = replica_throughput(paths_per_step, args.steps, sum(step_ms) / 1e3, world, f"cuda:{local}")
    value /= 1e6

    # End to end through the public API: render, wait, read the image back
    # (into one page-locked buffer, as a host would reuse between frames).
    e2e_steps = max(3, args.steps // 2)
    r.render()
    r.device.queue.onSubmittedWorkDone()
    pinned = torch.empty(args.size * args.size * 4, dtype=torch.float32).pin_memory()
    host = pinned.numpy()
    barrier()
    t0 = time.perf_counter()
    enqueue_s = 0.0
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        r.render()
        enqueue_s += time.perf_counter() - t1
        r.device.queue.onSubmittedWorkDone()
        px = r.readPixels(out=host)
    e2e_s = time.perf_counter() - t0
    e2e_value, _ = replica_throughput(paths_per_step, e2e_steps, e2e_s, world, f"cuda:{local}")
    e2e_value /= 1e6
    d2h = int(px.nbytes)

    result = None
    if rank == 0:
        threads = os.cpu_count() or 1
        # Algorithmic bytes per path from the oracle's instrumented f32 path
        # tracer on 1/64 of the frame (16 bands of 1 row), scaled to a launch.
        osc = OracleScene(scene)
        params = osc.params(camera, args.size, args.size, args.spp, args.bounces)
        paths_s, secs_s, bytes_per_path, rays_per_path, split = oracle_sample(osc, params, args.size, args.size, 1, 16,
                                                                              threads, detail=True)
        # CPU baseline: the same port, a bounded sample (16 bands of 2 rows;
        # for caustics the same share of the light paths and of the gather).
        if caustics:
            cpu_paths, cpu_light, cpu_s = caustics_cpu_sample(osc, camera, args.size, args.spp, args.bounces,
                                                              threads)
        else:
            cpu_paths, cpu_s, _, _ = oracle_sample(osc, params, args.size, args.size, 2, 16, threads)
        peak, peak_kind = measured_peak_hbm()
        wavefront = sum(ext_launches) > 0
        if wavefront:
            # Dominant kernel: k_wf_extend (closest-hit traversal). Algorithmic
            # bytes per launch = the frame's closest-hit traversal bytes over
            # its extend launches; duration = the mean event-timed launch.
            kernel = "k_wf_extend"
            launches_per_step = statistics.mean(ext_launches)
            bytes_per_launch = split["trav_closest"] * paths_per_step / launches_per_step
            launch_s = statistics.mean(ext_ms) / launches_per_step / 1e3
        else:
            kernel = "k_megakernel"
            bytes_per_launch = bytes_per_path * paths_per_step
            launch_s = statistics.mean(trace_ms) / 1e3
        achieved = bytes_per_launch / launch_s / 1e9
        traffic = l2_bytes = lanes = None
        if wavefront and not caustics:
            # From the ncu capture of a 512² frame of this scene (profile
            # k_wf_extend_shadow_traffic_sphere_field_512): per path over a
            # frame's extension launches, DRAM 267 B and 5,227 B through L2;
            # 11.7 of 32 lanes active per instruction. Scaled by this frame's
            # paths over its extend launches (traffic grows with the paths:
            # the scene stays in L2, the path state streams).
            traffic = EXTEND_DRAM_BYTES_PER_PATH * paths_per_step / launches_per_step
            l2_bytes = EXTEND_L2_BYTES_PER_PATH * paths_per_step / launches_per_step
            lanes = EXTEND_LANES_PER_INSTRUCTION
        result = {
            "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32 scene)",
            "config": frame_config(args, info, scene.pack().primitiveCount, world, caustics),
            "path": args.path, "tuning": tuning,
            "e2e": {"value": e2e_value, "unit": "Mpaths/s", "h2d_bytes_per_step": 208, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * e2e_s / e2e_steps, "render_call_ms": 1e3 * enqueue_s / e2e_steps},
            "gpu_launches": launches,
            "stages_ms": {"trace": statistics.mean(trace_ms), "step": statistics.mean(step_ms),
                          "extend": statistics.mean(ext_ms), "shade": statistics.mean(shade_ms),
                          "shadow": statistics.mean(shadow_ms), "caustics": statistics.mean(caustics_ms),
                          "denoise": statistics.mean(denoise_ms), "display": statistics.mean(display_ms)},
            "mrays_per_s": rays_per_path * paths_per_step * args.steps * world / total_s / 1e6,
            "rays_per_path": rays_per_path,
            "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": ("ncu capture of a 512² frame (dram__bytes_read + write of its extension "
                                            "launches), scaled by paths" if traffic else None),
                         "l2_bytes_per_launch": l2_bytes,
                         "l2_GBps": l2_bytes / launch_s / 1e9 if l2_bytes else None,
                         "active_lanes_per_instruction": lanes,
                         "bytes_per_launch": bytes_per_launch, "bytes_per_path": bytes_per_path,
                         "traversal_bytes_per_path": split,
                         "frame": frame_traversal(split, paths_per_step, statistics.mean(trace_ms), peak)
                         if wavefront else None},
            "cpu_baseline": {"value": cpu_paths / cpu_s / 1e6, "unit": "Mpaths/s", "cores": threads, "kind": "port",
                             "sample": f"16 bands of 2 rows x {args.size} px centred in equal slices of the image, "
                                       f"at {args.spp} spp (1/32 of a frame)"
                                       + (f", with {cpu_light} of the frame's light paths splatted and deposited "
                                          "and the photon map (those photons only) gathered on the bands"
                                          if caustics else "")},
            "clocks": clock_info,
        }
        if caustics:
            result["mphotons_per_s"] = CAUSTICS_LIGHT_PATHS * args.steps * world / total_s / 1e6
            result["photons"] = {"light_paths_per_frame": CAUSTICS_LIGHT_PATHS, "capacity": CAUSTICS_PHOTONS,
                                 "radius": CAUSTICS_RADIUS}
    r.dispose()
    if rank == 0 and not args.no_denoiser and not caustics:
        result["learned_denoiser"] = measure_denoiser(scene, camera, local, 10, 3)
    if rank == 0 and not args.no_rmse and not caustics and args.size == 1024:
        clocks = ClockSampler(local)
        clocks.start()
        result["time_to_rmse"] = time_to_rmse(scene, camera, local, args.size, args.spp, args.bounces,
                                              args.threshold, args.reference_spp, args.max_spp)
        result["time_to_rmse"]["clocks"] = clocks.stop()
    return result


def run_batch(args):
    """The batched workload: 64 seeded sphere-field instances rendered as
    one graph-replayed batched frame, against the same renderers rendering
    one at a time. Metric: Mpaths/s over the whole batch."""
    import torch

    import raymond_gb300 as rg
    from raymond_gb300 import scenes

    t0 = time.perf_counter()
    inst = scenes.batch_instances(args.batch, spheres=args.batch_spheres)
    rs = []
    for scene, camera, w, h, spp, info in inst:
        r = rg.Renderer.create(rg.Canvas(w, h))
        r.scene, r.camera = scene, camera
        r.maxBounces = args.bounces
        r.samplesPerFrame = spp
        r.caustics = False
        rs.append(r)
    setup_s = time.perf_counter() - t0
    paths = sum(w * h * spp for _, _, w, h, spp, _ in inst)
    # One launch at a time: each renderer's own frame, waited for before the next.
    for r in rs:
        r.render()
    torch.cuda.synchronize()
    for r in rs:
        r.device.queue.onSubmittedWorkDone()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for r in rs:
            r.render()
            r.device.queue.onSubmittedWorkDone()
    single_s = (time.perf_counter() - t0) / args.steps
    # Each renderer's own frame on its own stream, all in flight together.
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for r in rs:
            r.render()
        for r in rs:
            r.device.queue.onSubmittedWorkDone()
    streams_s = (time.perf_counter() - t0) / args.steps
    batch = rg.BatchRenderer(graph=True)
    for _ in range(args.warmup):
        batch.render(rs)
    batch.sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.render(rs)
    batch.sync()
    batch_s = (time.perf_counter() - t0) / args.steps
    st = batch.stats()
    out = {
        "metric": METRIC, "value": paths / batch_s / 1e6, "unit": "Mpaths/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": batch_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32 scenes)",
        "config": batch_config(inst, args.bounces),
        "executor": "one graph-replayed batched frame", "setup_s": setup_s,
        "one_at_a_time": {"value": paths / single_s / 1e6, "unit": "Mpaths/s", "ms_per_step": single_s * 1e3},
        "speedup_vs_one_at_a_time": single_s / batch_s,
        "concurrent_streams": {"value": paths / streams_s / 1e6, "unit": "Mpaths/s", "ms_per_step": streams_s * 1e3},
        "speedup_vs_concurrent_streams": streams_s / batch_s,
        "gpu_launches": int(st.launches) * args.steps,
    }
    for r in rs:
        r.dispose()
    batch.dispose()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--spp", type=int, default=4)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--bounces", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="auto", choices=["auto", "megakernel", "wavefront"])
    ap.add_argument("--workload", default="field", choices=["field", "caustics", "batch", "denoise", "rmse", "primary", "bvh"])
    ap.add_argument("--threshold", type=float, default=0.01)
    ap.add_argument("--reference-spp", type=int, default=16384)
    ap.add_argument("--max-spp", type=int, default=4096)
    ap.add_argument("--no-denoiser", action="store_true", help="skip the learned-denoiser sub-measurement")
    ap.add_argument("--no-rmse", action="store_true", help="skip the time-to-RMSE sub-measurement")
    ap.add_argument("--bvh-width", type=int, default=0, choices=[0, 2, 4],
                    help="force the binary (2) or 4-wide (4) traversal tree; 0 keeps the tuned choice")
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--batch-spheres", type=int, default=10000)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.init_process_group("nccl")
    if args.impl == "reference" and args.workload == "primary":
        out = run_primary_reference(args, rank, world)
    elif args.impl == "reference" and args.workload == "bvh":
        out = run_bvh_reference(args) if rank == 0 else None
    elif args.impl == "reference" and args.workload == "batch":
        out = run_batch_reference(args) if rank == 0 else None
    elif args.impl == "reference" and args.workload in REFERENCE_UNAVAILABLE:
        out = {"impl": "reference", "unavailable": REFERENCE_UNAVAILABLE[args.workload]} if rank == 0 else None
    elif args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "batch":
        out = run_batch(args) if rank == 0 else None
    elif args.workload == "denoise":
        out = run_denoise(args, local) if rank == 0 else None
    elif args.workload == "rmse":
        out = run_rmse(args, local) if rank == 0 else None
    elif args.workload == "primary":
        out = run_primary(args, local) if rank == 0 else None
    elif args.workload == "bvh":
        out = run_bvh(args) if rank == 0 else None
    else:
        out = run_ours(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
