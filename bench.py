#!/usr/bin/env python
"""Benchmark of the render path on the sphere-field workload: 1024×1024,
8 bounces, NEE+MIS, Russian roulette from bounce 3, FP32 accumulation, the
à-trous denoiser on (the renderer's default), 10,000 spheres on a 40×40
ground around a 499,280-triangle displaced geodesic sphere, gradient sky and
a 0.27° sun. A step is one frame, Renderer.render(): the trace, the
denoiser and the tone map. Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--spp S] [--impl ours|reference]

Under torchrun each rank renders its own copy of the frame (replicas; the
scene does not shard across GPUs here): value = paths of all ranks ÷ the
slowest rank's time.
"""

from __future__ import annotations

import argparse
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


def build_workload(size, spp, bounces):
    import raymond_gb300 as rg
    from raymond_gb300 import scenes

    scene, camera, info = scenes.sphere_field()
    return scene, camera, info


def oracle_sample(scene, params: bytes, size, rows_per_strip, strips, threads, detail=False):
    """The oracle's f32 path tracer on `strips` bands spread down the image:
    returns (paths, seconds, algorithmic bytes per path, rays per path), and
    with detail the per-path closest-hit and shadow traversal bytes too."""
    import oracle
    from raymond_gb300.renderer import light_table

    packed = scene.pack()
    words, _ = light_table(packed)
    tot = {"paths": 0, "bytes": 0, "rays": 0, "trav_closest": 0, "trav_shadow": 0, "rays_closest": 0,
           "rays_shadow": 0}
    t0 = time.perf_counter()
    for k in range(strips):
        y0 = (k * size) // strips
        r = oracle.render(packed, words, params, region=(0, y0, size, rows_per_strip), nthreads=threads)
        for key in tot:
            tot[key] += r[key]
    secs = time.perf_counter() - t0
    p = max(tot["paths"], 1)
    out = (tot["paths"], secs, tot["bytes"] / p, tot["rays"] / p)
    if detail:
        return out + ({k: tot[k] / p for k in ("trav_closest", "trav_shadow", "rays_closest", "rays_shadow")},)
    return out


def params_for(scene, camera, size, spp, bounces):
    """The uniform block a renderer writes for frame 0 of this workload."""
    from raymond_gb300.renderer import light_table, params_block

    packed = scene.pack()
    words, powers = light_table(packed)
    return params_block(scene, camera, size, size, light_count=len(powers), volume_count=len(packed.volumes),
                        max_bounces=bounces, spp=spp)


def run_reference(args, rank, world):
    """The reference's CPU path (the shader's path tracer restated, on all host cores)."""
    if rank != 0:
        return None
    scene, camera, info = build_workload(args.size, args.spp, args.bounces)
    params = params_for(scene, camera, args.size, args.spp, args.bounces)
    threads = os.cpu_count() or 1
    strips = 16
    rows = 2
    for _ in range(max(args.warmup, 0) and 1):
        oracle_sample(scene, params, args.size, 1, 1, threads)
    times, paths = [], 0
    for _ in range(args.steps):
        p, dt, _, _ = oracle_sample(scene, params, args.size, rows, strips, threads)
        times.append(dt)
        paths += p
    value = paths / sum(times) / 1e6
    sample = f"{strips} bands of {rows} rows x {args.size} px, {args.spp} spp per step (1/{args.size // (strips * rows)} of a frame)"
    return {
        "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "width": args.size, "height": args.size, "spp": args.spp,
                   "bounces": args.bounces, "triangles": info["triangles"], "spheres": info["spheres"],
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    import raymond_gb300 as rg
    from raymond_gb300 import _native

    torch.cuda.set_device(local)
    scene, camera, info = build_workload(args.size, args.spp, args.bounces)
    r = rg.Renderer.create(rg.Canvas(args.size, args.size), device=local)
    r.scene, r.camera = scene, camera
    r.maxBounces = args.bounces
    r.samplesPerFrame = args.spp
    r.caustics = False  # plain path tracing: light tracing and photon mapping are the caustics workload's
    r.flags = {"auto": 0, "megakernel": _native.FLAG_MEGAKERNEL, "wavefront": _native.FLAG_WAVEFRONT}[args.path]
    lib = _native.lib()
    stream = torch.cuda.ExternalStream(lib.raymond_get_stream(r.handle), device=local)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    tuning = None
    if args.path == "auto":
        tuning = r.autotune(trials=2, cache=os.path.join(ROOT, "gpurun_out", "tuning.json"))
    for _ in range(args.warmup):
        r.render()
    r.device.queue.onSubmittedWorkDone()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    stats = _native.Stats()
    step_ms, trace_ms, launches = [], [], 0
    ext_ms, ext_launches, shade_ms, shadow_ms = [], [], [], []
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
    torch.cuda.synchronize()
    barrier()
    clock_info = clocks.stop()

    total_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([total_s], device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    paths_per_step = args.size * args.size * args.spp
    value = paths_per_step * args.steps * world / total_s / 1e6

    # End to end through the public API: render, wait, read the image back.
    e2e_steps = max(3, args.steps // 2)
    r.render()
    r.device.queue.onSubmittedWorkDone()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        r.render()
        r.device.queue.onSubmittedWorkDone()
        px = r.readPixels()
    e2e_s = time.perf_counter() - t0
    e2e_value = paths_per_step * e2e_steps / e2e_s / 1e6
    d2h = int(px.nbytes)

    result = None
    if rank == 0:
        threads = os.cpu_count() or 1
        # Algorithmic bytes per path from the oracle's instrumented f32 path
        # tracer on 1/64 of the frame (16 bands of 1 row), scaled to a launch.
        params = params_for(scene, camera, args.size, args.spp, args.bounces)
        paths_s, secs_s, bytes_per_path, rays_per_path, split = oracle_sample(scene, params, args.size, 1, 16, threads,
                                                                              detail=True)
        # CPU baseline: the same port, a bounded sample (16 bands of 2 rows).
        cpu_paths, cpu_s, _, _ = oracle_sample(scene, params, args.size, 2, 16, threads)
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
        traffic = None
        prof = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(prof):
            try:
                with open(prof) as f:
                    traffic = json.load(f).get("megakernel_bytes_per_launch")
            except (OSError, ValueError):
                traffic = None
        result = {
            "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mulberry32 scene)",
            "config": {"workload": WORKLOAD, "width": args.size, "height": args.size, "spp": args.spp,
                       "bounces": args.bounces, "triangles": info["triangles"], "spheres": info["spheres"],
                       "primitives": scene.pack().primitiveCount, "parallelism": f"replicas x{world}", "path": args.path, "tuning": tuning,
                       "l2": "flushed between steps (512 MB write)"},
            "e2e": {"value": e2e_value, "unit": "Mpaths/s", "h2d_bytes_per_step": 208, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "stages_ms": {"trace": statistics.mean(trace_ms), "step": statistics.mean(step_ms),
                          "extend": statistics.mean(ext_ms), "shade": statistics.mean(shade_ms),
                          "shadow": statistics.mean(shadow_ms)},
            "mrays_per_s": rays_per_path * paths_per_step * args.steps * world / total_s / 1e6,
            "rays_per_path": rays_per_path,
            "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "bytes_per_launch": bytes_per_launch, "bytes_per_path": bytes_per_path,
                         "traversal_bytes_per_path": split},
            "cpu_baseline": {"value": cpu_paths / cpu_s / 1e6, "unit": "Mpaths/s", "cores": threads, "kind": "port",
                             "sample": f"16 bands of 2 rows x {args.size} px at {args.spp} spp (1/32 of a frame)"},
            "clocks": clock_info,
        }
    r.dispose()
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
    # One at a time (each renderer's own frame, tuned path).
    for r in rs:
        r.render()
    torch.cuda.synchronize()
    for r in rs:
        r.device.queue.onSubmittedWorkDone()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for r in rs:
            r.render()
        for r in rs:
            r.device.queue.onSubmittedWorkDone()
    single_s = (time.perf_counter() - t0) / args.steps
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
        "config": {"workload": f"batch of {len(rs)} sphere-field instances, one graph-replayed launch per frame",
                   "paths_per_frame": paths, "triangles": [i[5]["triangles"] for i in inst],
                   "resolutions": [f"{i[2]}x{i[3]}" for i in inst], "spp": [i[4] for i in inst],
                   "bounces": args.bounces, "setup_s": setup_s},
        "one_at_a_time": {"value": paths / single_s / 1e6, "unit": "Mpaths/s", "ms_per_step": single_s * 1e3},
        "speedup_vs_one_at_a_time": single_s / batch_s,
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
    ap.add_argument("--workload", default="field", choices=["field", "batch"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--batch-spheres", type=int, default=10000)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "batch":
        out = run_batch(args) if rank == 0 else None
    else:
        out = run_ours(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
