"""bench.py's lines that run without a GPU — the reference arm (the
oracle's CPU path) and the host BVH build — carry the keys of the bench
contract: one JSON line, the metric and its unit, the run's shape, the
e2e object with its copy sizes, and the CPU baseline's description."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def check_common(d, steps, warmup):
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert key in d, key
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert (d["steps"], d["warmup"]) == (steps, warmup)
    assert d["scaling"] in ("weak", "strong")
    assert "workload" in d["config"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] >= 0 and e2e["d2h_bytes_per_step"] >= 0
    cpu = d["cpu_baseline"]
    assert cpu["value"] > 0 and cpu["cores"] >= 1 and cpu["kind"] in ("port", "reference") and cpu["sample"]


@pytest.mark.parametrize("workload", ["field", "primary"])
def test_reference_arm_line(workload):
    args = ["--impl", "reference", "--steps", "1", "--warmup", "0"]
    if workload == "field":
        args += ["--size", "64"]
    else:
        args += ["--workload", "primary"]
    d = run(*args)
    check_common(d, 1, 0)
    assert d["impl"] == "reference"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["value"] == d["value"]


def test_bvh_build_line():
    d = run("--workload", "bvh", "--steps", "1", "--warmup", "1")
    check_common(d, 1, 1)
    assert d["unit"] == "Mprims/s" and d["gpu_launches"] == 0
    assert d["identical_to_oracle"] is True


def test_reference_arm_follows_the_workload():
    d = run("--impl", "reference", "--workload", "caustics", "--steps", "1", "--warmup", "0", "--size", "64")
    check_common(d, 1, 0)
    assert d["impl"] == "reference" and d["config"]["workload"].startswith("water caustics")
    assert "light paths" in d["cpu_baseline"]["sample"]
    d = run("--impl", "reference", "--workload", "batch", "--batch", "4", "--steps", "1", "--warmup", "0")
    check_common(d, 1, 0)
    assert d["impl"] == "reference" and d["config"]["workload"] == "batch of 4 seeded sphere-field instances"
    assert len(d["config"]["resolutions"]) == 4 and d["config"]["paths_per_frame"] > 0
    for workload in ("denoise", "rmse"):
        d = run("--impl", "reference", "--workload", workload, "--steps", "1", "--warmup", "0")
        assert d["impl"] == "reference" and d["unavailable"]


@pytest.mark.parametrize("workload", ["field", "caustics", "batch", "primary", "bvh"])
def test_reference_arm_maps_no_product_library(workload):
    """The reference arm packs its scenes with the oracle (oracle/pack.py,
    oracle/host.py) and never loads libraymond_cuda.so: after it runs, the
    process maps the oracle's library and not the product's."""
    args = ["--impl", "reference", "--workload", workload, "--steps", "1", "--warmup", "0"]
    args += {"field": ["--size", "32"], "caustics": ["--size", "32"], "batch": ["--batch", "2"]}.get(workload, [])
    code = ("import runpy, sys; sys.argv = ['bench.py'] + sys.argv[1:]; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', 'libraymond_cuda' in maps, 'liboracle' in maps)")
    r = subprocess.run([sys.executable, "-c", code, *args], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    marker = [ln for ln in r.stdout.splitlines() if ln.startswith("MAPS")]
    assert marker == ["MAPS False True"], r.stdout[-2000:]


def test_denoiser_lines_report_the_training_set():
    """The learned-denoiser lines carry how the shipped weights were trained,
    read from the report beside them, against the configured data set."""
    import bench

    note = bench.training_note()
    assert note is not None
    assert note["views"] > 0 and note["target_spp"] == 16384 and note["adam_steps"] > 0
    assert note["paths"] < note["configured_paths"]
    assert note["field_spheres"] and note["field_spheres"][0] <= note["field_spheres"][1]


def test_training_views_follow_the_density_options():
    """Sphere-field training views draw their sphere count and mesh frequency
    from the given ranges; the defaults keep the original sequence."""
    from raymond_gb300 import scenes

    dense = scenes.training_views(6, seed=3, spheres=(3000, 3100), frequency=(20, 22))
    fields = [info for _, _, info in dense if "spheres" in info]
    assert fields and all(3000 <= f["spheres"] < 3100 for f in fields)
    assert all(f["triangles"] in (20 * 20 * 20, 20 * 21 * 21) for f in fields)
    default = scenes.training_views(4, seed=99)
    again = scenes.training_views(4, seed=99, spheres=(300, 3000), frequency=(10, 55))
    assert [v[2] for v in default] == [v[2] for v in again]
