"""Golden fixtures (tests/golden/, written by make_golden.py from the oracle):
the oracle, the product's native BVH builder and packer, and the CUDA path
are all checked against the same committed bytes, so a result that drifts on
another machine or compiler (the GB300 machine is Arm) shows here."""

import os

import numpy as np
import pytest

import oracle
from parity import classify
from raymond_gb300 import Canvas, Renderer, scenes
from raymond_gb300.scene import BVH

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


def test_oracle_bvh_matches_golden():
    g = load("bvh_boxes.npz")
    nodes, order = oracle.bvh_build(g["mins"], g["maxs"])
    assert np.array_equal(nodes, g["nodes"])
    assert np.array_equal(order, g["order"])


@pytest.mark.parametrize("threads", [1, 8])
def test_native_bvh_matches_golden(threads):
    g = load("bvh_boxes.npz")
    b = BVH.build(g["mins"], g["maxs"], threads=threads)
    assert np.array_equal(b.nodes, g["nodes"])
    assert np.array_equal(b.order, g["order"])


@pytest.mark.parametrize("packer", ["product", "oracle"])
def test_packed_cornell_matches_golden(packer):
    """The fixture is the oracle's packing (oracle/pack.py, Scene.#pack
    restated); the product's packer must reproduce it byte for byte."""
    from oracle import host, pack

    g = load("cornell.npz")
    scene, camera = scenes.cornell_scene()
    packed = scene.pack() if packer == "product" else pack.pack(scene.objects)
    assert np.array_equal(packed.primitives, g["primitives"])
    assert np.array_equal(packed.nodes, g["nodes"])
    assert np.array_equal(packed.materials, g["materials"])
    assert np.array_equal(host.light_words(packed)[0], g["lights_words"])


def test_oracle_raycast_matches_golden():
    g = load("cornell.npz")
    scene, camera = scenes.cornell_scene()
    hits = oracle.raycast(scene.pack(), g["rays"])
    assert np.array_equal(hits["prim"], g["prim"])
    np.testing.assert_allclose(hits["t"], g["t"], rtol=1e-12, atol=0)


def test_oracle_path_tracer_matches_golden():
    g = load("cornell_image.npz")
    scene, camera = scenes.cornell_scene()
    packed = scene.pack()
    from raymond_gb300.renderer import light_table

    words, _ = light_table(packed)
    img = oracle.render(packed, words, g["params"].tobytes(), nthreads=1)
    # f32 arithmetic compiled without contraction; libm may differ in the
    # last place between machines, so compare to rounding, not bits.
    np.testing.assert_allclose(img["accum"], g["accum"], rtol=1e-4, atol=1e-5)


@pytest.mark.gpu
def test_gpu_hits_match_golden(gpu):
    g = load("cornell.npz")
    scene, camera = scenes.cornell_scene()
    r = Renderer.create(Canvas(1, 1))
    prim, t = r.tracePrimary(g["rays"], scene)
    r.dispose()
    ref = {"prim": g["prim"], "t": g["t"]}
    c = classify(scene.pack(), g["rays"], prim, t, ref)
    assert c["wrong"] == 0, c
    assert c["hit_miss"] + c["silhouettes"] <= 0.005 * c["n"], c


@pytest.mark.gpu
def test_gpu_image_matches_golden(gpu):
    g = load("cornell_image.npz")
    scene, camera = scenes.cornell_scene()
    r = Renderer.create(Canvas(16, 16))
    r.scene, r.camera = scene, camera
    # denoise on, as the fixture's block has it (the denoiser leaves accum alone)
    r.maxBounces, r.samplesPerFrame, r.fireflyClamp, r.denoise = 6, 4, 0, True
    r.render()
    assert r.params == g["params"].tobytes()  # the same 208-byte block
    accum, albedo, normal = r.readGuides()
    r.dispose()
    # same sample streams, f32 on both sides: most pixels agree to 1e-3
    rel = np.abs(accum[..., :3] - g["accum"][..., :3]) / np.maximum(np.abs(g["accum"][..., :3]), 1e-3)
    assert (rel.max(axis=2) < 1e-3).mean() > 0.9
    assert abs(accum[..., :3].mean() / g["accum"][..., :3].mean() - 1) < 0.02


@pytest.mark.gpu
def test_oracle_and_builder_match_golden_on_the_gpu_machine(gpu):
    """Run with the GPU tests so the oracle and the native builder, compiled
    on the GPU machine's own (Arm) cores, are pinned to the same bytes."""
    test_oracle_bvh_matches_golden()
    test_native_bvh_matches_golden(8)
    test_packed_cornell_matches_golden("product")
    test_packed_cornell_matches_golden("oracle")
    test_oracle_raycast_matches_golden()
    test_oracle_path_tracer_matches_golden()


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_native_bvh_matches_oracle_on_a_large_set(threads):
    """200,000 boxes: the top nodes' passes run split over the threads
    (nodes of 65,536 primitives and more), and the result is still the
    reference's build byte for byte."""
    rng = np.random.default_rng(5)
    centre = rng.uniform(-50, 50, (200_000, 3))
    centre[:100_000] = rng.normal(0, 3, (100_000, 3))  # a dense cluster among sparse ones
    half = rng.uniform(0.001, 0.3, (200_000, 3))
    mins, maxs = centre - half, centre + half
    nodes, order = oracle.bvh_build(mins, maxs)
    b = BVH.build(mins, maxs, threads=threads)
    assert np.array_equal(b.nodes, nodes)
    assert np.array_equal(b.order, order)


@pytest.mark.parametrize("threads", [1, 8])
def test_native_bvh_matches_oracle_on_degenerate_sets(threads):
    """Sets where the reference's fallbacks decide: every centroid equal (no
    axis to bin: split in the middle), all boxes in one plane (one axis
    without extent), and heavy duplicates in few bins."""
    rng = np.random.default_rng(9)
    same = np.tile([1.0, 2.0, 3.0], (5000, 1))
    flat = np.column_stack([rng.uniform(-5, 5, 80_000), rng.uniform(-5, 5, 80_000), np.zeros(80_000)])
    dup = np.repeat(rng.uniform(-1, 1, (7, 3)), 12_000, axis=0)
    for centre in (same, flat, dup):
        half = np.full_like(centre, 0.01)
        mins, maxs = centre - half, centre + half
        nodes, order = oracle.bvh_build(mins, maxs)
        b = BVH.build(mins, maxs, threads=threads)
        assert np.array_equal(b.nodes, nodes)
        assert np.array_equal(b.order, order)
