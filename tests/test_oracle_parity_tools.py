"""The oracle's tools for classifying GPU disagreements (tests/parity.py):
perturbation runs leave nothing behind, move results only slightly, and
light paths report their edge margins and ties."""

import numpy as np

import oracle
from oracle import host, pack
from parity import classify_pixels, perturbation_runs
from raymond_gb300 import Camera, Material, Quad, Scene, Sky, Sphere, Vec3, scenes


def cornell_frame():
    scene, camera = scenes.cornell_scene()
    packed = pack.pack(scene.objects)
    words, powers = host.light_words(packed)
    params = host.params(scene, camera, 24, 24, light_count=len(powers), spp=2, firefly_clamp=0.0)
    return lambda: oracle.render(packed, words, params)["accum"]


def test_perturbation_runs_leave_the_oracle_unchanged():
    run = cornell_frame()
    base = run()
    runs = perturbation_runs(run, runs=4)
    assert np.array_equal(run(), base)
    # they move results, mostly by little
    moved = [np.abs(r - base).max() for r in runs]
    assert max(moved) > 0
    c = classify_pixels(base, base, runs)
    assert c["agree"] == c["n"] and c["unexplained"] == 0


def test_classes_of_a_planted_difference():
    """A difference planted in the oracle's own image, on the CPU: far beyond
    what the perturbation runs move a pixel, it is unexplained."""
    run = cornell_frame()
    base = run()
    runs = perturbation_runs(run, runs=4)
    planted = base.copy()
    stable = np.argwhere(np.max([np.abs(r - base)[..., :3].max(-1) for r in runs], axis=0) == 0)[0]
    planted[stable[0], stable[1], :3] = base[stable[0], stable[1], :3] * 1.01 + 1e-3
    c = classify_pixels(planted, base, runs)
    assert c["unexplained"] == 1 and c["unexplained_idx"] == [list(stable)]


def test_light_paths_report_ties_on_coincident_faces():
    """Two quads on the same plane overlap, so a ray reaching the overlap
    meets both at one distance: a tie, margin 0. A ray through the open
    middle of the other quad reports its barycentric margin."""
    white = Material.diffuse(Vec3(0.5, 0.5, 0.5))
    glassy = Material.metal(Vec3(0.9, 0.9, 0.9), 0.0)
    scene = Scene(sky=Sky.black()).add(
        Quad(Vec3(-2, 0, 2), Vec3(4, 0, 0), Vec3(0, 0, -4), white),
        Quad(Vec3(-0.5, 1, 0.5), Vec3(1, 0, 0), Vec3(0, 0, -1), glassy),
        Quad(Vec3(-0.2, 1, 0.5), Vec3(1, 0, 0), Vec3(0, 0, -1), glassy),
        Sphere(Vec3(0, 3, 0), 0.2, Material.light(Vec3(1, 1, 1), 20.0)))
    camera = Camera(position=Vec3(0, 4, 4), target=Vec3(0, 0, 0))
    packed = pack.pack(scene.objects)
    words, powers = host.light_words(packed)
    deltas = host.delta_objects(scene.objects, packed)
    emitters = host.emitters(powers, deltas, scene.sky, len(powers))
    params = host.params(scene, camera, 32, 32, light_count=len(powers), spp=4, caustics=True, deltas=deltas)
    lt = oracle.light_trace(packed, words, params, emitters, 4096, margins=True)
    m = lt["path_margins"]
    assert len(m) == 4096 and (m == 0).sum() > 0 and (m > 1e-3).sum() > 0
    assert np.isin(lt["photon_ids"], np.nonzero(m >= 0)[0]).all()
    plain = oracle.light_trace(packed, words, params, emitters, 4096)
    assert np.array_equal(plain["photons"], lt["photons"]) and plain["path_margins"] is None
