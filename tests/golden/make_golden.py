"""Writes the golden fixtures of this folder from the CPU oracle (oracle/),
so that the oracle, the product's native BVH builder and packer, and the
CUDA path can be checked against the same committed bytes on every machine
(the oracle builds here on x86 and on the GB300 machine's Arm cores).

    python tests/golden/make_golden.py

Fixtures (numpy .npz):
  bvh_boxes.npz      2,000 seeded boxes and BVH.build's nodes and order for them
                     (oracle/bvh.cpp, src/BVH.mjs:57-234)
  cornell.npz        the C1 Cornell room packed by the oracle's Scene.#pack and lights
                     table (oracle/pack.py, oracle/host.py): primitives, nodes,
                     materials, lights words; 4,096 of its jittered primary rays (64², mulberry32 seed 1)
                     and Scene.raycast's answers for them (oracle/raycast.cpp,
                     src/Scene.mjs:202-283): hit primitive and distance
  cornell_image.npz  the shader's path tracer (oracle/pathtrace.cpp) on the room:
                     16×16, 4 samples, 6 bounces, the 208-byte uniform block used
                     (the oracle's #writeParams)
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import host, pack  # noqa: E402
from raymond_gb300 import scenes  # noqa: E402


def seeded_boxes(count: int, seed: int):
    u = scenes.mulberry32_array(seed, count * 6).astype(np.float64).reshape(count, 6)
    centre = (u[:, :3] - 0.5) * 20.0
    half = 0.01 + 0.5 * u[:, 3:]
    return centre - half, centre + half


def cornell_case():
    scene, camera = scenes.cornell_scene()
    packed = pack.pack(scene.objects)
    size = 64
    xi = scenes.mulberry32_array(1, 2 * size * size).reshape(-1, 2)
    ys, xs = np.meshgrid(np.arange(size), np.arange(size), indexing="ij")
    rays = scenes.camera_rays_f32(camera, size, size, xs.reshape(-1) + xi[:, 0], ys.reshape(-1) + xi[:, 1])
    return scene, camera, packed, np.ascontiguousarray(rays, dtype=np.float32)


def image_params(scene, camera, size=16, spp=4, bounces=6):
    words, powers = host.light_words(pack.pack(scene.objects))
    return host.params(scene, camera, size, size, light_count=len(powers), max_bounces=bounces, spp=spp,
                       firefly_clamp=0.0), words


def main():
    mins, maxs = seeded_boxes(2000, 11)
    nodes, order = oracle.bvh_build(mins, maxs)
    np.savez_compressed(os.path.join(HERE, "bvh_boxes.npz"), mins=mins, maxs=maxs, nodes=nodes, order=order)

    scene, camera, packed, rays = cornell_case()
    hits = oracle.raycast(packed, rays)
    words, _ = host.light_words(packed)
    np.savez_compressed(os.path.join(HERE, "cornell.npz"), primitives=packed.primitives, nodes=packed.nodes,
                        materials=packed.materials, lights_words=np.asarray(words, dtype=np.uint32), rays=rays,
                        prim=hits["prim"], t=hits["t"])

    params, words = image_params(scene, camera)
    img = oracle.render(packed, words, params, nthreads=1)
    np.savez_compressed(os.path.join(HERE, "cornell_image.npz"), params=np.frombuffer(params, dtype=np.uint8),
                        accum=img["accum"], albedo=img["albedo"], normal=img["normal"])
    for f in ("bvh_boxes.npz", "cornell.npz", "cornell_image.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
