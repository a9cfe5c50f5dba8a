"""The reference's own unit tests for the render path's inputs, restated:
tests/unit/bvh.test.mjs, scene.test.mjs and camera.test.mjs. They pin the
oracle (BVH.build and Scene.raycast restatements) and this package's scene
packer and native BVH builder against the reference's known answers."""

import math

import numpy as np
import pytest

import oracle
from raymond_gb300 import BVH, NONE, PRIMITIVE_KINDS, Box, Camera, Mat4, Material, Mesh, Quad, Scene, Sphere, Vec3

WHITE = Material.diffuse(Vec3(0.8, 0.8, 0.8))
LAMP = Material.light(Vec3(1, 1, 1), 5.0)


def lcg(seed):
    """tests/unit/helpers.mjs:29-34."""
    state = [seed]

    def nxt():
        state[0] = (state[0] * 1664525 + 1013904223) % 4294967296
        return state[0] / 4294967296

    return nxt


def random_boxes(count, seed):
    """tests/unit/bvh.test.mjs:7-24."""
    nxt = lcg(seed)
    mins = np.zeros(count * 3)
    maxs = np.zeros(count * 3)
    for i in range(count):
        size = 50.0 if nxt() < 0.05 else (5.0 if nxt() < 0.2 else 0.3)
        for a in range(3):
            c = (nxt() - 0.5) * 40.0
            half = size * nxt()
            mins[i * 3 + a] = c - half
            maxs[i * 3 + a] = c + half
    return mins, maxs


def read_nodes(nodes):
    u = nodes.reshape(-1, 8)
    f = u.view(np.float32)
    return [{"min": f[i, :3].astype(np.float64), "first": int(u[i, 3]), "max": f[i, 4:7].astype(np.float64),
             "count": int(u[i, 7])} for i in range(len(u))]


def contains(outer, inner_min, inner_max):
    return all(outer["min"][a] <= inner_min[a] + 1e-4 * max(1, abs(inner_min[a])) and
               outer["max"][a] >= inner_max[a] - 1e-4 * max(1, abs(inner_max[a])) for a in range(3))


def walk(nodes_u32, order, mins, maxs, max_leaf):
    nodes = read_nodes(nodes_u32)
    seen = np.zeros(len(order), dtype=np.int64)
    stack = [0]
    while stack:
        node = nodes[stack.pop()]
        if node["count"] > 0:
            assert node["count"] <= max_leaf
            for i in range(node["first"], node["first"] + node["count"]):
                p = order[i]
                seen[p] += 1
                assert contains(node, mins[p * 3:p * 3 + 3], maxs[p * 3:p * 3 + 3])
        else:
            for child in (node["first"], node["first"] + 1):
                assert 0 < child < len(nodes)
                assert contains(node, nodes[child]["min"], nodes[child]["max"])
                stack.append(child)
    return seen


BUILDERS = {
    "oracle": lambda mins, maxs, leaf=4: oracle.bvh_build(mins, maxs, leaf),
    "native": lambda mins, maxs, leaf=4: (lambda b: (b.nodes, b.order))(BVH.build(mins, maxs, leaf)),
}


@pytest.mark.parametrize("builder", sorted(BUILDERS))
def test_every_primitive_in_one_leaf(builder):
    for count in [1, 2, 3, 5, 17, 100, 2000]:
        mins, maxs = random_boxes(count, count)
        nodes, order = BUILDERS[builder](mins, maxs)
        seen = walk(nodes, order, mins, maxs, 4)
        assert list(seen) == [1] * count
        assert sorted(order.tolist()) == list(range(count))


@pytest.mark.parametrize("builder", sorted(BUILDERS))
def test_coincident_primitives_split_into_small_leaves(builder):
    count = 50
    mins = np.full(count * 3, -1.0)
    maxs = np.full(count * 3, 1.0)
    nodes, order = BUILDERS[builder](mins, maxs)
    assert list(walk(nodes, order, mins, maxs, 4)) == [1] * count


@pytest.mark.parametrize("builder", sorted(BUILDERS))
def test_tree_shallow_enough_for_64_entry_stack(builder):
    mins, maxs = random_boxes(20000, 9)
    nodes = read_nodes(BUILDERS[builder](mins, maxs)[0])
    deepest, stack = 0, [(0, 1)]
    while stack:
        n, depth = stack.pop()
        deepest = max(deepest, depth)
        if nodes[n]["count"] == 0:
            stack += [(nodes[n]["first"], depth + 1), (nodes[n]["first"] + 1, depth + 1)]
    assert deepest < 64


@pytest.mark.parametrize("builder", sorted(BUILDERS))
def test_clusters_split_at_root(builder):
    count = 40
    mins = np.zeros(count * 3)
    maxs = np.zeros(count * 3)
    for i in range(count):
        x = (-100 if i < count / 2 else 100) + (i % 7)
        mins[i * 3:i * 3 + 3] = [x, 0, 0]
        maxs[i * 3:i * 3 + 3] = [x + 0.5, 0.5, 0.5]
    nodes = read_nodes(BUILDERS[builder](mins, maxs)[0])
    left, right = nodes[nodes[0]["first"]], nodes[nodes[0]["first"] + 1]
    assert left["max"][0] < 0 or right["max"][0] < 0
    assert left["min"][0] > 0 or right["min"][0] > 0


def test_empty_tree_is_one_node():
    for name, b in BUILDERS.items():
        nodes, order = b(np.zeros(0), np.zeros(0))
        assert len(nodes) == 8 and len(order) == 0, name


def test_native_builder_matches_oracle_byte_for_byte():
    for count, seed in [(7, 1), (100, 3), (2000, 5), (30000, 7)]:
        mins, maxs = random_boxes(count, seed)
        on, oo = oracle.bvh_build(mins, maxs)
        for threads in (1, 4, 16):
            b = BVH.build(mins, maxs, threads=threads)
            assert np.array_equal(b.nodes, on) and np.array_equal(b.order, oo), (count, threads)


# ---- packing (tests/unit/scene.test.mjs:17-137) ----

def prim(packed, i):
    u = packed.primitives.reshape(-1, 16)[i]
    return {"kind": int(u[0]), "material": int(u[1]), "light": int(u[2]), "attributes": int(u[3]),
            "f": u.view(np.float32)}


def test_one_primitive_per_object_and_triangle():
    scene = Scene().add(Sphere(Vec3(0, 0, 0), 1, WHITE), Quad(Vec3(0, 0, 0), Vec3(1, 0, 0), Vec3(0, 0, 1), WHITE),
                        Box.fromCorners(Vec3(-1, -1, -1), Vec3(1, 1, 1), WHITE), Mesh.icosphere(WHITE, 1))
    packed = scene.pack()
    assert packed.primitiveCount == 3 + 80
    assert scene.primitiveCount == 83
    assert packed.primitives.nbytes == 83 * 64
    assert packed.nodes.nbytes == packed.nodeCount * BVH.NODE_BYTES
    assert len(packed.objects) == 83
    kinds = [prim(packed, i)["kind"] for i in range(83)]
    assert kinds.count(PRIMITIVE_KINDS["triangle"]) == 80
    assert all(k in kinds for k in (0, 1, 2))


def test_materials_shared():
    red = Material.plastic(Vec3(1, 0, 0), 0.3)
    packed = Scene().add(Sphere(Vec3(0, 0, 0), 1, red), Sphere(Vec3(3, 0, 0), 1, red),
                         Sphere(Vec3(6, 0, 0), 1, WHITE)).pack()
    f = packed.materials.view(np.float32)
    r = next(i for i, m in enumerate(packed.materialList) if m is red)
    assert packed.materialCount == 2
    assert list(f[r * 24:r * 24 + 3]) == [1, 0, 0]
    assert packed.materials[r * 24 + 3] == 2
    assert abs(f[r * 24 + 7] - 0.3) < 1e-6
    assert abs(f[r * 24 + 12] - 1.5) < 1e-6


def test_only_emissive_spheres_and_quads_are_lights():
    packed = Scene().add(Sphere(Vec3(0, 5, 0), 1, LAMP), Quad(Vec3(0, 4, 0), Vec3(1, 0, 0), Vec3(0, 0, 1), LAMP),
                         Box.fromCorners(Vec3(-1, -1, -1), Vec3(1, 1, 1), LAMP), Sphere(Vec3(0, 0, 0), 1, WHITE),
                         Sphere(Vec3(4, 0, 0), 1, Material.light(Vec3(1, 1, 1), 0.0))).pack()
    assert len(packed.lights) == 2
    for index, p in enumerate(packed.lights):
        assert prim(packed, int(p))["light"] == index
        assert isinstance(packed.objects[int(p)], (Sphere, Quad))
    for i in range(packed.primitiveCount):
        if i not in packed.lights:
            assert prim(packed, i)["light"] == NONE


def test_smooth_triangles_point_at_vertex_normals():
    smooth = Mesh.icosphere(WHITE, 0)
    flat = Mesh.icosphere(WHITE, 0, shading="flat")
    packed = Scene().add(smooth, flat).pack()
    for i in range(packed.primitiveCount):
        rec = prim(packed, i)
        if packed.objects[i] is flat:
            assert rec["attributes"] == NONE
        else:
            for k in range(3):
                n = packed.attributes[(rec["attributes"] + k) * 4:(rec["attributes"] + k) * 4 + 3]
                v = rec["f"][4 + k * 4:7 + k * 4]
                assert np.allclose(n, v, atol=1e-6)
            assert packed.attributes[(rec["attributes"] + 3) * 4 + 3] == 1


def test_packing_cached_until_objects_change():
    scene = Scene()
    first = scene.pack()
    assert scene.pack() is first
    version = scene.version
    sphere = Sphere(Vec3(0, 0, 0), 1, WHITE)
    scene.add(sphere)
    assert scene.version == version + 1
    assert scene.pack() is not first
    assert scene.remove(sphere) is True
    assert scene.remove(sphere) is False
    assert scene.pack().primitiveCount == 0


def test_empty_scene_packs_bindable_and_misses():
    scene = Scene()
    packed = scene.pack()
    assert packed.primitiveCount == 0
    assert packed.primitives.nbytes >= 64
    assert len(packed.lights) >= 1 and len(packed.attributes) >= 4
    assert packed.textures == []
    assert prim(packed, 0)["kind"] == NONE
    assert packed.nodes[7] == 1
    r = oracle.raycast(packed, np.array([0, 0, 5, 0, 0, -1], dtype=np.float32))
    assert r["prim"][0] == NONE
    assert scene.bounds() is None


def test_add_only_takes_scene_objects():
    with pytest.raises(TypeError):
        Scene().add(object())


# ---- raycast known answers (tests/unit/scene.test.mjs:139-315) ----

def cast(scene, origin, direction, max_distance=np.inf):
    packed = scene.pack()
    r = oracle.raycast(packed, np.array([*origin.tuple(), *direction.tuple()], dtype=np.float32), t_max=max_distance)
    if r["prim"][0] == NONE:
        return None
    return {"distance": r["t"][0], "normal": r["normal"][0], "front": bool(r["front"][0]),
            "point": np.array(origin.tuple()) + np.array(direction.tuple()) * r["t"][0]}


def test_sphere_near_side_or_far_from_inside():
    scene = Scene().add(Sphere(Vec3(0, 0, 0), 1, WHITE))
    out = cast(scene, Vec3(0, 0, 5), Vec3(0, 0, -1))
    assert abs(out["distance"] - 4) < 1e-6 and np.allclose(out["normal"], [0, 0, 1], atol=1e-6) and out["front"]
    ins = cast(scene, Vec3(0, 0, 0), Vec3(1, 0, 0))
    assert abs(ins["distance"] - 1) < 1e-6 and np.allclose(ins["normal"], [-1, 0, 0], atol=1e-6) and not ins["front"]
    assert cast(scene, Vec3(0, 2, 5), Vec3(0, 0, -1)) is None
    assert cast(scene, Vec3(0, 0, 5), Vec3(0, 0, -1), 3.9) is None


def test_distance_in_units_of_direction_length():
    hit = cast(Scene().add(Sphere(Vec3(0, 0, 0), 1, WHITE)), Vec3(0, 0, 5), Vec3(0, 0, -2))
    assert abs(hit["distance"] - 2) < 1e-6 and np.allclose(hit["point"], [0, 0, 1], atol=1e-6)


def test_quad_inside_edges_either_side():
    quad = Quad(Vec3(-1, 0, 1), Vec3(2, 0, 0), Vec3(0, 0, -2), WHITE)
    scene = Scene().add(quad)
    assert np.allclose(quad.normal.tuple(), (0, 1, 0)) and abs(quad.area - 4) < 1e-9
    above = cast(scene, Vec3(0.5, 3, 0.5), Vec3(0, -1, 0))
    assert abs(above["distance"] - 3) < 1e-6 and above["front"]
    below = cast(scene, Vec3(0.5, -3, 0.5), Vec3(0, 1, 0))
    assert not below["front"] and np.allclose(below["normal"], [0, -1, 0], atol=1e-6)
    assert cast(scene, Vec3(1.5, 3, 0), Vec3(0, -1, 0)) is None


def test_turned_stretched_box_faces():
    t = Mat4.translate(0, 1, 0).multiplyMat4(Mat4.rotateY(math.pi / 2)).multiplyMat4(Mat4.scale(2, 1, 1))
    scene = Scene().add(Box(t, WHITE))
    front = cast(scene, Vec3(0, 1, 10), Vec3(0, 0, -1))
    assert abs(front["distance"] - 8) < 1e-5 and np.allclose(front["normal"], [0, 0, 1], atol=1e-6)
    side = cast(scene, Vec3(10, 1, 0), Vec3(-1, 0, 0))
    assert abs(side["distance"] - 9) < 1e-5 and np.allclose(side["normal"], [1, 0, 0], atol=1e-6)
    top = cast(scene, Vec3(0.5, 10, 1.5), Vec3(0, -1, 0))
    assert abs(top["distance"] - 8) < 1e-5 and np.allclose(top["normal"], [0, 1, 0], atol=1e-6)
    inside = cast(scene, Vec3(0, 1, 0), Vec3(0, 1, 0))
    assert abs(inside["distance"] - 1) < 1e-5 and not inside["front"]


def test_smooth_triangles_interpolate_normals():
    scene = Scene().add(Mesh.icosphere(WHITE, 3))
    nxt = lcg(5)
    for _ in range(50):
        target = Vec3(nxt() - 0.5, nxt() - 0.5, nxt() - 0.5).normalized().scale(0.3)
        origin = Vec3(nxt() - 0.5, nxt() - 0.5, nxt() - 0.5).normalized().scale(4)
        hit = cast(scene, origin, target.subtract(origin))
        p = hit["point"]
        assert abs(np.linalg.norm(p) - 1.0) < 0.01
        assert np.dot(hit["normal"], p / np.linalg.norm(p)) > 0.999
        assert hit["front"]


def many_objects(nxt):
    objects = []
    for i in range(60):
        c = Vec3(nxt() * 10 - 5, nxt() * 10 - 5, nxt() * 10 - 5)
        kind = i % 4
        if kind == 0:
            objects.append(Sphere(c, 0.2 + nxt(), WHITE))
        elif kind == 1:
            objects.append(Quad(c, Vec3(nxt() * 2, nxt(), 0), Vec3(0, nxt(), nxt() * 2), WHITE))
        elif kind == 2:
            objects.append(Box.fromCorners(c, c.add(Vec3(nxt() + 0.1, nxt() + 0.1, nxt() + 0.1)), WHITE, nxt() * 3))
        else:
            objects.append(Mesh.torus(WHITE, radius=0.5, tube=0.2, segments=12, sides=6).transformed(
                Mat4.translate(c.x, c.y, c.z).multiplyMat4(Mat4.rotateX(nxt() * 3))))
    return objects


def test_nearest_of_many_matches_brute_force():
    nxt = lcg(11)
    objects = many_objects(nxt)
    scene = Scene().add(*objects)
    singles = [Scene().add(o) for o in objects]
    for _ in range(300):
        origin = Vec3(nxt() * 30 - 15, nxt() * 30 - 15, nxt() * 30 - 15)
        direction = Vec3(nxt() - 0.5, nxt() - 0.5, nxt() - 0.5)
        best = None
        for s in singles:
            h = cast(s, origin, direction)
            if h and (best is None or h["distance"] < best["distance"]):
                best = h
        hit = cast(scene, origin, direction)
        if best is None:
            assert hit is None
        else:
            assert hit is not None and abs(hit["distance"] - best["distance"]) <= 1e-6


def test_bounds_hold_every_object():
    scene = Scene().add(Sphere(Vec3(5, 0, 0), 1, WHITE), Box.fromCorners(Vec3(-3, -2, -1), Vec3(0, 0, 0), WHITE))
    b = scene.bounds()
    mn, mx = b["min"], b["max"]
    assert mn.x <= -3 and mn.y <= -2 and mn.z <= -1
    assert mx.x >= 6 and mx.y >= 1 and mx.z >= 1
    assert mn.x > -3.01 and mx.x < 6.01


def test_stick_between_points():
    a, b = Vec3(1, 2, 3), Vec3(-2, 4, 0)
    stick = Box.between(a, b, 0.2, WHITE)
    scene = Scene().add(stick)
    along = b.subtract(a).normalized()
    hit = cast(scene, a.subtract(along), along)
    assert abs(hit["distance"] - 1.0) < 1e-5 and np.allclose(hit["normal"], along.negate().tuple(), atol=1e-6)
    middle = a.add(b).scale(0.5)
    c = Vec3(stick.transform.value(0, 0), stick.transform.value(1, 0), stick.transform.value(2, 0))
    across = Vec3(c.x, c.y, c.z).normalized()
    assert abs(across.dot(along)) < 1e-9
    side = cast(scene, middle.add(across.scale(5)), across.negate())
    assert abs(side["distance"] - (5 - 0.1)) < 1e-5
    up = cast(Scene().add(Box.between(Vec3(0, 0, 0), Vec3(0, 3, 0), 0.1, WHITE)), Vec3(0, 10, 0), Vec3(0, -1, 0))
    assert up["distance"] - 7 < 1e-5
    with pytest.raises(ValueError):
        Box.between(a, a, 0.1, WHITE)


# ---- camera (tests/unit/camera.test.mjs) ----

def test_camera_axes():
    cam = Camera(position=Vec3(3, 4, 5), target=Vec3(-1, 0, 2))
    b = cam.basis()
    for axis in b.values():
        assert abs(axis.length() - 1.0) < 1e-9
    assert abs(b["right"].dot(b["up"])) < 1e-9 and abs(b["up"].dot(b["forward"])) < 1e-9
    assert np.allclose(b["forward"].tuple(), cam.target.subtract(cam.position).normalized().tuple(), atol=1e-6)
    assert np.allclose(b["right"].cross(b["up"]).tuple(), b["forward"].negate().tuple(), atol=1e-6)
    assert b["up"].y > 0


def test_camera_rays_at_fov():
    cam = Camera(position=Vec3(0, 0, 0), target=Vec3(0, 0, -1), fov=math.pi / 2)
    assert np.allclose(cam.ray(0, 0, 2.0)["direction"].tuple(), (0, 0, -1), atol=1e-6)
    assert np.allclose(cam.ray(0, 1, 2.0)["direction"].tuple(), Vec3(0, 1, -1).normalized().tuple(), atol=1e-6)
    assert np.allclose(cam.ray(1, 0, 2.0)["direction"].tuple(), Vec3(2, 0, -1).normalized().tuple(), atol=1e-6)
    assert np.allclose(cam.pixelRay(0, 0, 4, 2)["direction"].tuple(), cam.ray(-0.75, 0.5, 2.0)["direction"].tuple(),
                       atol=1e-6)


def test_focus_distance():
    cam = Camera(position=Vec3(0, 0, 10), target=Vec3(0, 0, 4))
    assert abs(cam.effectiveFocusDistance - 6.0) < 1e-9
    cam.focusDistance = 2.5
    assert abs(cam.effectiveFocusDistance - 2.5) < 1e-9
    cam.aperture = -1
    assert cam.aperture == 0
