"""tests/unit/mesh.test.mjs of the reference, restated for the Python
mirror (the meshes the workloads build: icospheres, surfaces, tori): closed meshes are watertight and wound outwards, they approximate
their shapes, smooth normals point out, transforms keep the winding, and
degenerate or malformed input is handled as there (ValueError for the
reference's RangeError)."""

import math

import numpy as np
import pytest

from raymond_gb300 import Mat4, Material, Mesh, Vec3

WHITE = Material.diffuse(Vec3(0.8, 0.8, 0.8))


def signed_volume(mesh):
    """By the divergence theorem: positive when triangles wind anticlockwise seen from outside."""
    p = mesh.positions
    t = mesh.indices.reshape(-1, 3).astype(np.int64)
    a, b, c = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def assert_watertight(mesh, name):
    """Every edge used once in each direction, edges compared by where their
    ends are (a texture seam repeats vertices)."""
    at = [" ".join(f"{c:.9f}" for c in p) for p in mesh.positions]
    t = mesh.indices.reshape(-1, 3)
    edges = {}
    for tri in t:
        for k in range(3):
            key = (at[tri[k]], at[tri[(k + 1) % 3]])
            edges[key] = edges.get(key, 0) + 1
    for (a, b), count in edges.items():
        assert count == 1, f"{name}: edge used once"
        assert edges.get((b, a)) == 1, f"{name}: edge has a twin"


CLOSED = {
    "icosphere": lambda: Mesh.icosphere(WHITE, 2),
    "torus": lambda: Mesh.torus(WHITE, radius=1.0, tube=0.3, segments=24, sides=12),
}


@pytest.mark.parametrize("name", list(CLOSED))
def test_closed_meshes_are_watertight_and_wound_outwards(name):
    mesh = CLOSED[name]()
    assert_watertight(mesh, name)
    assert signed_volume(mesh) > 0.0


def test_meshes_approximate_their_shapes():
    assert abs(signed_volume(Mesh.icosphere(WHITE, 4)) - 4.0 / 3.0 * math.pi) <= 0.01
    torus = Mesh.torus(WHITE, radius=1.0, tube=0.3, segments=96, sides=48)
    assert abs(signed_volume(torus) - 2.0 * math.pi * math.pi * 1.0 * 0.09) <= 0.01
    for p in Mesh.icosphere(WHITE, 2).positions:
        assert abs(np.linalg.norm(p) - 1.0) < 1e-9


@pytest.mark.parametrize("name", list(CLOSED))
def test_smooth_normals_are_unit_and_point_outwards(name):
    mesh = CLOSED[name]()
    n = mesh.normals
    assert np.all(np.abs(np.linalg.norm(n, axis=1) - 1.0) < 1e-9)
    t = mesh.indices.reshape(-1, 3).astype(np.int64)
    p = mesh.positions
    face = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    for k in range(3):
        assert np.all(np.einsum("ij,ij->i", n[t[:, k]], face) > 0.0)


def test_flat_meshes_have_no_vertex_normals():
    assert Mesh.icosphere(WHITE, 1, shading="flat").normals is None


@pytest.mark.parametrize("transform", [Mat4.scale(2, 1, 0.5), Mat4.scale(-1, 1, 1),
                                       Mat4.translate(3, 0, 0).multiplyMat4(Mat4.rotateX(1))])
def test_transforms_keep_meshes_wound_outwards(transform):
    moved = Mesh.icosphere(WHITE, 1).transformed(transform)
    assert signed_volume(moved) > 0.0
    p, n = moved.positions, moved.normals
    t = moved.indices.reshape(-1, 3).astype(np.int64)
    face = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    face /= np.linalg.norm(face, axis=1)[:, None]
    assert np.all(np.einsum("ij,ij->i", n[t[:, 0]], face) > 0.5)


def test_surfaces_drop_degenerate_triangles():
    def sphere(u, v):
        theta, phi = u * math.pi, v * 2.0 * math.pi
        return Vec3(math.sin(theta) * math.cos(phi), math.cos(theta), math.sin(theta) * math.sin(phi))

    mesh = Mesh.surface(sphere, 8, 12, WHITE, vWrap="closed")
    # 8 × 12 cells of two triangles, less one of each pair at each pole
    assert mesh.triangleCount == 8 * 12 * 2 - 2 * 12


def test_bad_meshes_are_refused():
    p = [Vec3(0, 0, 0), Vec3(1, 0, 0), Vec3(0, 1, 0)]
    with pytest.raises(ValueError):
        Mesh(p, [0, 1], WHITE)  # not a multiple of 3
    with pytest.raises(ValueError):
        Mesh(p, [0, 1, 3], WHITE)  # no vertex 3
    with pytest.raises(ValueError):
        Mesh(p, [0, 1, 2], WHITE, normals=[Vec3(0, 0, 1)])  # too few normals

