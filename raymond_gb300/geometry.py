"""Scene objects (src/Sphere.mjs, src/Quad.mjs, src/Box.mjs, src/Mesh.mjs).

Meshes keep their vertices as float64 numpy arrays rather than lists of
Vec3, so scenes of millions of triangles pack quickly; the arithmetic (area-
weighted vertex normals, degenerate-triangle removal, transforms) keeps the
reference's operation order."""

from __future__ import annotations

import math

import numpy as np

from .vec import Mat4, Vec3


class Sphere:
    def __init__(self, center: Vec3, radius: float, material, rotation: Mat4 | None = None):
        if not (radius > 0.0):
            raise ValueError("A sphere's radius must be more than 0.")
        self.center = center
        self.radius = float(radius)
        self.material = material
        self.rotation = rotation if rotation is not None else Mat4.identity()

    def axes(self):
        """The globe's x axis and north pole, for textures (src/Sphere.mjs)."""
        return {"x": self.rotation.multiplyDirection(Vec3(1, 0, 0)).normalized(),
                "north": self.rotation.multiplyDirection(Vec3(0, 1, 0)).normalized()}


class Quad:
    def __init__(self, corner: Vec3, u: Vec3, v: Vec3, material):
        if not (u.cross(v).length() > 0.0):
            raise ValueError("A quad's edges must not be parallel.")
        self.corner, self.u, self.v, self.material = corner, u, v, material

    @property
    def normal(self):
        return self.u.cross(self.v).normalized()

    @property
    def area(self):
        return self.u.cross(self.v).length()


class Box:
    def __init__(self, transform: Mat4, material):
        self.transform = transform
        self.inverse = transform.inverse()
        self.material = material

    @staticmethod
    def fromCorners(mn: Vec3, mx: Vec3, material, rotateY: float = 0.0) -> "Box":
        center = mn.add(mx).scale(0.5)
        half = mx.subtract(mn).scale(0.5)
        t = (Mat4.translate(center.x, center.y, center.z).multiplyMat4(Mat4.rotateY(rotateY))
             .multiplyMat4(Mat4.scale(half.x, half.y, half.z)))
        return Box(t, material)

    @staticmethod
    def between(a: Vec3, b: Vec3, thickness: float, material) -> "Box":
        center = a.add(b).scale(0.5)
        along = b.subtract(a)
        half_length = along.length() / 2.0
        if not (half_length > 0.0):
            raise ValueError("A stick's ends must differ.")
        z = along.normalized()
        helper = Vec3(0, 1, 0) if abs(z.y) < 0.9 else Vec3(1, 0, 0)
        x = helper.cross(z).normalized()
        y = z.cross(x)
        t = thickness / 2.0
        return Box(Mat4(x.x * t, y.x * t, z.x * half_length, center.x,
                        x.y * t, y.y * t, z.y * half_length, center.y,
                        x.z * t, y.z * t, z.z * half_length, center.z,
                        0.0, 0.0, 0.0, 1.0), material)

    def corners(self):
        return [self.transform.multiplyVector3(Vec3(x, y, z))
                for x in (-1.0, 1.0) for y in (-1.0, 1.0) for z in (-1.0, 1.0)]


def _points(values) -> np.ndarray:
    if isinstance(values, np.ndarray):
        a = np.asarray(values, dtype=np.float64)
        return a.reshape(-1, a.shape[-1]) if a.ndim > 1 else a.reshape(-1, 3)
    return np.array([[p.x, p.y, p.z] for p in values], dtype=np.float64).reshape(-1, 3)


def _uvs(values) -> np.ndarray:
    if isinstance(values, np.ndarray):
        return np.asarray(values, dtype=np.float64).reshape(-1, 2)
    return np.array([[p.x, p.y] for p in values], dtype=np.float64).reshape(-1, 2)


def _cross(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)


def _length(a: np.ndarray) -> np.ndarray:
    return np.sqrt(a[:, 0] * a[:, 0] + a[:, 1] * a[:, 1] + a[:, 2] * a[:, 2])


class Mesh:
    """Triangles over shared vertices (src/Mesh.mjs)."""

    def __init__(self, positions, indices, material, shading="smooth", normals=None, uvs=None):
        pos = _points(positions)
        idx = np.asarray(indices, dtype=np.int64).reshape(-1)
        if idx.size % 3 != 0:
            raise ValueError("A mesh needs three indices per triangle.")
        if idx.size and (idx.min() < 0 or idx.max() >= len(pos)):
            bad = idx[(idx < 0) | (idx >= len(pos))][0]
            raise ValueError(f"Index {bad} has no vertex.")
        nrm = _points(normals) if normals is not None else None
        if nrm is not None and len(nrm) != len(pos):
            raise ValueError("A mesh needs one normal per vertex.")
        uv = _uvs(uvs) if uvs is not None else None
        if uv is not None and len(uv) != len(pos):
            raise ValueError("A mesh needs one texture coordinate per vertex.")
        self.positions = pos
        self.indices = idx.astype(np.uint32)
        self.material = material
        if nrm is None and shading == "smooth":
            nrm = Mesh.vertexNormals(pos, self.indices)
        self.normals = nrm
        self.uvs = uv

    @property
    def triangleCount(self) -> int:
        return self.indices.size // 3

    def transformed(self, transform: Mat4) -> "Mesh":
        m = transform.v
        p = self.positions
        positions = np.stack([m[0] * p[:, 0] + m[1] * p[:, 1] + m[2] * p[:, 2] + m[3],
                              m[4] * p[:, 0] + m[5] * p[:, 1] + m[6] * p[:, 2] + m[7],
                              m[8] * p[:, 0] + m[9] * p[:, 1] + m[10] * p[:, 2] + m[11]], axis=1)
        indices = self.indices
        if transform.determinant() < 0.0:
            indices = indices.reshape(-1, 3)[:, [0, 2, 1]].reshape(-1)
        normals = None
        if self.normals is not None:
            nm = transform.inverse().transpose().v
            n = self.normals
            d = np.stack([nm[0] * n[:, 0] + nm[1] * n[:, 1] + nm[2] * n[:, 2],
                          nm[4] * n[:, 0] + nm[5] * n[:, 1] + nm[6] * n[:, 2],
                          nm[8] * n[:, 0] + nm[9] * n[:, 1] + nm[10] * n[:, 2]], axis=1)
            normals = d / _length(d)[:, None]
        return Mesh(positions, indices, self.material, shading="flat", normals=normals, uvs=self.uvs)

    @staticmethod
    def vertexNormals(positions: np.ndarray, indices: np.ndarray) -> np.ndarray:
        """Area-weighted face normals summed per vertex, in triangle order (src/Mesh.mjs:358-378)."""
        tri = indices.reshape(-1, 3).astype(np.int64)
        a, b, c = positions[tri[:, 0]], positions[tri[:, 1]], positions[tri[:, 2]]
        n = _cross(b - a, c - a)
        sums = np.zeros_like(positions)
        np.add.at(sums, tri.reshape(-1), np.repeat(n, 3, axis=0))
        length = _length(sums)
        out = np.empty_like(sums)
        ok = length > 0.0
        out[ok] = sums[ok] / length[ok, None]
        out[~ok] = (0.0, 1.0, 0.0)
        return out

    @staticmethod
    def withoutDegenerates(positions: np.ndarray, indices) -> np.ndarray:
        """Drops triangles of area ≤ 1e-12 (src/Mesh.mjs:385-400)."""
        tri = np.asarray(indices, dtype=np.int64).reshape(-1, 3)
        a, b, c = positions[tri[:, 0]], positions[tri[:, 1]], positions[tri[:, 2]]
        keep = _length(_cross(b - a, c - a)) > 1e-12
        return tri[keep].reshape(-1)

    @staticmethod
    def surface(point, uSegments: int, vSegments: int, material, uWrap="open", vWrap="open",
                shading="smooth") -> "Mesh":
        """A parametric grid (src/Mesh.mjs:127-181)."""
        u_rows = uSegments + 1 if uWrap == "open" else uSegments
        v_rows = vSegments + 1 if vWrap == "open" else vSegments
        welded = []
        for i in range(u_rows):
            for j in range(v_rows):
                p = point(i / uSegments, j / vSegments)
                welded.append((p.x, p.y, p.z))
        welded = np.array(welded, dtype=np.float64)
        ii, jj = np.meshgrid(np.arange(uSegments + 1), np.arange(vSegments + 1), indexing="ij")
        weld_index = (ii % u_rows) * v_rows + (jj % v_rows)
        positions = welded[weld_index.reshape(-1)]
        uvs = np.stack([(ii / uSegments).reshape(-1), (jj / vSegments).reshape(-1)], axis=1)
        columns = vSegments + 1
        gi, gj = np.meshgrid(np.arange(uSegments), np.arange(vSegments), indexing="ij")
        gi, gj = gi.reshape(-1), gj.reshape(-1)

        def full(i, j):
            return i * columns + j

        def weld(i, j):
            return (i % u_rows) * v_rows + (j % v_rows)

        indices = np.stack([full(gi, gj), full(gi + 1, gj), full(gi + 1, gj + 1),
                            full(gi, gj), full(gi + 1, gj + 1), full(gi, gj + 1)], axis=1).reshape(-1)
        welded_idx = np.stack([weld(gi, gj), weld(gi + 1, gj), weld(gi + 1, gj + 1),
                               weld(gi, gj), weld(gi + 1, gj + 1), weld(gi, gj + 1)], axis=1).reshape(-1)
        normals = None
        if shading == "smooth":
            wn = Mesh.vertexNormals(welded, Mesh.withoutDegenerates(welded, welded_idx).astype(np.uint32))
            normals = wn[weld_index.reshape(-1)]
        return Mesh(positions, Mesh.withoutDegenerates(positions, indices), material, shading=shading,
                    normals=normals, uvs=uvs)

    @staticmethod
    def icosphere(material, subdivisions: int = 3, shading="smooth") -> "Mesh":
        """A unit sphere by midpoint subdivision of an icosahedron (src/Mesh.mjs:190-237)."""
        t = (1.0 + math.sqrt(5.0)) / 2.0
        base = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
        positions = [Vec3(*p).normalized().tuple() for p in base]
        faces = [0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11,
                 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
                 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9,
                 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1]
        for _ in range(subdivisions):
            midpoints = {}

            def midpoint(a, b):
                key = (a, b) if a < b else (b, a)
                idx = midpoints.get(key)
                if idx is None:
                    pa, pb = positions[a], positions[b]
                    s = Vec3(pa[0] + pb[0], pa[1] + pb[1], pa[2] + pb[2]).normalized()
                    idx = len(positions)
                    positions.append(s.tuple())
                    midpoints[key] = idx
                return idx

            nxt = []
            for i in range(0, len(faces), 3):
                a, b, c = faces[i], faces[i + 1], faces[i + 2]
                ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
                nxt += [a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca]
            faces = nxt
        pos = np.array(positions, dtype=np.float64)
        if shading == "smooth":
            return Mesh(pos, faces, material, normals=pos)
        return Mesh(pos, faces, material, shading=shading)

    @staticmethod
    def torus(material, radius=1.0, tube=0.35, segments=64, sides=32) -> "Mesh":
        """src/Mesh.mjs:293-303."""
        def point(u, v):
            a = u * 2.0 * math.pi
            b = v * 2.0 * math.pi
            r = radius + tube * math.cos(b)
            return Vec3(r * math.cos(a), tube * math.sin(b), -r * math.sin(a))
        return Mesh.surface(point, segments, sides, material, uWrap="closed", vWrap="closed")
