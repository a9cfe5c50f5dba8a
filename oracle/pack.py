"""Scene.#pack restated (src/Scene.mjs:294-539) — TEST INFRASTRUCTURE ONLY.

The oracle's own packer of a scene's objects into the buffers the shader
reads, so that the product's packer (raymond_gb300/scene.py) is checked
against an independent restatement and the reference arm of the bench
never touches the product. It follows the reference step by step:

1. every object in order becomes primitives (a sphere, quad or box one, a
   mesh one per triangle) with a 16-float record, its extreme points'
   box padded by 1e-4·max(1, |min|, |max|) per axis (src/Scene.mjs:334-389)
   and, for a triangle with normals or texture coordinates, a 16-float
   attribute block (:412-423);
2. materials are numbered by identity as they are met (:300-311);
3. volumes leave the BVH and go after its primitives (:428-470);
4. BVH.build over the surfaces' boxes (the oracle's restatement,
   oracle/bvh.cpp), the records put in leaf order, each attribute block
   appended as its triangle is placed, and emissive spheres and quads
   listed as lights in that order (:472-491);
5. materials as 24 words each, textures and normal maps numbered as the
   materials meet them (:493-513).

The objects' derived values are worked out here as the reference's classes
do: a sphere's globe axes (src/Sphere.mjs:56-61), a box's inverse by
cofactors (src/Mat4.mjs:96-128, 363-390; src/Mat3.mjs:62-75;
src/Mat2.mjs:30-33) and its corners (src/Box.mjs:92-103), and a glass's
dispersion from its Abbe number (src/Material.mjs:196-200). Scene objects
are read by their fields only (center, radius, rotation; corner, u, v;
transform; positions, indices, normals, uvs; material), so any object
model with those fields packs here."""

from __future__ import annotations

import math

import numpy as np

NONE = 0xFFFFFFFF
KINDS = {"sphere": 0, "quad": 1, "box": 2, "triangle": 3}
MATERIAL_CODES = {"diffuse": 0, "metal": 1, "plastic": 2, "glass": 3, "light": 4, "volume": 5}
SMOOTH, TEXTURED = 1, 2
LAMBDA_F, LAMBDA_C = 0.4861, 0.6563


class Packed:
    """The packed buffers, with PackedScene's field names (src/Scene.mjs:44-60)."""

    def __init__(self, **fields):
        self.__dict__.update(fields)


def _kind(obj) -> str:
    if hasattr(obj, "indices"):
        return "mesh"
    if hasattr(obj, "radius") and hasattr(obj, "center"):
        return "sphere"
    if hasattr(obj, "corner"):
        return "quad"
    if hasattr(obj, "transform"):
        return "box"
    raise TypeError("A scene holds spheres, quads, boxes and meshes.")


def _values(m) -> list:
    """A Mat4's 16 values, row-major."""
    return [float(x) for x in m.v]


def _det2(a, b, c, d):
    return a * d - b * c


def _det3(v):
    # Expansion along the first row, minors left to right (src/Mat3.mjs:62-75).
    det = 0.0
    for col in range(3):
        rest = [v[r * 3 + c] for r in (1, 2) for c in range(3) if c != col]
        minor = _det2(*rest)
        det += v[col] * (-minor if col % 2 == 1 else minor)
    return det


def _cofactor(v, row, col):
    sub = [v[i * 4 + j] for i in range(4) for j in range(4) if i != row and j != col]
    minor = _det3(sub)
    return -minor if (row + col) % 2 == 1 else minor


def _inverse(v) -> list:
    """Mat4.inverse: the adjugate over the determinant, each cofactor divided
    by the determinant and written transposed (src/Mat4.mjs:96-128)."""
    det = 0.0
    for col in range(4):
        det += v[col] * _cofactor(v, 0, col)
    if det == 0.0:
        raise ValueError("The matrix has no inverse.")
    out = [0.0] * 16
    for row in range(4):
        for col in range(4):
            out[col * 4 + row] = _cofactor(v, row, col) / det
    return out


def _direction(v, x, y, z):
    return (v[0] * x + v[1] * y + v[2] * z, v[4] * x + v[5] * y + v[6] * z, v[8] * x + v[9] * y + v[10] * z)


def _point(v, x, y, z):
    return (v[0] * x + v[1] * y + v[2] * z + v[3], v[4] * x + v[5] * y + v[6] * z + v[7],
            v[8] * x + v[9] * y + v[10] * z + v[11])


def _normalized(p):
    length = math.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2])
    return (p[0] / length, p[1] / length, p[2] / length)


def _xyz(p):
    return (float(p.x), float(p.y), float(p.z))


def dispersion(m) -> float:
    if m.type != "glass" or m.abbe <= 0.0:
        return 0.0
    return (m.ior - 1.0) / (m.abbe * (LAMBDA_F ** -2 - LAMBDA_C ** -2))


def _padded(mn: np.ndarray, mx: np.ndarray):
    pad = 1e-4 * np.maximum(np.maximum(1.0, np.abs(mn)), np.abs(mx))
    return mn - pad, mx + pad


def box_corners(transform) -> list:
    """src/Box.mjs:92-103: the unit cube's corners, x outermost."""
    v = _values(transform)
    return [_point(v, x, y, z) for x in (-1.0, 1.0) for y in (-1.0, 1.0) for z in (-1.0, 1.0)]


def pack(objects, bvh_build=None) -> Packed:
    """The packed scene of `objects`, as Scene.#pack makes it."""
    if bvh_build is None:
        from . import bvh_build
    material_index, material_list = {}, []

    def material_of(m):
        i = material_index.get(id(m))
        if i is None:
            i = len(material_list)
            material_list.append(m)
            material_index[id(m)] = i
        return i

    # Step 1: per object, its primitives' records (f64, rounded when stored),
    # bounds and attribute blocks, in object order.
    rec_parts, min_parts, max_parts, block_parts, has_parts, owner_parts, mat_parts = [], [], [], [], [], [], []
    for oi, obj in enumerate(objects):
        kind = _kind(obj)
        if obj.material.type == "volume" and kind not in ("sphere", "box"):
            raise TypeError("A volume must be a Sphere or a Box.")
        mat = material_of(obj.material)
        if kind == "mesh":
            pos = np.asarray(obj.positions, dtype=np.float64).reshape(-1, 3)
            tri = np.asarray(obj.indices, dtype=np.int64).reshape(-1, 3)
            n = len(tri)
            a, b, c = pos[tri[:, 0]], pos[tri[:, 1]], pos[tri[:, 2]]
            rec = np.zeros((n, 12), dtype=np.float64)
            rec[:, 0:3], rec[:, 4:7], rec[:, 8:11] = a, b, c
            mn = np.minimum(np.minimum(a, b), c)
            mx = np.maximum(np.maximum(a, b), c)
            normals = None if obj.normals is None else np.asarray(obj.normals, dtype=np.float64).reshape(-1, 3)
            uvs = None if obj.uvs is None else np.asarray(obj.uvs, dtype=np.float64).reshape(-1, 2)
            blk = np.zeros((n, 16), dtype=np.float64)
            if normals is not None or uvs is not None:
                for k in range(3):
                    if normals is not None:
                        blk[:, 4 * k:4 * k + 3] = normals[tri[:, k]]
                    if uvs is not None:
                        blk[:, 4 * k + 3] = uvs[tri[:, k], 0]
                        blk[:, 12 + k] = uvs[tri[:, k], 1]
                blk[:, 15] = (SMOOTH if normals is not None else 0) + (TEXTURED if uvs is not None else 0)
                has = np.ones(n, dtype=bool)
            else:
                has = np.zeros(n, dtype=bool)
            kinds = np.full(n, KINDS["triangle"], dtype=np.uint32)
        else:
            if kind == "sphere":
                cx, cy, cz = _xyz(obj.center)
                r = float(obj.radius)
                rv = _values(obj.rotation)
                x = _normalized(_direction(rv, 1.0, 0.0, 0.0))
                north = _normalized(_direction(rv, 0.0, 1.0, 0.0))
                p = [cx, cy, cz, r, *x, 0.0, *north, 0.0]
                pts = [(cx - r, cy - r, cz - r), (cx + r, cy + r, cz + r)]
            elif kind == "quad":
                q, u, v = _xyz(obj.corner), _xyz(obj.u), _xyz(obj.v)
                qu = (q[0] + u[0], q[1] + u[1], q[2] + u[2])
                qv = (q[0] + v[0], q[1] + v[1], q[2] + v[2])
                quv = (qu[0] + v[0], qu[1] + v[1], qu[2] + v[2])
                p = [*q, 0.0, *u, 0.0, *v, 0.0]
                pts = [q, qu, qv, quv]
            else:
                inv = _inverse(_values(obj.transform))
                p = inv[:12]
                pts = box_corners(obj.transform)
            arr = np.array(pts, dtype=np.float64)
            mn, mx = arr.min(axis=0, keepdims=True), arr.max(axis=0, keepdims=True)
            rec = np.array([p], dtype=np.float64)
            blk = np.zeros((1, 16), dtype=np.float64)
            has = np.zeros(1, dtype=bool)
            kinds = np.array([KINDS[kind]], dtype=np.uint32)
        lo, hi = _padded(mn, mx)
        rec_parts.append((kinds, rec))
        min_parts.append(lo)
        max_parts.append(hi)
        block_parts.append(blk)
        has_parts.append(has)
        owner_parts.append(np.full(len(kinds), oi, dtype=np.int64))
        mat_parts.append(np.full(len(kinds), mat, dtype=np.uint32))

    total = sum(len(k) for k, _ in rec_parts)
    records = np.zeros((total, 16), dtype=np.uint32)
    if total:
        floats = records.view(np.float32)
        at = 0
        for kinds, rec in rec_parts:
            n = len(kinds)
            records[at:at + n, 0] = kinds
            floats[at:at + n, 4:16] = rec.astype(np.float32)
            at += n
        records[:, 1] = np.concatenate(mat_parts)
        records[:, 2] = NONE
        records[:, 3] = NONE
        mins = np.concatenate(min_parts)
        maxs = np.concatenate(max_parts)
        blocks = np.concatenate(block_parts)
        has_block = np.concatenate(has_parts)
        owners = np.concatenate(owner_parts)
    else:
        mins = maxs = np.zeros((0, 3))
        blocks = np.zeros((0, 16))
        has_block = np.zeros(0, dtype=bool)
        owners = np.zeros(0, dtype=np.int64)

    # Step 3: volumes out of the BVH.
    is_volume = np.array([material_list[int(m)].type == "volume" for m in records[:, 1]], dtype=bool)
    surface_ids = np.nonzero(~is_volume)[0]
    volume_ids = np.nonzero(is_volume)[0]
    count = len(surface_ids)

    # Step 4: the BVH, then the records in its leaf order.
    nodes, order = bvh_build(mins[surface_ids], maxs[surface_ids])
    nodes = nodes.copy()
    slots = max(count, 1)
    prims = np.zeros((slots + len(volume_ids), 16), dtype=np.uint32)
    if count == 0:
        prims[0, 0] = NONE
        nodes[7] = 1
    volume_list = []
    for k, vid in enumerate(volume_ids):
        prims[slots + k] = records[vid]
        volume_list.append(slots + k)
    attribute_list, light_list, packed_owners = [], [], []
    emissive = [m.type == "light" and (m.emission.x + m.emission.y + m.emission.z > 0.0) for m in material_list]
    for i in range(count):
        source = int(surface_ids[int(order[i])])
        prims[i] = records[source]
        packed_owners.append(int(owners[source]))
        if has_block[source]:
            prims[i, 3] = len(attribute_list) * 4
            attribute_list.append(source)
        if emissive[int(prims[i, 1])] and int(prims[i, 0]) in (KINDS["sphere"], KINDS["quad"]):
            prims[i, 2] = len(light_list)
            light_list.append(i)
    attributes = (blocks[np.array(attribute_list, dtype=np.int64)].astype(np.float32).reshape(-1)
                  if attribute_list else np.zeros(4, dtype=np.float32))

    # Step 5: materials and the texture lists they number.
    mats = np.zeros((max(len(material_list), 1), 24), dtype=np.uint32)
    mf = mats.view(np.float32)
    textures, tex_index, normal_maps, nrm_index = [], {}, [], {}

    def texture_of(t, index, lst):
        if t is None:
            return NONE
        i = index.get(id(t))
        if i is None:
            i = len(lst)
            lst.append(t)
            index[id(t)] = i
        return i

    for i, m in enumerate(material_list):
        mf[i, 0:3] = _xyz(m.color)
        mats[i, 3] = MATERIAL_CODES[m.type]
        mf[i, 4:8] = [*_xyz(m.emission), m.roughness]
        if m.checker is not None:
            mf[i, 8:12] = [*_xyz(m.checker), m.checkerSize]
        mf[i, 12] = m.ior
        mats[i, 13] = texture_of(m.texture, tex_index, textures)
        mf[i, 14:16] = [m.textureScale.x, m.textureScale.y]
        mats[i, 16] = texture_of(m.normalMap, nrm_index, normal_maps)
        mf[i, 17] = m.normalScale
        mats[i, 18] = texture_of(m.emissionTexture, tex_index, textures)
        mf[i, 19] = dispersion(m)
        mf[i, 20] = m.density
        mf[i, 21] = m.anisotropy

    return Packed(
        primitives=prims.reshape(-1), primitiveCount=count, nodes=nodes, nodeCount=len(nodes) // 8,
        materials=mats.reshape(-1), materialCount=len(material_list), attributes=attributes, textures=textures,
        normalMaps=normal_maps,
        lights=np.array(light_list if light_list else [NONE], dtype=np.uint32), volumes=volume_list,
        objects=[objects[k] for k in packed_owners], materialList=material_list,
        objectIndex=np.array(packed_owners, dtype=np.int64))
