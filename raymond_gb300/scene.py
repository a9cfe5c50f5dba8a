"""Scenes and their packed GPU form (src/Scene.mjs:15-539) and the BVH
(src/BVH.mjs). The packed layout is the drop-in contract: 64-byte
primitives in BVH leaf order then volumes, 32-byte nodes, 96-byte
materials, 16-float attribute blocks, the lights list."""

from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .geometry import Box, Mesh, Quad, Sphere
from .material import MATERIAL_TYPES
from .sky import Sky
from .vec import Mat4, Vec3

PRIMITIVE_KINDS = {"sphere": 0, "quad": 1, "box": 2, "triangle": 3}
NONE = 0xFFFFFFFF
SMOOTH, TEXTURED = 1, 2
PRIMITIVE_FLOATS = 16
MATERIAL_FLOATS = 24


class BVH:
    """A packed binned-SAH BVH (src/BVH.mjs), built natively."""

    NODE_BYTES = 32

    def __init__(self, nodes: np.ndarray, node_count: int, order: np.ndarray):
        self.nodes = nodes
        self.nodeCount = node_count
        self.order = order

    @staticmethod
    def build(mins, maxs, maxLeafSize: int = 4, threads: int | None = None) -> "BVH":
        mins = np.ascontiguousarray(mins, dtype=np.float64).reshape(-1)
        maxs = np.ascontiguousarray(maxs, dtype=np.float64).reshape(-1)
        count = mins.size // 3
        nodes = np.zeros(max(1, 2 * count - 1) * 8, dtype=np.uint32)
        order = np.zeros(count, dtype=np.uint32)
        n = _native.lib().raymond_bvh_build(_native.ptr(mins), _native.ptr(maxs), count, maxLeafSize,
                                            _native.ptr(nodes), _native.ptr(order),
                                            threads if threads else (os.cpu_count() or 1))
        if n == 0:
            raise ValueError("BVH build failed: bad arguments")
        return BVH(nodes[: n * 8].copy(), int(n), order)


@dataclass
class PackedScene:
    primitives: np.ndarray        # uint32, 16 words per slot (floats viewable via .view(np.float32))
    primitiveCount: int
    nodes: np.ndarray             # uint32, 8 words per node
    nodeCount: int
    materials: np.ndarray         # uint32, 24 words per material
    materialCount: int
    attributes: np.ndarray        # float32, 16 per block
    textures: list
    normalMaps: list
    lights: np.ndarray            # uint32 primitive indices, [NONE] if none
    volumes: list
    objects: list                 # the object each BVH primitive came from
    materialList: list
    objectIndex: np.ndarray = field(default=None)  # per BVH primitive: index of its object in the scene


class Scene:
    """Objects and sky (src/Scene.mjs:97-200)."""

    def __init__(self, sky: Sky | None = None):
        self._objects = []
        self.sky = sky if sky is not None else Sky()
        self._version = 0
        self._packed = None

    @property
    def objects(self):
        return list(self._objects)

    @property
    def version(self):
        return self._version

    def add(self, *objects):
        for o in objects:
            if not isinstance(o, (Sphere, Quad, Box, Mesh)):
                raise TypeError("Scenes hold Spheres, Quads, Boxes and Meshes.")
        self._objects.extend(objects)
        self._changed()
        return self

    def remove(self, obj) -> bool:
        for i, o in enumerate(self._objects):
            if o is obj:
                del self._objects[i]
                self._changed()
                return True
        return False

    def clear(self):
        self._objects = []
        self._changed()

    @property
    def primitiveCount(self) -> int:
        return sum(o.triangleCount if isinstance(o, Mesh) else 1 for o in self._objects)

    def bounds(self):
        packed = self.pack()
        if packed.primitiveCount == 0:
            return None
        f = packed.nodes[:8].view(np.float32)
        return {"min": Vec3(f[0], f[1], f[2]), "max": Vec3(f[4], f[5], f[6])}

    def pack(self) -> PackedScene:
        if self._packed is None:
            self._packed = pack_objects(self._objects)
        return self._packed

    def _changed(self):
        self._version += 1
        self._packed = None


def _pad_bounds(mn: np.ndarray, mx: np.ndarray):
    """Bounds padding 1e-4·max(1, |min|, |max|) per axis (src/Scene.mjs:383-387)."""
    pad = 1e-4 * np.maximum(np.maximum(1.0, np.abs(mn)), np.abs(mx))
    return mn - pad, mx + pad


def pack_objects(objects) -> PackedScene:
    """Scene.#pack (src/Scene.mjs:294-539)."""
    material_index, material_list = {}, []

    def material_of(m):
        i = material_index.get(id(m))
        if i is None:
            i = len(material_list)
            material_list.append(m)
            material_index[id(m)] = i
        return i

    # Per object: records (n,16) float32 with header words, bounds (n,3)×2 in double, blocks or None.
    rec_parts, min_parts, max_parts, block_parts, has_block_parts, owner_parts = [], [], [], [], [], []
    # Materials are numbered in object order, as the reference meets them.
    mat_ids = [material_of(o.material) for o in objects]
    # Unrotated spheres pack in bulk (their globe axes are x and y); records
    # are put back in object order below.
    identity = Mat4.identity().v
    bulk = [oi for oi, o in enumerate(objects) if type(o) is Sphere and o.rotation.v == identity]
    bulk_set = set(bulk)
    if bulk:
        n = len(bulk)
        cr = np.array([(objects[i].center.x, objects[i].center.y, objects[i].center.z, objects[i].radius)
                       for i in bulk], dtype=np.float64)
        mats = np.array([mat_ids[i] for i in bulk], dtype=np.uint32)
        rec = np.zeros((n, 16), dtype=np.float32)
        rec[:, 4:8] = cr
        rec[:, 8] = 1.0   # globe x axis
        rec[:, 13] = 1.0  # north pole
        hdr = rec.view(np.uint32)
        hdr[:, 0] = PRIMITIVE_KINDS["sphere"]
        hdr[:, 1] = mats
        hdr[:, 2] = NONE
        hdr[:, 3] = NONE
        mn, mx = _pad_bounds(cr[:, :3] - cr[:, 3:4], cr[:, :3] + cr[:, 3:4])
        rec_parts.append(rec)
        min_parts.append(mn)
        max_parts.append(mx)
        block_parts.append(np.zeros((n, 16), dtype=np.float32))
        has_block_parts.append(np.zeros(n, dtype=bool))
        owner_parts.append(np.array(bulk, dtype=np.int64))
    for oi, obj in enumerate(objects):
        if oi in bulk_set:
            continue
        if obj.material.type == "volume" and not isinstance(obj, (Sphere, Box)):
            raise TypeError("A volume must be a Sphere or a Box.")
        mat = mat_ids[oi]
        if isinstance(obj, Mesh):
            tri = obj.indices.reshape(-1, 3).astype(np.int64)
            n = len(tri)
            p = obj.positions
            a, b, c = p[tri[:, 0]], p[tri[:, 1]], p[tri[:, 2]]
            rec = np.zeros((n, 16), dtype=np.float32)
            rec[:, 4:7], rec[:, 8:11], rec[:, 12:15] = a, b, c
            hdr = rec.view(np.uint32)
            hdr[:, 0] = PRIMITIVE_KINDS["triangle"]
            hdr[:, 1] = mat
            hdr[:, 2] = NONE
            hdr[:, 3] = NONE
            mn = np.minimum(np.minimum(a, b), c)
            mx = np.maximum(np.maximum(a, b), c)
            if obj.normals is not None or obj.uvs is not None:
                blk = np.zeros((n, 16), dtype=np.float32)
                if obj.normals is not None:
                    for k in range(3):
                        blk[:, k * 4: k * 4 + 3] = obj.normals[tri[:, k]]
                if obj.uvs is not None:
                    for k in range(3):
                        blk[:, k * 4 + 3] = obj.uvs[tri[:, k], 0]
                        blk[:, 12 + k] = obj.uvs[tri[:, k], 1]
                blk[:, 15] = (SMOOTH if obj.normals is not None else 0) + (TEXTURED if obj.uvs is not None else 0)
                block_parts.append(blk)
                has_block_parts.append(np.ones(n, dtype=bool))
            else:
                block_parts.append(np.zeros((n, 16), dtype=np.float32))
                has_block_parts.append(np.zeros(n, dtype=bool))
        else:
            rec = np.zeros((1, 16), dtype=np.float32)
            hdr = rec.view(np.uint32)
            if isinstance(obj, Sphere):
                c, r = obj.center, obj.radius
                ax = obj.axes()
                x, north = ax["x"], ax["north"]
                rec[0, 4:16] = [c.x, c.y, c.z, r, x.x, x.y, x.z, 0.0, north.x, north.y, north.z, 0.0]
                hdr[0, 0] = PRIMITIVE_KINDS["sphere"]
                pts = [c.subtract(Vec3(r, r, r)), c.add(Vec3(r, r, r))]
            elif isinstance(obj, Quad):
                q, u, v = obj.corner, obj.u, obj.v
                rec[0, 4:16] = [q.x, q.y, q.z, 0.0, u.x, u.y, u.z, 0.0, v.x, v.y, v.z, 0.0]
                hdr[0, 0] = PRIMITIVE_KINDS["quad"]
                pts = [q, q.add(u), q.add(v), q.add(u).add(v)]
            else:
                m = obj.inverse
                rec[0, 4:16] = [m.value(r_, c_) for r_ in range(3) for c_ in range(4)]
                hdr[0, 0] = PRIMITIVE_KINDS["box"]
                pts = obj.corners()
            hdr[0, 1] = mat
            hdr[0, 2] = NONE
            hdr[0, 3] = NONE
            arr = np.array([[p.x, p.y, p.z] for p in pts], dtype=np.float64)
            mn = arr.min(axis=0, keepdims=True)
            mx = arr.max(axis=0, keepdims=True)
            block_parts.append(np.zeros((1, 16), dtype=np.float32))
            has_block_parts.append(np.zeros(1, dtype=bool))
        mn, mx = _pad_bounds(mn, mx)
        rec_parts.append(rec)
        min_parts.append(mn)
        max_parts.append(mx)
        owner_parts.append(np.full(len(rec), oi, dtype=np.int64))

    if rec_parts:
        records = np.concatenate(rec_parts)
        mins_all = np.concatenate(min_parts)
        maxs_all = np.concatenate(max_parts)
        blocks = np.concatenate(block_parts)
        has_block = np.concatenate(has_block_parts)
        owners = np.concatenate(owner_parts)
        if bulk:
            order = np.argsort(owners, kind="stable")
            records, mins_all, maxs_all = records[order], mins_all[order], maxs_all[order]
            blocks, has_block, owners = blocks[order], has_block[order], owners[order]
    else:
        records = np.zeros((0, 16), dtype=np.float32)
        mins_all = maxs_all = np.zeros((0, 3))
        blocks = np.zeros((0, 16), dtype=np.float32)
        has_block = np.zeros(0, dtype=bool)
        owners = np.zeros(0, dtype=np.int64)

    rec_u = records.view(np.uint32)
    vol_material = np.array([m.type == "volume" for m in material_list], dtype=bool)
    is_volume = vol_material[rec_u[:, 1]] if len(records) else np.zeros(0, dtype=bool)
    surface_ids = np.nonzero(~is_volume)[0]
    volume_ids = np.nonzero(is_volume)[0]
    count = len(surface_ids)

    bvh = BVH.build(mins_all[surface_ids], maxs_all[surface_ids])
    slots = max(count, 1)
    prims = np.zeros((slots + len(volume_ids), 16), dtype=np.uint32)
    nodes = bvh.nodes.copy()
    if count == 0:
        prims[0, 0] = NONE
        nodes[7] = 1  # an empty scene's root is a leaf of one primitive nothing hits

    for k, vid in enumerate(volume_ids):
        prims[slots + k] = rec_u[vid]
    volume_list = [slots + k for k in range(len(volume_ids))]

    source = surface_ids[bvh.order.astype(np.int64)] if count else np.zeros(0, dtype=np.int64)
    if count:
        prims[:count] = rec_u[source]
        # Attribute blocks in leaf order.
        hb = has_block[source]
        block_index = np.cumsum(hb) - 1
        prims[:count, 3] = np.where(hb, (block_index * 4).astype(np.uint32), NONE)
        attributes = blocks[source[hb]].reshape(-1)
        # Lights: emissive spheres and quads, in leaf order.
        emissive = np.array([m.emissive for m in material_list], dtype=bool)
        kinds = prims[:count, 0]
        is_light = emissive[prims[:count, 1]] & ((kinds == 0) | (kinds == 1))
        light_list = np.nonzero(is_light)[0].astype(np.uint32)
        prims[light_list, 2] = np.arange(len(light_list), dtype=np.uint32)
    else:
        attributes = np.zeros(0, dtype=np.float32)
        light_list = np.zeros(0, dtype=np.uint32)

    mats = np.zeros((max(len(material_list), 1), MATERIAL_FLOATS), dtype=np.float32)
    mu = mats.view(np.uint32)
    tex_index, tex_list, nrm_index, nrm_list = {}, [], {}, []

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
        mats[i, 0:3] = [m.color.x, m.color.y, m.color.z]
        mu[i, 3] = MATERIAL_TYPES[m.type]
        mats[i, 4:8] = [m.emission.x, m.emission.y, m.emission.z, m.roughness]
        if m.checker is not None:
            mats[i, 8:12] = [m.checker.x, m.checker.y, m.checker.z, m.checkerSize]
        mats[i, 12] = m.ior
        mu[i, 13] = texture_of(m.texture, tex_index, tex_list)
        mats[i, 14:16] = [m.textureScale.x, m.textureScale.y]
        mu[i, 16] = texture_of(m.normalMap, nrm_index, nrm_list)
        mats[i, 17] = m.normalScale
        mu[i, 18] = texture_of(m.emissionTexture, tex_index, tex_list)
        mats[i, 19] = m.dispersion
        mats[i, 20] = m.density
        mats[i, 21] = m.anisotropy

    objs = [objects[int(o)] for o in owners[source]] if count else []
    return PackedScene(
        primitives=prims.reshape(-1),
        primitiveCount=count,
        nodes=nodes,
        nodeCount=bvh.nodeCount,
        materials=mu.reshape(-1).copy(),
        materialCount=len(material_list),
        attributes=attributes.astype(np.float32) if attributes.size else np.zeros(4, dtype=np.float32),
        textures=tex_list,
        normalMaps=nrm_list,
        lights=light_list if light_list.size else np.array([NONE], dtype=np.uint32),
        volumes=volume_list,
        objects=objs,
        materialList=material_list,
        objectIndex=owners[source] if count else np.zeros(0, dtype=np.int64),
    )
