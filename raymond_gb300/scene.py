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

    # Every object's records go straight to their place in object order:
    # records (16 words, header words as u32), bounds in double, attribute
    # blocks and whether there is one, and the owning object's index.
    mat_ids = [material_of(o.material) for o in objects]  # numbered as the reference meets them
    counts = np.array([o.triangleCount if isinstance(o, Mesh) else 1 for o in objects], dtype=np.int64)
    offsets = np.zeros(len(objects) + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    total = int(offsets[-1])
    records = np.zeros((total, 16), dtype=np.float32)
    hdr_all = records.view(np.uint32)
    mins_all = np.zeros((total, 3))
    maxs_all = np.zeros((total, 3))
    blocks = np.zeros((total, 16), dtype=np.float32)
    has_block = np.zeros(total, dtype=bool)
    owners = np.repeat(np.arange(len(objects), dtype=np.int64), counts)
    hdr_all[:, 2] = NONE
    hdr_all[:, 3] = NONE

    # Unrotated spheres pack in bulk (their globe axes are x and y).
    identity = Mat4.identity().v
    bulk = [oi for oi, o in enumerate(objects) if type(o) is Sphere and o.rotation.v == identity]
    bulk_set = set(bulk)
    if bulk:
        at = offsets[np.array(bulk, dtype=np.int64)]
        cr = np.array([(objects[i].center.x, objects[i].center.y, objects[i].center.z, objects[i].radius)
                       for i in bulk], dtype=np.float64)
        records[at, 4:8] = cr
        records[at, 8] = 1.0   # globe x axis
        records[at, 13] = 1.0  # north pole
        hdr_all[at, 0] = PRIMITIVE_KINDS["sphere"]
        hdr_all[at, 1] = np.array([mat_ids[i] for i in bulk], dtype=np.uint32)
        mins_all[at], maxs_all[at] = _pad_bounds(cr[:, :3] - cr[:, 3:4], cr[:, :3] + cr[:, 3:4])
    for oi, obj in enumerate(objects):
        if oi in bulk_set:
            continue
        if obj.material.type == "volume" and not isinstance(obj, (Sphere, Box)):
            raise TypeError("A volume must be a Sphere or a Box.")
        lo, hi = int(offsets[oi]), int(offsets[oi + 1])
        rec, hdr = records[lo:hi], hdr_all[lo:hi]
        hdr[:, 1] = mat_ids[oi]
        if isinstance(obj, Mesh):
            n = hi - lo
            tri = obj.indices.reshape(-1, 3).astype(np.int64)
            # Corners in double for the bounds; the records take them
            # rounded to f32, rounded per vertex before the gather (the same
            # values, a third of the conversions).
            pt = np.take(obj.positions, tri, axis=0)
            rec[:, 4:16].reshape(n, 3, 4)[:, :, :3] = np.take(obj.positions.astype(np.float32), tri, axis=0)
            hdr[:, 0] = PRIMITIVE_KINDS["triangle"]
            a, b, c = pt[:, 0], pt[:, 1], pt[:, 2]
            mn = np.minimum(np.minimum(a, b), c)
            mx = np.maximum(np.maximum(a, b), c)
            if obj.normals is not None or obj.uvs is not None:
                blk = blocks[lo:hi]
                if obj.normals is not None:
                    blk[:, 0:12].reshape(n, 3, 4)[:, :, :3] = np.take(obj.normals.astype(np.float32), tri, axis=0)
                if obj.uvs is not None:
                    for k in range(3):
                        blk[:, k * 4 + 3] = obj.uvs[tri[:, k], 0]
                        blk[:, 12 + k] = obj.uvs[tri[:, k], 1]
                blk[:, 15] = (SMOOTH if obj.normals is not None else 0) + (TEXTURED if obj.uvs is not None else 0)
                has_block[lo:hi] = True
        else:
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
            arr = np.array([[p.x, p.y, p.z] for p in pts], dtype=np.float64)
            mn = arr.min(axis=0, keepdims=True)
            mx = arr.max(axis=0, keepdims=True)
        mins_all[lo:hi], maxs_all[lo:hi] = _pad_bounds(mn, mx)

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

    # The float words of every material in one array (rounded to f32 as
    # they are stored), then the u32 words over them: type, and the colour,
    # normal-map and emission textures, numbered in the order met.
    values, words = [], []
    for m in material_list:
        ck = m.checker
        c4 = (ck.x, ck.y, ck.z, m.checkerSize) if ck is not None else (0.0, 0.0, 0.0, 0.0)
        values.append((m.color.x, m.color.y, m.color.z, 0.0, m.emission.x, m.emission.y, m.emission.z, m.roughness,
                       *c4, m.ior, 0.0, m.textureScale.x, m.textureScale.y, 0.0, m.normalScale, 0.0, m.dispersion,
                       m.density, m.anisotropy))
        words.append((MATERIAL_TYPES[m.type], texture_of(m.texture, tex_index, tex_list),
                      texture_of(m.normalMap, nrm_index, nrm_list), texture_of(m.emissionTexture, tex_index, tex_list)))
    if material_list:
        k = len(material_list)
        mats[:k, :22] = np.array(values, dtype=np.float64)
        mu[:k, [3, 13, 16, 18]] = np.array(words, dtype=np.uint32)

    objs = list(map(objects.__getitem__, owners[source].tolist())) if count else []
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
