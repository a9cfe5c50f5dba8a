"""raymond_gb300 — a GB300 (sm_103a) backend for Raymond's GPU render path.

The public names mirror the JavaScript library's (src/index.mjs): scene
objects, materials, sky, camera, Scene with its packed buffers, BVH and
Renderer. Rendering runs in libraymond_cuda.so through its C ABI
(include/raymond.h); there is no CPU fallback.
"""

from .vec import Mat4, Vec2, Vec3
from .material import MATERIAL_TYPES, Material
from .geometry import Box, Mesh, Quad, Sphere
from .sky import Camera, Sky
from .scene import BVH, NONE, PRIMITIVE_KINDS, PackedScene, Scene
from .renderer import BatchRenderer, Canvas, Renderer
from .texture import EnvironmentMap, Texture

__all__ = [
    "BatchRenderer", "BVH", "Box", "Camera", "Canvas", "MATERIAL_TYPES", "Mat4", "Material", "Mesh", "NONE", "PRIMITIVE_KINDS",
    "PackedScene", "Quad", "Renderer", "Scene", "Sky", "Sphere", "Vec2", "Vec3", "Texture", "EnvironmentMap",
]
