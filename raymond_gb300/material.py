"""Materials (src/Material.mjs): the same fields, clamps, type codes and
constructors as the JavaScript library."""

from __future__ import annotations


from .vec import Vec2, Vec3

MATERIAL_TYPES = {"diffuse": 0, "metal": 1, "plastic": 2, "glass": 3, "light": 4, "volume": 5}

# Wavelengths (µm) of the Abbe number's lines: helium d, hydrogen F and C.
LAMBDA_D = 0.5876
LAMBDA_F = 0.4861
LAMBDA_C = 0.6563


class Material:
    def __init__(self, type="diffuse", color=None, roughness=0.0, ior=1.5, emission=None, checker=None,
                 checkerSize=1.0, texture=None, textureScale=None, normalMap=None, normalScale=1.0,
                 emissionTexture=None, abbe=0.0, density=1.0, anisotropy=0.0):
        if type not in MATERIAL_TYPES:
            raise ValueError(f'Unknown material type "{type}".')
        self.type = type
        self.color = color if color is not None else Vec3(0.8, 0.8, 0.8)
        self.roughness = min(max(float(roughness), 0.0), 1.0)
        self.ior = max(float(ior), 1.0)
        self.emission = emission if emission is not None else Vec3(0.0, 0.0, 0.0)
        self.checker = checker
        self.checkerSize = float(checkerSize)
        self.texture = texture
        self.textureScale = textureScale if textureScale is not None else Vec2(1.0, 1.0)
        self.normalMap = normalMap
        self.normalScale = float(normalScale)
        self.emissionTexture = emissionTexture
        self.abbe = max(float(abbe), 0.0)
        self.density = max(float(density), 0.0)
        self.anisotropy = min(max(float(anisotropy), -0.99), 0.99)

    @property
    def dispersion(self) -> float:
        """Cauchy's B from the Abbe number (src/Material.mjs:196-200)."""
        if self.type != "glass" or self.abbe <= 0.0:
            return 0.0
        return (self.ior - 1.0) / (self.abbe * (LAMBDA_F ** -2 - LAMBDA_C ** -2))

    def iorAt(self, wavelength: float) -> float:
        l = wavelength / 1000.0
        return self.ior + self.dispersion * (l ** -2 - LAMBDA_D ** -2)

    @property
    def emissive(self) -> bool:
        return self.type == "light" and self.glows

    @property
    def glows(self) -> bool:
        return self.emission.x + self.emission.y + self.emission.z > 0.0

    def _with(self, **changes):
        fields = dict(type=self.type, color=self.color, roughness=self.roughness, ior=self.ior,
                      emission=self.emission, checker=self.checker, checkerSize=self.checkerSize,
                      texture=self.texture, textureScale=self.textureScale, normalMap=self.normalMap,
                      normalScale=self.normalScale, emissionTexture=self.emissionTexture, abbe=self.abbe,
                      density=self.density, anisotropy=self.anisotropy)
        fields.update(changes)
        return Material(**fields)

    def withTexture(self, texture, scale=1.0, color=None):
        ts = Vec2(scale, scale) if isinstance(scale, (int, float)) else scale
        return self._with(color=color if color is not None else Vec3(1.0, 1.0, 1.0), checker=None,
                          texture=texture, textureScale=ts)

    def withNormalMap(self, normalMap, strength=1.0):
        return self._with(normalMap=normalMap, normalScale=strength)

    def withEmission(self, color, strength=1.0, texture=None):
        return self._with(emission=color.scale(strength), emissionTexture=texture)

    @staticmethod
    def diffuse(color):
        return Material(type="diffuse", color=color)

    @staticmethod
    def metal(color, roughness=0.0):
        return Material(type="metal", color=color, roughness=roughness)

    @staticmethod
    def plastic(color, roughness=0.2):
        return Material(type="plastic", color=color, roughness=roughness)

    @staticmethod
    def glass(ior=1.5, tint=None, abbe=0.0):
        return Material(type="glass", color=tint if tint is not None else Vec3(1.0, 1.0, 1.0), ior=ior, abbe=abbe)

    @staticmethod
    def volume(color, density, anisotropy=0.0):
        return Material(type="volume", color=color, density=density, anisotropy=anisotropy)

    @staticmethod
    def light(color, strength=1.0):
        return Material(type="light", emission=color.scale(strength))

    @staticmethod
    def checkered(color, other, size=1.0):
        return Material(type="diffuse", color=color, checker=other, checkerSize=size)

