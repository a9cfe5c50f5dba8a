"""The sky (src/Sky.mjs) and the camera (src/Camera.mjs)."""

from __future__ import annotations

import math

from .vec import Mat4, Vec3


class Sky:
    def __init__(self, zenith=None, horizon=None, ground=None, sunDirection=None, sunColor=None, sunStrength=0.0,
                 sunSize=0.05, environment=None, environmentStrength=1.0, environmentRotation=0.0):
        self.zenith = zenith if zenith is not None else Vec3(0.25, 0.45, 0.9)
        self.horizon = horizon if horizon is not None else Vec3(0.85, 0.9, 1.0)
        self.ground = ground if ground is not None else Vec3(0.3, 0.28, 0.25)
        self.sunDirection = (sunDirection if sunDirection is not None else Vec3(0.5, 0.8, 0.3)).normalized()
        self.sunColor = sunColor if sunColor is not None else Vec3(1.0, 0.95, 0.85)
        self.sunStrength = max(float(sunStrength), 0.0)
        self.sunSize = min(max(float(sunSize), 0.001), math.pi / 4.0)
        self.environment = environment
        self.environmentStrength = max(float(environmentStrength), 0.0)
        self.environmentRotation = float(environmentRotation)

    @staticmethod
    def environment_sky(environment, strength=1.0, rotation=0.0) -> "Sky":
        return Sky(environment=environment, environmentStrength=strength, environmentRotation=rotation)

    @staticmethod
    def black() -> "Sky":
        b = Vec3(0.0, 0.0, 0.0)
        return Sky(zenith=b, horizon=b, ground=b)

    @property
    def sunRadiance(self) -> Vec3:
        """Radiance that makes the disc deliver sunStrength at normal incidence (src/Sky.mjs:132-136)."""
        solid_angle = 2.0 * math.pi * (1.0 - math.cos(self.sunSize))
        return self.sunColor.scale(self.sunStrength / solid_angle)

    def radiance(self, d: Vec3) -> Vec3:
        """What the sky shows along unit direction d (src/Sky.mjs:144-154)."""
        if self.environment is not None:
            from .texture import EnvironmentMap
            u, v = EnvironmentMap.uv(d)
            turned = EnvironmentMap.direction(u - self.environmentRotation / (2.0 * math.pi), v)
            return self.environment.sample(turned).scale(self.environmentStrength)
        t = math.sqrt(min(abs(d.y), 1.0))
        return self.horizon.lerp(self.zenith, t) if d.y >= 0.0 else self.horizon.lerp(self.ground, t)


class Camera:
    def __init__(self, position=None, target=None, up=None, fov=40.0 * math.pi / 180.0, aperture=0.0,
                 focusDistance=0.0):
        self.position = position if position is not None else Vec3(0.0, 0.0, 5.0)
        self.target = target if target is not None else Vec3(0.0, 0.0, 0.0)
        self.up = up if up is not None else Vec3(0.0, 1.0, 0.0)
        self.fov = float(fov)
        self._aperture = max(float(aperture), 0.0)
        self._focus = max(float(focusDistance), 0.0)

    @property
    def aperture(self):
        return self._aperture

    @aperture.setter
    def aperture(self, value):
        self._aperture = max(float(value), 0.0)

    @property
    def focusDistance(self):
        return self._focus

    @focusDistance.setter
    def focusDistance(self, value):
        self._focus = max(float(value), 0.0)

    @property
    def effectiveFocusDistance(self) -> float:
        return self._focus if self._focus > 0.0 else self.target.subtract(self.position).length()

    @property
    def matrix(self) -> Mat4:
        return Mat4.lookAt(self.position, self.target, self.up)

    def basis(self):
        m = self.matrix
        return {"right": Vec3(m.value(0, 0), m.value(1, 0), m.value(2, 0)),
                "up": Vec3(m.value(0, 1), m.value(1, 1), m.value(2, 1)),
                "forward": Vec3(-m.value(0, 2), -m.value(1, 2), -m.value(2, 2))}

    def ray(self, x, y, aspectRatio):
        b = self.basis()
        tan_half = math.tan(self.fov / 2.0)
        direction = b["forward"].add(b["right"].scale(x * tan_half * aspectRatio)).add(
            b["up"].scale(y * tan_half)).normalized()
        return {"origin": self.position, "direction": direction}

    def pixelRay(self, px, py, width, height):
        x = 2.0 * (px + 0.5) / width - 1.0
        y = 1.0 - 2.0 * (py + 0.5) / height
        return self.ray(x, y, width / height)
