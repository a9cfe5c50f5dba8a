"""Textures (src/Texture.mjs) and environment maps (src/EnvironmentMap.mjs):
8-bit RGBA images sampled bilinearly with repeat, and equirectangular HDR
skies with the importance table light sampling searches. numpy-vectorized;
the arithmetic follows the reference's."""

from __future__ import annotations

import math

import numpy as np

from .vec import Vec3

_SRGB_TO_LINEAR = np.array([(i / 255) / 12.92 if i / 255 <= 0.04045 else ((i / 255 + 0.055) / 1.055) ** 2.4
                            for i in range(256)], dtype=np.float64)


_PLAIN = np.arange(256) / 255.0  # a byte as a plain number in [0, 1]


def _js_round(x):
    return np.floor(np.asarray(x, dtype=np.float64) + 0.5)


def to_srgb_byte(c):
    """Linear value to an sRGB-encoded byte (src/Texture.mjs toSrgbByte)."""
    x = np.minimum(np.maximum(np.asarray(c, dtype=np.float64), 0.0), 1.0)
    s = np.where(x <= 0.0031308, x * 12.92, 1.055 * np.power(x, 1 / 2.4) - 0.055)
    return _js_round(s * 255).astype(np.uint8)


class Texture:
    def __init__(self, width: int, height: int, data):
        if not (isinstance(width, int) and isinstance(height, int) and width > 0 and height > 0):
            raise ValueError("A texture needs a whole number of pixels each way.")
        data = np.asarray(data, dtype=np.uint8).reshape(-1)
        if data.size != width * height * 4:
            raise ValueError(f"A {width} × {height} texture needs {width * height * 4} bytes.")
        self.width, self.height, self.data = width, height, data.copy()

    @staticmethod
    def procedural(width, height, color) -> "Texture":
        """Texels from color(u, v) at texel centres, sRGB-encoded."""
        data = np.zeros((height, width, 4), dtype=np.uint8)
        for y in range(height):
            for x in range(width):
                c = color((x + 0.5) / width, (y + 0.5) / height)
                data[y, x, :3] = to_srgb_byte([c.x, c.y, c.z])
        data[..., 3] = 255
        return Texture(width, height, data)

    @staticmethod
    def normalMap(width, height, heightAt) -> "Texture":
        """A tangent-space normal map from a height function (src/Texture.mjs normalMap)."""
        h = np.zeros((height, width))
        for y in range(height):
            for x in range(width):
                h[y, x] = heightAt((x + 0.5) / width, (y + 0.5) / height)
        right = (np.roll(h, -1, axis=1) - np.roll(h, 1, axis=1)) * width / 2.0
        down = (np.roll(h, -1, axis=0) - np.roll(h, 1, axis=0)) * width / 2.0
        length = np.sqrt(right * right + down * down + 1.0)
        data = np.zeros((height, width, 4), dtype=np.uint8)
        data[..., 0] = _js_round((-right / length * 0.5 + 0.5) * 255)
        data[..., 1] = _js_round((down / length * 0.5 + 0.5) * 255)
        data[..., 2] = _js_round((1.0 / length * 0.5 + 0.5) * 255)
        data[..., 3] = 255
        return Texture(width, height, data)

    def sample_many(self, u, v, srgb=True) -> np.ndarray:
        """Bilinear, repeating; decodes sRGB bytes first (src/Texture.mjs sample): (n, 3)."""
        u = np.asarray(u, dtype=np.float64)
        v = np.asarray(v, dtype=np.float64)
        x = u * self.width - 0.5
        y = v * self.height - 0.5
        x0, y0 = np.floor(x), np.floor(y)
        fx, fy = x - x0, y - y0
        img = self.data.reshape(self.height, self.width, 4)[..., :3]
        # Decoded after the gather: only the texels the samples touch.
        table = _SRGB_TO_LINEAR if srgb else _PLAIN
        out = np.zeros(u.shape + (3,))
        for dx, dy, w in ((0, 0, (1 - fx) * (1 - fy)), (1, 0, fx * (1 - fy)), (0, 1, (1 - fx) * fy), (1, 1, fx * fy)):
            px = np.mod(x0 + dx, self.width).astype(np.int64)
            py = np.mod(y0 + dy, self.height).astype(np.int64)
            out += w[..., None] * table[img[py, px]]
        return out

    def _sample_grid(self, us, vs, srgb) -> np.ndarray:
        """sample_many over the grid of columns us × rows vs: (rows, columns,
        3). Each column's x and each row's y are worked out once and the
        texels gathered a row and a column at a time; every value is the
        same as sample_many's (the weights are the same two factors)."""
        x = us * self.width - 0.5
        y = vs * self.height - 0.5
        x0, y0 = np.floor(x), np.floor(y)
        fx, fy = x - x0, y - y0
        img = self.data.reshape(self.height, self.width, 4)[..., :3]
        table = _SRGB_TO_LINEAR if srgb else _PLAIN
        out = np.zeros((len(vs), len(us), 3))
        for dx, dy in ((0, 0), (1, 0), (0, 1), (1, 1)):
            wx = fx if dx else 1 - fx
            wy = fy if dy else 1 - fy
            px = np.mod(x0 + dx, self.width).astype(np.int64)
            py = np.mod(y0 + dy, self.height).astype(np.int64)
            out += (wy[:, None] * wx[None, :])[..., None] * table[img[py][:, px]]
        return out

    def sample(self, u, v, srgb=True) -> Vec3:
        c = self.sample_many(np.array([u]), np.array([v]), srgb)[0]
        return Vec3(*c)

    def resized(self, width, height, srgb=True) -> "Texture":
        """Resampled to width × height at texel centres (src/Texture.mjs resized)."""
        if width == self.width and height == self.height:
            return self
        c = self._sample_grid((np.arange(width) + 0.5) / width, (np.arange(height) + 0.5) / height, srgb)
        data = np.zeros((height, width, 4), dtype=np.uint8)
        if srgb:
            data[..., :3] = to_srgb_byte(c)
        else:
            data[..., :3] = _js_round(c * 255).astype(np.uint8)
        data[..., 3] = 255
        return Texture(width, height, data)


class EnvironmentMap:
    """An equirectangular HDR sky (src/EnvironmentMap.mjs)."""

    def __init__(self, width: int, height: int, data):
        if not (isinstance(width, int) and isinstance(height, int) and width > 0 and height > 0):
            raise ValueError("An environment map needs a whole number of pixels each way.")
        data = np.asarray(data, dtype=np.float32).reshape(-1)
        if data.size != width * height * 3:
            raise ValueError(f"A {width} × {height} environment map needs {width * height * 3} floats.")
        data = np.where(np.isfinite(data), np.maximum(data, 0.0), 0.0).astype(np.float32)
        self.width, self.height, self.data = width, height, data
        self._importance = None

    @staticmethod
    def direction(u, v) -> Vec3:
        phi = (u - 0.5) * 2.0 * math.pi
        theta = v * math.pi
        return Vec3(math.sin(theta) * math.sin(phi), math.cos(theta), -math.sin(theta) * math.cos(phi))

    @staticmethod
    def uv(d):
        u = 0.5 + math.atan2(d.x, -d.z) / (2.0 * math.pi)
        return u - math.floor(u), math.acos(min(max(d.y, -1.0), 1.0)) / math.pi

    @staticmethod
    def procedural(width, height, radiance) -> "EnvironmentMap":
        data = np.zeros((height, width, 3), dtype=np.float32)
        for y in range(height):
            for x in range(width):
                c = radiance(EnvironmentMap.direction((x + 0.5) / width, (y + 0.5) / height))
                data[y, x] = (c.x, c.y, c.z)
        return EnvironmentMap(width, height, data)

    def importance(self):
        """Row CDFs (cw × ch) and the CDF over rows (one more row), by
        luminance × sin θ over ≤512×256 cells (src/EnvironmentMap.mjs:202-247).

        Vectorised across each row of cells with the reference's arithmetic
        kept step for step, so the table is bit-identical: each cell's light
        summed in double over its pixels, row-major; the running sum along
        the row (a sequential cumulative sum) stored as f32, then divided by
        the row's double total and stored as f32 again; the rows' totals
        summed in order for the CDF down."""
        if self._importance is not None:
            return self._importance
        W, H = self.width, self.height
        cw = min(W, 512)
        ch = min(H, 256, cw)
        data = np.zeros(cw * (ch + 1), dtype=np.float32)
        rows = np.zeros(ch)
        img = self.data.reshape(H, W, 3).astype(np.float64)
        lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
        xs = np.arange(cw)
        x0 = (xs * W) // cw  # floor(x·W/cw): exact in integers
        x1 = np.maximum(x0 + 1, ((xs + 1) * W) // cw)
        widths = x1 - x0
        for y in range(ch):
            y0 = (y * H) // ch
            y1 = max(y0 + 1, ((y + 1) * H) // ch)
            sin = math.sin((y + 0.5) / ch * math.pi)
            light = np.zeros(cw)
            for py in range(y0, y1):
                line = lum[py]
                for k in range(int(widths.max())):
                    inside = k < widths
                    light += np.where(inside, line[np.minimum(x0 + k, W - 1)], 0.0)
            running = np.cumsum(light / ((y1 - y0) * widths) * sin)
            s = float(running[-1])
            cells = running.astype(np.float32)
            if s > 0:
                data[y * cw:(y + 1) * cw] = cells.astype(np.float64) / s
            else:
                data[y * cw:(y + 1) * cw] = (xs + 1) / cw
            rows[y] = s
        down = np.cumsum(rows)
        total = float(down[-1])
        data[ch * cw:ch * cw + ch] = down / total if total > 0 else (np.arange(ch) + 1) / ch
        data[ch * cw + ch - 1] = 1.0
        data[cw - 1:ch * cw:cw] = 1.0
        self._importance = {"width": cw, "height": ch, "data": data}
        return self._importance

    def sampleDirection(self, xi):
        """A direction by the importance table from 4 uniforms, with its pdf."""
        imp = self.importance()
        cw, ch, data = imp["width"], imp["height"], imp["data"]

        def search(offset, n, x):
            lo, hi = 0, n - 1
            while lo < hi:
                mid = (lo + hi) >> 1
                if data[offset + mid] > x:
                    hi = mid
                else:
                    lo = mid + 1
            return lo

        y = search(ch * cw, ch, xi[0])
        x = search(y * cw, cw, xi[1])
        direction = EnvironmentMap.direction((x + xi[2]) / cw, (y + xi[3]) / ch)
        return {"direction": direction, "pdf": self.pdf(direction)}

    def pdf(self, d) -> float:
        imp = self.importance()
        cw, ch, data = imp["width"], imp["height"], imp["data"]
        u, v = EnvironmentMap.uv(d)
        x, y = min(math.floor(u * cw), cw - 1), min(math.floor(v * ch), ch - 1)
        row = data[ch * cw + y] - (data[ch * cw + y - 1] if y > 0 else 0.0)
        cell = data[y * cw + x] - (data[y * cw + x - 1] if x > 0 else 0.0)
        s = math.sin(v * math.pi)
        return float(row * cell * cw * ch / (2.0 * math.pi * math.pi * s)) if s > 0 else 0.0

    def sample(self, d) -> Vec3:
        u, v = EnvironmentMap.uv(d)
        x = u * self.width - 0.5
        y = min(max(v * self.height - 0.5, 0.0), self.height - 1)
        x0, y0 = math.floor(x), math.floor(y)
        fx, fy = x - x0, y - y0
        img = self.data.reshape(self.height, self.width, 3)
        out = np.zeros(3)
        for dx, dy, w in ((0, 0, (1 - fx) * (1 - fy)), (1, 0, fx * (1 - fy)), (0, 1, (1 - fx) * fy), (1, 1, fx * fy)):
            px = ((x0 + dx) % self.width + self.width) % self.width
            py = min(y0 + dy, self.height - 1)
            out += w * img[py, px]
        return Vec3(*out)
