"""The fast preview while the camera moves, as the reference's page drives a
renderer (main.mjs:25-33, 145-212): while the camera moves, at most 3
bounces, one sample a frame, always denoised, and a resolution scaled (0.15
to 1 of the full one each way, starting at 0.5) so that a frame takes about
33 ms; 250 ms after the last move, full quality again.

It is caller-side policy: it only sets the renderer's properties and its
canvas size, so it works the same for a Renderer rendered alone or in a
BatchRenderer's frame (each size change means new buffers, so small changes
are left, as there)."""

from __future__ import annotations

import math
import time

FRAME_MS = 33.0
BOUNCES = 3
SCALE_MIN, SCALE_MAX = 0.15, 1.0
SETTLE_MS = 250.0


class Preview:
    """Drives one renderer: call moved() whenever the camera changes and
    frame(ms) after each frame with the time it took."""

    def __init__(self, renderer, width: int, height: int, bounces: int = 8, samples_per_frame: int = 1,
                 denoise: bool = True, clock=time.monotonic):
        self.renderer = renderer
        self.full = (int(width), int(height))
        self.bounces = int(bounces)
        self.samples_per_frame = int(samples_per_frame)
        self.denoise = bool(denoise)
        self.scale = 0.5  # main.mjs:70
        self.moving = False
        self._clock = clock
        self._settle_at = 0.0
        self.apply()

    def _now_ms(self) -> float:
        return self._clock() * 1e3

    def moved(self) -> None:
        """The camera moved: preview until it has been still for SETTLE_MS (main.mjs:172-186)."""
        self._settle_at = self._now_ms() + SETTLE_MS
        if not self.moving:
            self.moving = True
            self.apply()

    def frame(self, ms: float) -> None:
        """After a frame that took `ms`: back to full quality once settled, else
        nudge the preview's scale towards FRAME_MS — time goes with the pixel
        count, so with the square of the scale; changes under 10% are left
        (main.mjs:189-201)."""
        if self.moving and self._now_ms() >= self._settle_at:
            self.moving = False
            self.apply()
            return
        if not self.moving:
            return
        factor = min(max(math.sqrt(FRAME_MS / max(ms, 1.0)), 0.7), 1.3)
        scale = min(max(self.scale * factor, SCALE_MIN), SCALE_MAX)
        if abs(scale / self.scale - 1.0) > 0.1:
            self.scale = scale
            self._resize()

    def size(self) -> tuple[int, int]:
        """The canvas size for the current quality (main.mjs:145-151)."""
        ratio = self.scale if self.moving else 1.0
        return max(1, round(self.full[0] * ratio)), max(1, round(self.full[1] * ratio))

    def apply(self) -> None:
        """The renderer's settings that the preview cheapens (main.mjs:205-211)."""
        r = self.renderer
        r.maxBounces = min(self.bounces, BOUNCES) if self.moving else self.bounces
        r.samplesPerFrame = 1 if self.moving else self.samples_per_frame
        r.denoise = self.moving or self.denoise
        self._resize()

    def _resize(self) -> None:
        w, h = self.size()
        canvas = self.renderer.canvas
        if (canvas.width, canvas.height) != (w, h):
            canvas.width, canvas.height = w, h
