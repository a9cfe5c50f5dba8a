"""The fast-preview policy (raymond_gb300/preview.py, after main.mjs:25-33,
145-212) on a stand-in renderer with a fake clock: what moving sets, how the
scale follows frame times, and the return to full quality after 250 ms."""

from raymond_gb300 import Canvas
from raymond_gb300.preview import Preview


class FakeRenderer:
    def __init__(self, w, h):
        self.canvas = Canvas(w, h)
        self.maxBounces = 8
        self.samplesPerFrame = 4
        self.denoise = False


class Clock:
    def __init__(self):
        self.t = 100.0

    def __call__(self):
        return self.t


def test_still_camera_keeps_full_quality():
    r = FakeRenderer(800, 600)
    p = Preview(r, 800, 600, bounces=8, samples_per_frame=4, denoise=False, clock=Clock())
    assert (r.maxBounces, r.samplesPerFrame, r.denoise) == (8, 4, False)
    assert (r.canvas.width, r.canvas.height) == (800, 600)
    p.frame(500.0)  # slow frames do not matter while still
    assert (r.canvas.width, r.canvas.height) == (800, 600)


def test_moving_cheapens_then_settles():
    clock = Clock()
    r = FakeRenderer(800, 600)
    p = Preview(r, 800, 600, bounces=8, samples_per_frame=4, denoise=False, clock=clock)
    p.moved()
    assert (r.maxBounces, r.samplesPerFrame, r.denoise) == (3, 1, True)
    assert (r.canvas.width, r.canvas.height) == (400, 300)  # half scale to start
    # a slow frame shrinks the preview (at most by 0.7 a step)
    p.frame(132.0)
    assert abs(p.scale - 0.35) < 1e-9
    assert (r.canvas.width, r.canvas.height) == (280, 210)
    # a frame near the target leaves it (change under 10%)
    p.frame(30.0)
    assert abs(p.scale - 0.35) < 1e-9
    # fast frames grow it, up to 1.3 a step
    p.frame(5.0)
    assert abs(p.scale - 0.455) < 1e-9
    # moving again postpones the settle
    clock.t += 0.2
    p.moved()
    clock.t += 0.2
    p.frame(33.0)
    assert p.moving
    clock.t += 0.06
    p.frame(33.0)
    assert not p.moving
    assert (r.maxBounces, r.samplesPerFrame, r.denoise) == (8, 4, False)
    assert (r.canvas.width, r.canvas.height) == (800, 600)


def test_scale_bounds():
    clock = Clock()
    r = FakeRenderer(1000, 1000)
    p = Preview(r, 1000, 1000, clock=clock)
    p.moved()
    for _ in range(20):
        p.frame(10_000.0)
    assert abs(p.scale - 0.15) < 1e-9 and r.canvas.width == 150
    for _ in range(20):
        p.frame(1.0)
    # ×1.3 steps from 0.15 stop at 0.941: the last step to 1.0 is under 10%
    assert 0.9 < p.scale <= 1.0 and r.canvas.width == round(1000 * p.scale)
