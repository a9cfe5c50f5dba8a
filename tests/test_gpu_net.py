"""The learned denoiser's tensor-core kernels against the CPU oracle
(oracle/net.cpp): each convolution mode on its own, then the whole network's
loss and gradients, then training on the GPU."""

import ctypes

import numpy as np
import pytest

import oracle
from raymond_gb300 import _native
from raymond_gb300.denoiser import Denoiser, make_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _bf16(rng, shape, scale=1.0):
    """Random BF16 CUDA tensor and its exact float32 values."""
    t = (torch.from_numpy(rng.standard_normal(shape).astype(np.float32)) * scale).to(torch.bfloat16)
    return t.cuda(), t.float().numpy()


def _run_conv(mode, n, h, w, src0, c0, shift0, src1, c1, cout, weight, bias=None, dy=None, out=None, out_f32=None,
              mask=None, dw=None, db=None, act=0, status=None, kernel=0):
    c = _native.Conv()
    c.kernel = kernel
    c.n, c.height, c.width, c.cin, c.cout = n, h, w, c0 + c1, cout
    c.src0, c.src0_channels, c.src0_stride, c.src0_shift = src0.data_ptr(), c0, c0, shift0
    if src1 is not None:
        c.src1, c.src1_channels, c.src1_stride = src1.data_ptr(), c1, c1
    c.weight = weight.data_ptr()
    c.bias = bias.data_ptr() if bias is not None else None
    if dy is not None:
        c.dy, c.dy_stride = dy.data_ptr(), cout
    if out is not None:
        c.out, c.out_stride = out.data_ptr(), out.shape[-1]
    if out_f32 is not None:
        c.out_f32, c.out_stride = out_f32.data_ptr(), out_f32.shape[-1]
    if mask is not None:
        c.mask, c.mask_stride = mask.data_ptr(), mask.shape[-1]
    if dw is not None:
        c.dweight, c.dbias = dw.data_ptr(), db.data_ptr()
    c.activation = act
    c.status = status.data_ptr()
    fn = [_native.lib().raymond_conv3x3_forward, _native.lib().raymond_conv3x3_backward_data,
          _native.lib().raymond_conv3x3_backward_weight][mode]
    _native.check(fn(ctypes.byref(c), None))
    torch.cuda.synchronize()
    assert int(status.item()) == 0


# (n, h, w, c0, shift0, c1, cout): odd tile tails, concatenation with upsampling, wide outputs
CASES = [
    (2, 20, 28, 16, 0, 0, 32),
    (1, 24, 40, 64, 1, 32, 32),
    (2, 16, 16, 128, 1, 128, 128),
    (1, 12, 20, 96, 0, 0, 16),
    (1, 16, 24, 128, 1, 96, 96),
    (1, 18, 9, 32, 0, 48, 64),
    (3, 7, 5, 32, 0, 0, 96),
    (2, 22, 26, 32, 1, 16, 32),
]
# forward and input-gradient kernels: 0 the library's choice, 1 pixel-row tiles, 2 halo tiles
KERNELS = [0, 1, 2]


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("case", CASES)
def test_conv_kernels_match_oracle(gpu, case, kernel):
    n, h, w, c0, shift0, c1, cout = case
    rng = np.random.default_rng(sum(case))
    cin = c0 + c1
    src0, s0 = _bf16(rng, (n, h >> shift0, w >> shift0, c0))
    src1, s1 = _bf16(rng, (n, h, w, c1)) if c1 else (None, None)
    weight, wv = _bf16(rng, (cout, 9, cin), 1.0 / np.sqrt(9 * cin))
    bias = torch.from_numpy(rng.standard_normal(cout).astype(np.float32)).cuda()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")

    # forward, BF16 out with the activation, and FP32 out without
    out = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    # every case takes halo tiles (weights that do not stay in shared memory are streamed)
    _run_conv(0, n, h, w, src0, c0, shift0, src1, c1, cout, weight, bias=bias, out=out, act=1, status=status,
              kernel=kernel)
    want = oracle.conv3x3(0, s0, wv, bias.cpu().numpy(), src1=s1, shift0=shift0, act=1)
    got = out.float().cpu().numpy()
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 8e-3 * scale
    out32 = torch.empty((n, h, w, cout), dtype=torch.float32, device="cuda")
    _run_conv(0, n, h, w, src0, c0, shift0, src1, c1, cout, weight, bias=bias, out_f32=out32, status=status,
              kernel=kernel)
    want = oracle.conv3x3(0, s0, wv, bias.cpu().numpy(), src1=s1, shift0=shift0, act=0)
    np.testing.assert_allclose(out32.cpu().numpy(), want, rtol=1e-4, atol=1e-4 * scale)

    # input gradient, with the activation slope of a mask tensor
    dy, dyv = _bf16(rng, (n, h, w, cout))
    mask, mv = _bf16(rng, (n, h, w, cin))
    dx = torch.empty((n, h, w, cin), dtype=torch.bfloat16, device="cuda")
    _run_conv(1, n, h, w, src0, c0, shift0, src1, c1, cout, weight, dy=dy, out=dx, mask=mask, status=status,
              kernel=kernel)
    want = oracle.conv3x3(1, s0, wv, src1=s1, shift0=shift0, dy=dyv, mask=mv)
    got = dx.float().cpu().numpy()
    assert np.abs(got - want).max() <= 8e-3 * np.abs(want).max()
    if kernel:
        return

    # weight and bias gradients, accumulated onto what is there
    dw = torch.full((cout, 9, cin), 0.5, dtype=torch.float32, device="cuda")
    db = torch.full((cout,), -0.25, dtype=torch.float32, device="cuda")
    _run_conv(2, n, h, w, src0, c0, shift0, src1, c1, cout, weight, dy=dy, dw=dw, db=db, status=status)
    want_w, want_b = oracle.conv3x3(2, s0, wv, src1=s1, shift0=shift0, dy=dyv)
    sw = np.abs(want_w).max()
    np.testing.assert_allclose(dw.cpu().numpy() - 0.5, want_w, rtol=0, atol=2e-4 * sw)
    np.testing.assert_allclose(db.cpu().numpy() + 0.25, want_b, rtol=0, atol=2e-4 * np.abs(want_b).max())


def test_conv_rejects_bad_shapes(gpu):
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    x = torch.zeros((1, 8, 8, 24), dtype=torch.bfloat16, device="cuda")
    wt = torch.zeros((16, 9, 24), dtype=torch.bfloat16, device="cuda")
    out = torch.zeros((1, 8, 8, 16), dtype=torch.bfloat16, device="cuda")
    b = torch.zeros(16, device="cuda")
    c = _native.Conv()
    c.n, c.height, c.width, c.cin, c.cout = 1, 8, 8, 24, 16
    c.src0, c.src0_channels, c.src0_stride = x.data_ptr(), 24, 24
    c.weight, c.bias, c.out, c.out_stride, c.status = wt.data_ptr(), b.data_ptr(), out.data_ptr(), 16, status.data_ptr()
    assert _native.lib().raymond_conv3x3_forward(ctypes.byref(c), None) == _native.EINVAL
    assert b"multiples of 16" in _native.lib().raymond_last_error(None)


def _random_params(count, layout, rng):
    p = np.zeros(count, np.float32)
    for wo, bo, cin, cout in layout:
        p[wo:wo + cout * 9 * cin] = rng.uniform(-1, 1, cout * 9 * cin) * np.sqrt(6.0 / (1.01 * 9 * cin))
        p[bo:bo + cout] = rng.uniform(-0.05, 0.05, cout)
    return p


def _scene_like(rng, n, h, w, spp):
    """Render-like buffers: smooth albedo and normals, noisy radiance around a smooth target."""
    yy, xx = np.meshgrid(np.linspace(0, 1, h), np.linspace(0, 1, w), indexing="ij")
    accum = np.zeros((n, h, w, 4), np.float32)
    albedo = np.zeros_like(accum)
    normal = np.zeros_like(accum)
    target = np.zeros_like(accum)
    for i in range(n):
        base = 0.3 + 0.25 * np.sin(6 * xx + i) * np.cos(4 * yy - i)
        for c in range(3):
            target[i, ..., c] = base * (0.6 + 0.2 * c) + 0.2 * (xx > 0.5)
            albedo[i, ..., c] = (0.4 + 0.3 * np.cos(3 * xx + c)) * spp
            noise = rng.gamma(2.0, 0.5, (h, w)) * target[i, ..., c]
            accum[i, ..., c] = noise * spp
        nv = np.stack([np.sin(xx * 3), np.cos(yy * 2), np.ones_like(xx)], -1)
        normal[i, ..., :3] = nv / np.linalg.norm(nv, axis=-1, keepdims=True) * spp
        normal[i, ..., 3] = (2.0 + yy) * spp
        lum = accum[i, ..., 0] * 0.2126 + accum[i, ..., 1] * 0.7152 + accum[i, ..., 2] * 0.0722
        accum[i, ..., 3] = lum * lum / spp * 1.3
    return accum, albedo, normal, target


def test_parameter_layout_matches_oracle(gpu):
    net = Denoiser(seed=5)
    count, layout = oracle.net_layout()
    assert net.param_count == count
    assert net.layout() == layout
    p = net.get_params()
    assert np.isfinite(p).all() and np.abs(p).max() < 1.0
    net.dispose()


@pytest.mark.parametrize("w_log,w_rel,rel_eps", [(1.0, 0.0, 0.01), (0.5, 2.0, 0.01), (0.5, 1.0, 0.5)])
def test_network_gradients_match_oracle(gpu, w_log, w_rel, rel_eps):
    rng = np.random.default_rng(21)
    net = Denoiser(seed=3)
    net.set_loss(w_log, w_rel, rel_eps)
    count, layout = oracle.net_layout()
    params = _random_params(count, layout, rng)
    # BF16-exact weights so both sides multiply the same numbers
    params = torch.from_numpy(params).to(torch.bfloat16).float().numpy()
    net.set_params(params)
    n, h, w, spp = 2, 32, 48, 4.0
    accum, albedo, normal, target = _scene_like(rng, n, h, w, spp)
    dev = {k: torch.from_numpy(v).cuda() for k, v in
           dict(accum=accum, albedo=albedo, normal=normal, target=target).items()}
    batch = make_batch(dev["accum"], dev["albedo"], dev["normal"], dev["target"], samples_all=spp)
    loss, grads = net.gradients(batch)
    want_loss, want, _ = oracle.net_loss_grad(params.astype(np.float64), accum, albedo, normal, target, spp, bf16=True,
                                              w_log=w_log, w_rel=w_rel, rel_eps=rel_eps)
    assert abs(loss - want_loss) <= 2e-3 * want_loss
    cos_all = float(np.dot(grads, want) / (np.linalg.norm(grads) * np.linalg.norm(want)))
    assert cos_all > 0.999
    for li, (wo, bo, cin, cout) in enumerate(layout):
        g = grads[wo:wo + cout * 9 * cin]
        r = want[wo:wo + cout * 9 * cin]
        if li == 18:
            # only the three predicted channels and the blend weight carry a gradient
            g = g.reshape(cout, -1)[:4].ravel()
            r = r.reshape(cout, -1)[:4].ravel()
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel < 0.05, (li, rel)
    net.dispose()


def test_training_reduces_the_loss(gpu):
    rng = np.random.default_rng(8)
    net = Denoiser(seed=9)
    n, h, w, spp = 4, 64, 64, 4.0
    accum, albedo, normal, target = _scene_like(rng, n, h, w, spp)
    dev = [torch.from_numpy(v).cuda() for v in (accum, albedo, normal, target)]
    batch = make_batch(*dev, samples_all=spp)
    first = net.train_step(batch, 1e-3, want_loss=True)
    for _ in range(300):
        net.train_step(batch, 1e-3)
    last = net.train_step(batch, 1e-3, want_loss=True)
    assert np.isfinite(first) and np.isfinite(last)
    assert last < 0.7 * first, (first, last)
    net.dispose()


@pytest.mark.parametrize("kernel", [1, 2])
@pytest.mark.parametrize("shape", [(1, 384, 385, 16, 16), (2, 100, 203, 64, 32)])
def test_conv_many_tiles_per_cta_match_oracle(gpu, kernel, shape):
    """Forward and input gradient run as persistent CTAs over pixel tiles with
    one pipeline across tile boundaries: an image of 1,152 row tiles (or
    1,200 halo tiles) gives every CTA several, including partial ones at the
    right and bottom edges."""
    rng = np.random.default_rng(77)
    n, h, w, c0, cout = shape
    src0, s0 = _bf16(rng, (n, h, w, c0))
    weight, wv = _bf16(rng, (cout, 9, c0), 1.0 / np.sqrt(9 * c0))
    bias = torch.from_numpy(rng.standard_normal(cout).astype(np.float32)).cuda()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    _run_conv(0, n, h, w, src0, c0, 0, None, 0, cout, weight, bias=bias, out=out, act=1, status=status,
              kernel=kernel)
    want = oracle.conv3x3(0, s0, wv, bias.cpu().numpy(), act=1)
    assert np.abs(out.float().cpu().numpy() - want).max() <= 8e-3 * np.abs(want).max()
    dy, dyv = _bf16(rng, (n, h, w, cout))
    dx = torch.empty((n, h, w, c0), dtype=torch.bfloat16, device="cuda")
    _run_conv(1, n, h, w, src0, c0, 0, None, 0, cout, weight, dy=dy, out=dx, status=status, kernel=kernel)
    want = oracle.conv3x3(1, s0, wv, dy=dyv)
    assert np.abs(dx.float().cpu().numpy() - want).max() <= 8e-3 * np.abs(want).max()
