"""The learned denoiser's CPU oracle (oracle/net.cpp) checked on its own:
its direct convolutions against PyTorch's CPU conv2d in float64, and its
reverse-mode network gradients against FP64 central finite differences.
These pin the oracle that the GPU kernels' tests then compare against."""

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
F = torch.nn.functional


def _torch_conv(src0, weight, bias, src1=None, shift0=0, act=0):
    x0 = torch.from_numpy(src0.astype(np.float64)).permute(0, 3, 1, 2)
    if shift0:
        x0 = x0.repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)
    x = x0 if src1 is None else torch.cat([x0, torch.from_numpy(src1.astype(np.float64)).permute(0, 3, 1, 2)], 1)
    cout, _, cin = weight.shape
    w = torch.from_numpy(weight.astype(np.float64)).reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = F.conv2d(x, w, torch.from_numpy(bias.astype(np.float64)), padding=1)
    if act:
        y = torch.where(y > 0, y, 0.1 * y)
    return x, w, y


@pytest.mark.parametrize("shift0,c0,c1,cout", [(0, 16, 0, 32), (1, 32, 16, 16)])
def test_oracle_conv_matches_torch(shift0, c0, c1, cout):
    rng = np.random.default_rng(3)
    n, h, w = 2, 8, 10
    src0 = rng.standard_normal((n, h >> shift0, w >> shift0, c0)).astype(np.float32)
    src1 = rng.standard_normal((n, h, w, c1)).astype(np.float32) if c1 else None
    weight = (0.1 * rng.standard_normal((cout, 9, c0 + c1))).astype(np.float32)
    bias = rng.standard_normal(cout).astype(np.float32)
    x, wt, y = _torch_conv(src0, weight, bias, src1, shift0, act=1)
    got = oracle.conv3x3(0, src0, weight, bias, src1=src1, shift0=shift0, act=1)
    np.testing.assert_allclose(got, y.permute(0, 2, 3, 1).numpy(), rtol=1e-5, atol=1e-5)

    # gradients of sum(y * dy) with respect to the concatenated input and the weights
    dy = rng.standard_normal((n, h, w, cout)).astype(np.float32)
    x = x.detach().requires_grad_(True)
    wt = wt.detach().requires_grad_(True)
    b = torch.from_numpy(bias.astype(np.float64)).requires_grad_(True)
    pre = F.conv2d(x, wt, b, padding=1)
    (pre * torch.from_numpy(dy.astype(np.float64)).permute(0, 3, 1, 2)).sum().backward()
    dx = oracle.conv3x3(1, src0, weight, src1=src1, shift0=shift0, dy=dy)
    np.testing.assert_allclose(dx, x.grad.permute(0, 2, 3, 1).numpy(), rtol=1e-5, atol=1e-5)
    dw, db = oracle.conv3x3(2, src0, weight, src1=src1, shift0=shift0, dy=dy)
    want_dw = wt.grad.permute(0, 2, 3, 1).reshape(cout, 9, c0 + c1).numpy()
    np.testing.assert_allclose(dw, want_dw, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(db, b.grad.numpy(), rtol=1e-9, atol=1e-9)


def _inputs(rng, n, h, w, spp=4.0, level=0.4):
    accum = np.zeros((n, h, w, 4), np.float32)
    accum[..., :3] = rng.gamma(2.0, level, (n, h, w, 3)) * spp
    lum = accum[..., 0] * 0.2126 + accum[..., 1] * 0.7152 + accum[..., 2] * 0.0722
    accum[..., 3] = lum * lum / spp * 1.5
    albedo = np.zeros_like(accum)
    albedo[..., :3] = rng.uniform(0.05 if level > 0.2 else 0.4, 0.9, (n, h, w, 3)) * spp
    normal = np.zeros_like(accum)
    v = rng.standard_normal((n, h, w, 3))
    normal[..., :3] = v / np.linalg.norm(v, axis=-1, keepdims=True) * spp
    normal[..., 3] = rng.uniform(1.0, 5.0, (n, h, w)) * spp
    target = np.zeros_like(accum)
    target[..., :3] = rng.gamma(2.0, level, (n, h, w, 3))
    return accum, albedo, normal, target


# The relative term holds its denominator constant (it is not differentiated),
# so its finite-difference check uses an ε large enough that the denominator
# barely moves; the GPU test checks the production ε against the oracle.
@pytest.mark.parametrize("w_log,w_rel,rel_eps", [(1.0, 0.0, 0.01), (0.5, 4e6, 1e6)])
def test_oracle_network_gradients_match_finite_differences(w_log, w_rel, rel_eps):
    count, layout = oracle.net_layout()
    rng = np.random.default_rng(11)
    params = np.zeros(count, np.float64)
    for wo, bo, cin, cout in layout:
        params[wo:wo + cout * 9 * cin] = rng.uniform(-1, 1, cout * 9 * cin) * np.sqrt(6.0 / (1.01 * 9 * cin))
        params[bo:bo + cout] = rng.uniform(-0.05, 0.05, cout)
    # radiance low enough that no gradient element reaches the clip
    accum, albedo, normal, target = _inputs(rng, 1, 16, 16, level=0.4 if w_rel == 0 else 0.1)
    loss, grads, _ = oracle.net_loss_grad(params, accum, albedo, normal, target, 4.0, w_log=w_log, w_rel=w_rel,
                                          rel_eps=rel_eps)
    assert np.isfinite(loss) and loss > 0
    # weights and biases of the first, a middle, a skip-concatenating and the last layer
    picks = []
    for li in (0, 8, 10, 16, 18):
        wo, bo, cin, cout = layout[li]
        picks += list(rng.integers(wo, wo + cout * 9 * cin, 3)) + [bo + int(rng.integers(0, min(cout, 3)))]
    eps = 1e-6
    for i in picks:
        p1 = params.copy()
        p1[i] += eps
        p2 = params.copy()
        p2[i] -= eps
        lp = oracle.net_loss_grad(p1, accum, albedo, normal, target, 4.0, grads=False, w_log=w_log, w_rel=w_rel,
                                  rel_eps=rel_eps)[0]
        lm = oracle.net_loss_grad(p2, accum, albedo, normal, target, 4.0, grads=False, w_log=w_log, w_rel=w_rel,
                                  rel_eps=rel_eps)[0]
        fd = (lp - lm) / (2 * eps)
        # absolute slack: one pixel whose L1 term changes sign within ±eps moves the
        # central difference by about 3e-9 here
        assert abs(fd - grads[i]) <= 1e-3 * max(abs(fd), abs(grads[i])) + 5e-9, (i, fd, grads[i])
