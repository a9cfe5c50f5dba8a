"""The learned denoiser: a BF16 U-Net whose forward, backward and Adam
kernels are this library's own tcgen05 kernels (include/raymond.h,
raymond_net_*). It stands beside the à-trous filter and, like it, only
filters the displayed image; a renderer's running sums are its inputs.

Device memory for batches is handed over as CUDA tensors (anything with
``data_ptr()``): float32, shape [n, h, w, 4], laid out like a renderer's
accumulation buffers (sums over the samples)."""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _native

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
DEFAULT_WEIGHTS = os.path.join(WEIGHTS_DIR, "denoiser_unet.npz")
CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy: the legacy default stream's handle


def _addr(t):
    return None if t is None else int(t.data_ptr())


def make_batch(accum, albedo, normal, target=None, samples=None, samples_all=1.0):
    """A raymond_net_batch over CUDA tensors [n, h, w, 4] (float32)."""
    n, h, w = int(accum.shape[0]), int(accum.shape[1]), int(accum.shape[2])
    b = _native.NetBatch()
    b.accum, b.albedo, b.normal = _addr(accum), _addr(albedo), _addr(normal)
    b.target = _addr(target)
    b.samples = _addr(samples)
    b.samples_all = float(samples_all)
    b.n, b.width, b.height = n, w, h
    return b


class Denoiser:
    """One network on one GPU, with its FP32 master weights and Adam state."""

    def __init__(self, device: int = 0, seed: int = 1, weights: str | None = None):
        lib = _native.lib()
        cfg = _native.NetConfig()
        cfg.device, cfg.seed = device, seed
        h = ctypes.c_void_p()
        _native.check(lib.raymond_net_create(ctypes.byref(h), ctypes.byref(cfg)))
        self.handle = h.value
        self.device = device
        self.param_count = int(lib.raymond_net_param_count(self.handle))
        if weights is not None:
            self.load(weights)

    # ---- parameters
    def layout(self):
        """Per layer: (weight offset, bias offset, cin, cout)."""
        wo = np.zeros(19, np.uint64)
        bo = np.zeros(19, np.uint64)
        ci = np.zeros(19, np.uint32)
        co = np.zeros(19, np.uint32)
        self._check(_native.lib().raymond_net_layout(self.handle, _native.ptr(wo), _native.ptr(bo), _native.ptr(ci),
                                                     _native.ptr(co), 19))
        return [(int(wo[i]), int(bo[i]), int(ci[i]), int(co[i])) for i in range(19)]

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count, np.float32)
        self._check(_native.lib().raymond_net_get_params(self.handle, _native.ptr(p), self.param_count))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(_native.lib().raymond_net_set_params(self.handle, _native.ptr(p), p.size))

    def save(self, path: str) -> None:
        """Weights as BF16 bit patterns (what the kernels multiply with) and the blend guard."""
        p = self.get_params()
        bits = (p.view(np.uint32) + np.uint32(0x7FFF) + ((p.view(np.uint32) >> 16) & 1)) >> 16
        np.savez_compressed(path, bf16=bits.astype(np.uint16), count=np.int64(self.param_count),
                            tau=np.float32(self.blend))

    def load(self, path: str) -> None:
        with np.load(path) as z:
            bits = z["bf16"].astype(np.uint32) << 16
            if int(z["count"]) != self.param_count:
                raise ValueError(f"{path}: {int(z['count'])} parameters, the network has {self.param_count}")
            tau = float(z["tau"]) if "tau" in z.files else 0.1
        self.set_params(bits.view(np.float32))
        self.blend = tau

    @property
    def blend(self) -> float:
        """The display blend's guard τ (α = sigmoid(gate) · v/(v + τ²))."""
        return float(_native.lib().raymond_net_get_blend(self.handle))

    @blend.setter
    def blend(self, tau: float) -> None:
        self._check(_native.lib().raymond_net_set_blend(self.handle, float(tau)))

    # ---- training
    def set_loss(self, w_log: float = 1.0, w_rel: float = 0.0, rel_eps: float = 0.01) -> None:
        """Loss weights: w_log on |log radiance error|, w_rel on the relative
        squared error (v − t)² / (v̂² + rel_eps)."""
        self._check(_native.lib().raymond_net_set_loss(self.handle, float(w_log), float(w_rel), float(rel_eps)))

    def gradients(self, batch):
        """(loss, gradients) of one batch, without a step."""
        g = np.zeros(self.param_count, np.float32)
        loss = ctypes.c_float()
        self._check(_native.lib().raymond_net_gradients(self.handle, ctypes.byref(batch), _native.ptr(g),
                                                        self.param_count, ctypes.byref(loss)))
        return float(loss.value), g

    def train_step(self, batch, learning_rate: float, want_loss: bool = False):
        loss = ctypes.c_float()
        self._check(_native.lib().raymond_net_train_step(self.handle, ctypes.byref(batch), float(learning_rate),
                                                         ctypes.byref(loss) if want_loss else None))
        return float(loss.value) if want_loss else None

    def sync(self) -> None:
        self._check(_native.lib().raymond_net_sync(self.handle))

    # ---- inference
    def infer(self, batch, out, stream=None) -> None:
        """Denoised radiance into `out` (CUDA float32 [n, h, w, 4])."""
        self._check(_native.lib().raymond_net_infer(self.handle, ctypes.byref(batch), _addr(out), stream))

    @property
    def stream(self):
        return _native.lib().raymond_net_get_stream(self.handle)

    def use_stream(self, stream) -> None:
        """Enqueue on this cudaStream_t (an int handle, e.g. a torch stream's
        cuda_stream), ordered with the caller's work on the batch tensors.
        0 is the legacy default stream (torch's default), passed on as
        cudaStreamLegacy; None returns to the network's own stream."""
        if stream == 0:
            stream = CUDA_STREAM_LEGACY
        self._check(_native.lib().raymond_net_set_stream(self.handle, stream))

    def dispose(self) -> None:
        if self.handle:
            _native.lib().raymond_net_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.dispose()
        except Exception:
            pass

    def _check(self, rc):
        _native.check_net(rc, self.handle)
