"""Learned warm start for the L2-NNLS solve (no counterpart in the
reference): a U-Net on the project's CUDA kernels (msot_unet_*), trained on
pairs the plain GPU solver generates, whose prediction seeds both splitting
variables of rec_nn_with_L2_reg (image w and multiplier v, kkt_multiplier).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .model import _stream_ptr


class UNet:
    """msot_unet_create(levels, base_channels, side, max_batch, seed)."""

    def __init__(self, levels=4, base_channels=32, side=128, max_batch=16, seed=0):
        self.levels, self.base, self.side, self.max_batch = levels, base_channels, side, max_batch
        h = C.c_void_p()
        _lib.check(_lib.load().msot_unet_create(levels, base_channels, side, max_batch, seed,
                                                C.byref(h)))
        self._h = h
        n = C.c_size_t()
        _lib.check(_lib.load().msot_unet_param_count(h, C.byref(n)))
        self.n_params = n.value
        self.step_count = 0

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.load().msot_unet_destroy(self._h)
            self._h = None

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n_params, dtype=np.float32)
        _lib.check(_lib.load().msot_unet_get_params(self._h, p.ctypes.data_as(
            C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        _lib.check(_lib.load().msot_unet_set_params(self._h, p.ctypes.data_as(
            C.POINTER(C.c_float))))

    def _dev(self, x):
        t = torch.as_tensor(x)
        if not t.is_cuda:
            t = t.cuda()
        return t.to(torch.float32).reshape(-1, 1, self.side, self.side).contiguous()

    def forward(self, x, stream=None):
        x = self._dev(x)
        out = torch.empty_like(x)
        for c0 in range(0, x.shape[0], self.max_batch):
            xs = x[c0:c0 + self.max_batch]
            _lib.check(_lib.load().msot_unet_forward(self._h, C.c_void_p(xs.data_ptr()),
                                                     C.c_void_p(out[c0:].data_ptr()),
                                                     xs.shape[0], _stream_ptr(stream)))
        return out

    def gradients(self, x, target, stream=None):
        x, t = self._dev(x), self._dev(target)
        loss = C.c_double()
        g = np.empty(self.n_params, dtype=np.float32)
        _lib.check(_lib.load().msot_unet_gradients(self._h, C.c_void_p(x.data_ptr()),
                                                   C.c_void_p(t.data_ptr()), x.shape[0],
                                                   C.byref(loss),
                                                   g.ctypes.data_as(C.POINTER(C.c_float)),
                                                   _stream_ptr(stream)))
        return loss.value, g

    def train_step(self, x, target, lr=1e-3, stream=None):
        x, t = self._dev(x), self._dev(target)
        loss = C.c_double()
        _lib.check(_lib.load().msot_unet_gradients(self._h, C.c_void_p(x.data_ptr()),
                                                   C.c_void_p(t.data_ptr()), x.shape[0],
                                                   C.byref(loss), None, _stream_ptr(stream)))
        self.step_count += 1
        _lib.check(_lib.load().msot_unet_adam_step(self._h, float(lr), self.step_count,
                                                   _stream_ptr(stream)))
        return loss.value
