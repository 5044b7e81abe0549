"""The warm-start network over the C ABI (nsdg_net_*): 3x3 convolutions on
the cell grid, BF16 tensor-core kernels with FP32 accumulation, trained with
Adam on the GPU."""
from __future__ import annotations

import ctypes
from ctypes import byref, c_float, c_int, c_size_t, c_void_p

import numpy as np

from . import _lib
from ._lib import NsdgError


class Net:
    def __init__(self, channels, height, width, max_batch=1, used_outputs=None, seed=0):
        self._l = _lib.load()
        self.channels = list(channels)
        self.L = len(channels) - 1
        self.H, self.W, self.max_batch = height, width, max_batch
        self.used = used_outputs or channels[-1]
        ch = (c_int * len(channels))(*channels)
        h = c_void_p()
        st = self._l.nsdg_net_create(self.L, ch, height, width, max_batch, self.used, seed, byref(h))
        if st != _lib.NSDG_OK:
            raise NsdgError(st, f"nsdg_net_create: {self._l.nsdg_status_string(st).decode()}")
        self._h = h
        n = c_size_t()
        self._check(self._l.nsdg_net_param_count(self._h, byref(n)))
        self.n_params = n.value

    def _check(self, st):
        if st != _lib.NSDG_OK:
            raise NsdgError(st, self._l.nsdg_net_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._l.nsdg_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameters: per layer W[co][3*dy+dx][ci] then b[co]
    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        self._check(self._l.nsdg_net_get_params(self._h, out.ctypes.data_as(c_void_p), self.n_params))
        return out

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self._l.nsdg_net_set_params(self._h, a.ctypes.data_as(c_void_p), self.n_params))

    def get_grads(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        self._check(self._l.nsdg_net_get_grads(self._h, out.ctypes.data_as(c_void_p), self.n_params))
        return out

    def unpack(self, flat):
        """flat parameter vector -> lists of W [3,3,ci,co] and b [co] (oracle layout)."""
        Ws, bs, off = [], [], 0
        for l in range(self.L):
            ci, co = self.channels[l], self.channels[l + 1]
            w = np.asarray(flat[off:off + co * 9 * ci], dtype=np.float64).reshape(co, 3, 3, ci)
            Ws.append(np.transpose(w, (1, 2, 3, 0)).copy())
            off += co * 9 * ci
            bs.append(np.asarray(flat[off:off + co], dtype=np.float64))
            off += co
        return Ws, bs

    def set_batch(self, x, target=None, mask=None):
        x = np.ascontiguousarray(x, dtype=np.float32)
        B = x.shape[0]
        t = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        self._check(self._l.nsdg_net_set_batch(
            self._h, B, x.ctypes.data_as(c_void_p), None if t is None else t.ctypes.data_as(c_void_p),
            None if m is None else m.ctypes.data_as(c_void_p)))
        self._B = B

    def forward(self):
        out = np.empty((self._B, self.H, self.W, self.channels[-1]), dtype=np.float32)
        self._check(self._l.nsdg_net_forward(self._h, self._B, out.ctypes.data_as(c_void_p)))
        return out

    def loss_backward(self) -> float:
        loss = c_float()
        self._check(self._l.nsdg_net_loss_backward(self._h, self._B, byref(loss)))
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self._check(self._l.nsdg_net_adam_step(self._h, lr, beta1, beta2, eps))
