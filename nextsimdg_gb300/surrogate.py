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

    def forward(self, copy: bool = True):
        """The forward pass of the batch set last; its output copied to the
        host (copy=False: left on the device, for a following loss_backward)."""
        if not copy:
            self._check(self._l.nsdg_net_forward(self._h, self._B, None))
            return None
        out = np.empty((self._B, self.H, self.W, self.channels[-1]), dtype=np.float32)
        self._check(self._l.nsdg_net_forward(self._h, self._B, out.ctypes.data_as(c_void_p)))
        return out

    def time_forward(self, reps: int = 10) -> float:
        """Milliseconds per forward pass of the batch set last (CUDA events,
        no copies)."""
        ms = c_float()
        self._check(self._l.nsdg_net_time_forward(self._h, self._B, int(reps), byref(ms)))
        return ms.value

    def loss_backward(self) -> float:
        loss = c_float()
        self._check(self._l.nsdg_net_loss_backward(self._h, self._B, byref(loss)))
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self._check(self._l.nsdg_net_adam_step(self._h, lr, beta1, beta2, eps))

    # -- warm-start dataset and training (all on the device) -------------------
    def dataset_reserve(self, capacity: int):
        self._check(self._l.nsdg_net_dataset_reserve(self._h, int(capacity)))
        self.capacity = int(capacity)

    def dataset_normalise(self, count: int):
        self._check(self._l.nsdg_net_dataset_normalise(self._h, int(count)))

    def train(self, count: int, iterations: int, batch: int = 1, lr: float = 1e-3, seed: int = 0) -> float:
        loss = c_float()
        self._check(self._l.nsdg_net_train(self._h, int(count), int(iterations), int(batch), float(lr),
                                           int(seed), byref(loss)))
        return loss.value

    def get_normalisation(self) -> np.ndarray:
        out = np.empty(_lib.NET_NORM_FLOATS, dtype=np.float32)
        self._check(self._l.nsdg_net_get_normalisation(self._h, out.ctypes.data_as(c_void_p), out.size))
        return out

    def set_normalisation(self, stats):
        a = np.ascontiguousarray(stats, dtype=np.float32)
        self._check(self._l.nsdg_net_set_normalisation(self._h, a.ctypes.data_as(c_void_p), a.size))


WARM_CHANNELS = (_lib.WARM_FEATURES, 48, 48, 48, 48, 48, _lib.WARM_TARGETS)


def warm_net(nx: int, ny: int, max_batch: int = 1, seed: int = 0, channels=WARM_CHANNELS) -> Net:
    """A network shaped for the warm start of an nx x ny grid."""
    return Net(channels, ny, nx, max_batch=max_batch, used_outputs=_lib.WARM_USED, seed=seed)


def train_warm_start(kernel, forcing, samples: int, k_iters: int, dt: float, net: Net | None = None,
                     stride: int = 1, iterations: int = 2000, batch: int = 1,
                     schedule=((0.4, 1e-3), (0.3, 3e-4), (0.3, 1e-4)), seed: int = 0, t0: float = 0.0,
                     nx: int | None = None, ny: int | None = None):
    """Runs the plain sub-cycle of `kernel` for samples * stride steps
    (forcing(kernel, step) sets each step's inputs), recording every
    stride-th step as a training sample; then normalises and trains with
    Adam over `schedule` ((fraction of the iterations, learning rate), ...).
    Returns (net, kappa, loss): kappa is the largest last-iteration ratio of
    the plain sub-cycle over the recorded steps."""
    if net is None:
        net = warm_net(nx, ny, max_batch=batch, seed=seed)
    net.dataset_reserve(samples)
    ratios = []
    step = 0
    for j in range(samples):
        for i in range(stride):
            forcing(kernel, step)
            slot = j if i == stride - 1 else -1
            r = kernel.warm_sample(t0 + step * dt, dt, k_iters, net, slot)
            if slot >= 0:
                ratios.append(r)
            step += 1
    net.dataset_normalise(samples)
    loss = float("nan")
    for i, (frac, lr) in enumerate(schedule):
        loss = net.train(samples, max(1, int(iterations * frac)), batch=batch, lr=lr, seed=seed + i)
    return net, float(max(ratios)), loss
