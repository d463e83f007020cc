"""Learned sample allocator: the MLP of ``csrc/mlp.cu`` behind ``gbpt_mlp_*``.

A 24 -> 64 -> 64 -> 1 GELU network with BF16 weights and FP32 accumulation,
trained and evaluated by hand-written tcgen05 kernels.  The reference has no
counterpart (CudaPT links FANN but never calls it).
"""
import ctypes

import numpy as np

from ._native import check, load, ptr

N_FEATURES = 24


class MLP:
    def __init__(self, seed=0, params=None):
        L = load()
        h = ctypes.c_void_p()
        check(L.gbpt_mlp_create(int(seed), ctypes.addressof(h)))
        self._h = h
        self.n_params = int(L.gbpt_mlp_param_count())
        if params is not None:
            self.params = params

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().gbpt_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        w = np.zeros(self.n_params, np.float32)
        check(load().gbpt_mlp_get_params(self._h, ptr(w)))
        return w

    @params.setter
    def params(self, w):
        w = np.ascontiguousarray(w, np.float32)
        if w.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        check(load().gbpt_mlp_set_params(self._h, ptr(w)))

    @staticmethod
    def _x(x):
        x = np.ascontiguousarray(x, np.float32)
        if x.ndim != 2 or x.shape[1] != N_FEATURES:
            raise ValueError(f"features must be (n, {N_FEATURES})")
        return x

    def forward(self, x):
        x = self._x(x)
        y = np.zeros(len(x), np.float32)
        check(load().gbpt_mlp_forward(self._h, ptr(x), len(x), ptr(y), 0))
        return y

    def gradients(self, x, t):
        x = self._x(x)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        check(load().gbpt_mlp_gradients(self._h, ptr(x), ptr(t), len(x), 0, ptr(g), ctypes.addressof(loss)))
        return g, loss.value

    def train_step(self, x, t, lr=1e-3):
        x = self._x(x)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_float()
        check(load().gbpt_mlp_train_step(self._h, ptr(x), ptr(t), len(x), ctypes.c_float(lr), 0,
                                         ctypes.addressof(loss)))
        return loss.value
