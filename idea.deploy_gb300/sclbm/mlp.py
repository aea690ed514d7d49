"""The warm-start MLP on the device (``sclbm_mlp_*`` of include/sclbm.h).

5 inputs -> 64 -> 64 -> 64 -> 1 output, SiLU, BF16 parameters with an FP32
master copy, FP32 accumulation, Adam; training, gradients and inference run
in the library's own CUDA kernels (warp-level BF16 tensor-core MMAs).
"""
import ctypes

import numpy as np

from . import _lib


def param_count():
    n = ctypes.c_int()
    _lib.call('sclbm_mlp_param_count', ctypes.byref(n))
    return n.value


class MLP:
    def __init__(self, seed=0, device=0):
        h = ctypes.c_void_p()
        _lib.call('sclbm_mlp_create', int(device), ctypes.c_uint64(int(seed)), ctypes.byref(h))
        self.h = h
        self.n_params = param_count()

    def close(self):
        if getattr(self, 'h', None):
            _lib.load().sclbm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        w = np.empty(self.n_params, np.float32)
        _lib.call('sclbm_mlp_get_params', self.h, _lib.ptr(w))
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(np.asarray(w, np.float32))
        assert w.size == self.n_params
        _lib.call('sclbm_mlp_set_params', self.h, _lib.ptr(w))

    def set_data(self, x, t):
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, 5))
        t = np.ascontiguousarray(np.asarray(t, np.float32).ravel())
        assert x.shape[0] == t.size
        _lib.call('sclbm_mlp_set_data', self.h, int(t.size), _lib.ptr(x), _lib.ptr(t))

    def train(self, steps, batch=8192, lr=1e-3):
        """Run Adam steps; returns the loss of every step."""
        loss = np.empty(int(steps), np.float32)
        _lib.call('sclbm_mlp_train', self.h, int(steps), int(batch), ctypes.c_float(lr),
                  _lib.ptr(loss) if steps else None)
        return loss

    def gradient(self, x, t):
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, 5))
        t = np.ascontiguousarray(np.asarray(t, np.float32).ravel())
        g = np.empty(self.n_params, np.float32)
        loss = ctypes.c_float()
        _lib.call('sclbm_mlp_gradient', self.h, int(t.size), _lib.ptr(x), _lib.ptr(t), _lib.ptr(g),
                  ctypes.byref(loss))
        return g, loss.value

    def predict(self, x):
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, 5))
        y = np.empty(x.shape[0], np.float32)
        _lib.call('sclbm_mlp_predict', self.h, int(x.shape[0]), _lib.ptr(x), _lib.ptr(y))
        return y
