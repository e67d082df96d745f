"""ctypes binding of the learned correction's network (include/pstep_mlp.h).

Training, gradients and inference run in libpstep.so's tcgen05 kernels; this
module only marshals arguments. There is no CPU path: without the library or a
Blackwell-class CUDA device the constructor raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

N_IN, N_HID, N_OUT, NPARAM = 10, 64, 4, 6288

EXPORTS = ["pmlp_create", "pmlp_destroy", "pmlp_set_stream", "pmlp_get_params", "pmlp_set_params", "pmlp_set_data",
           "pmlp_train", "pmlp_gradient", "pmlp_forward", "pmlp_steps", "pmlp_launch_count", "pmlp_last_error"]

_VP = C.c_void_p
_F = C.POINTER(C.c_float)


def lib():
    L = _lib.load_pstep()
    if getattr(L, "_mlp_typed", False):
        return L
    L.pmlp_create.argtypes = [C.c_uint64, C.POINTER(_VP)]
    L.pmlp_destroy.argtypes = [_VP]
    L.pmlp_set_stream.argtypes = [_VP, _VP]
    L.pmlp_get_params.argtypes = [_VP, _F]
    L.pmlp_set_params.argtypes = [_VP, _F]
    L.pmlp_set_data.argtypes = [_VP, _VP, _VP, C.c_int64, C.c_int]
    L.pmlp_train.argtypes = [_VP, C.c_int64, C.c_int, C.c_float, C.c_uint64, _F]
    L.pmlp_gradient.argtypes = [_VP, C.c_int, _F, _F]
    L.pmlp_forward.argtypes = [_VP, _VP, C.c_int64, _VP, C.c_int]
    L.pmlp_steps.argtypes = [_VP]
    L.pmlp_steps.restype = C.c_int64
    L.pmlp_launch_count.argtypes = [_VP]
    L.pmlp_launch_count.restype = C.c_int64
    L.pmlp_last_error.argtypes = [_VP]
    L.pmlp_last_error.restype = C.c_char_p
    L._mlp_typed = True
    return L


class MlpError(RuntimeError):
    pass


def _f32(a, shape_tail):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if a.ndim != 2 or a.shape[1] != shape_tail:
        raise ValueError(f"expected an array of shape (n, {shape_tail})")
    return a


class Mlp:
    """The 10 -> 64 SiLU -> 64 SiLU -> 4 network on the current CUDA device."""

    def __init__(self, seed: int = 0):
        self.L = lib()
        self.h = _VP()
        rc = self.L.pmlp_create(C.c_uint64(seed), C.byref(self.h))
        if rc != 0:
            raise MlpError(f"pmlp_create failed with status {rc} (needs a Blackwell-class GPU)")

    def _check(self, rc):
        if rc != 0:
            raise MlpError(f"status {rc}: {self.L.pmlp_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.L.pmlp_destroy(self.h)
            self.h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        out = np.empty(NPARAM, dtype=np.float32)
        self._check(self.L.pmlp_get_params(self.h, out.ctypes.data_as(_F)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
        if p.shape != (NPARAM,):
            raise ValueError(f"expected {NPARAM} parameters")
        self._check(self.L.pmlp_set_params(self.h, p.ctypes.data_as(_F)))

    def set_data(self, x, y):
        x = _f32(x, N_IN)
        y = _f32(y, N_OUT)
        if x.shape[0] != y.shape[0]:
            raise ValueError("x and y differ in length")
        self._keep = (x, y)
        self._check(self.L.pmlp_set_data(self.h, x.ctypes.data, y.ctypes.data, x.shape[0], 0))

    def train(self, steps: int, batch: int = 8192, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        loss = np.empty(max(int(steps), 1), dtype=np.float32)
        self._check(self.L.pmlp_train(self.h, int(steps), int(batch), C.c_float(lr), C.c_uint64(seed),
                                      loss.ctypes.data_as(_F)))
        return loss[:steps]

    def gradient(self, batch: int):
        g = np.empty(NPARAM, dtype=np.float32)
        l = C.c_float()
        self._check(self.L.pmlp_gradient(self.h, int(batch), g.ctypes.data_as(_F), C.byref(l)))
        return g, float(l.value)

    def forward(self, x) -> np.ndarray:
        x = _f32(x, N_IN)
        y = np.empty((x.shape[0], N_OUT), dtype=np.float32)
        self._check(self.L.pmlp_forward(self.h, x.ctypes.data, x.shape[0], y.ctypes.data, 0))
        return y

    @property
    def steps(self) -> int:
        return int(self.L.pmlp_steps(self.h))

    @property
    def launches(self) -> int:
        return int(self.L.pmlp_launch_count(self.h))
