"""ctypes binding of the GPU machine gas step (include/pstep_gas.h).

The kernels run in libpstep.so; this module marshals arguments. There is no
CPU path: without the library or a CUDA device the constructor raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

FIELDS = ["RU_x", "RU_y", "RU_z", "Rho", "P", "T", "U_x", "U_y", "U_z", "C", "RHS_RU_x", "RHS_RU_y", "RHS_RU_z",
          "RHS_Part_Temp", "divergence", "Rho_new"]
EXPORTS = ["pgas_create", "pgas_destroy", "pgas_set_stream", "pgas_init", "pgas_step", "pgas_stage", "pgas_end_step",
           "pgas_get_field", "pgas_p0", "pgas_last_iterations", "pgas_last_error"]

_VP = C.c_void_p


class GasConfig(C.Structure):
    _fields_ = [("n", C.c_int32), ("cooling", C.c_int32), ("iterations", C.c_int32), ("twc", C.c_int32),
                ("l", C.c_double), ("dt", C.c_double), ("mu0", C.c_double), ("k", C.c_double), ("cp", C.c_double),
                ("cv", C.c_double), ("rho0", C.c_double), ("u0", C.c_double), ("a_force", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double), ("mp", C.c_double),
                ("epsilon", C.c_double)]


def lib():
    L = _lib.load_pstep()
    if getattr(L, "_gas_typed", False):
        return L
    L.pgas_create.argtypes = [C.POINTER(GasConfig), C.POINTER(_VP)]
    L.pgas_destroy.argtypes = [_VP]
    L.pgas_set_stream.argtypes = [_VP, _VP]
    L.pgas_init.argtypes = [_VP, _VP] + [_VP] * 4 + [C.c_double, C.c_int]
    L.pgas_step.argtypes = [_VP, _VP]
    L.pgas_stage.argtypes = [_VP, _VP, C.c_int]
    L.pgas_end_step.argtypes = [_VP, _VP]
    L.pgas_get_field.argtypes = [_VP, C.c_int, _VP, C.c_int]
    L.pgas_p0.argtypes = [_VP, C.POINTER(C.c_double)]
    L.pgas_last_iterations.argtypes = [_VP]
    L.pgas_last_error.argtypes = [_VP]
    L.pgas_last_error.restype = C.c_char_p
    L._gas_typed = True
    return L


class GasError(RuntimeError):
    pass


class GasStep:
    """grid.cpp's box gas step on the GPU, driving an optional pstep.ParticleStep."""

    def __init__(self, gcfg: dict, particles=None):
        self.L = lib()
        c = GasConfig()
        for k in ("n", "cooling", "iterations", "twc"):
            setattr(c, k, int(gcfg[k]))
        for k in ("l", "dt", "mu0", "k", "cp", "cv", "rho0", "u0", "a_force", "gx", "gy", "gz", "mp", "epsilon"):
            setattr(c, k, float(gcfg[k]))
        self.n = int(gcfg["n"])
        self.p0_init = float(gcfg.get("p0", 1.0))
        self.particles = particles
        self.h = _VP()
        rc = self.L.pgas_create(C.byref(c), C.byref(self.h))
        if rc != 0:
            raise GasError(f"pgas_create failed with status {rc}")

    def _ok(self, rc):
        if rc != 0:
            raise GasError(f"status {rc}: {self.L.pgas_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.L.pgas_destroy(self.h)
            self.h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ph(self):
        return self.particles.h if self.particles is not None else None

    def init(self, ru_x, ru_y, ru_z, rho, p0=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ru_x, ru_y, ru_z, rho)]
        self._ok(self.L.pgas_init(self.h, self._ph(), *[a.ctypes.data for a in arrs],
                                  float(self.p0_init if p0 is None else p0), 0))

    def step(self, nsteps: int = 1):
        for _ in range(nsteps):
            self._ok(self.L.pgas_step(self.h, self._ph()))

    def stage(self, k: int):
        self._ok(self.L.pgas_stage(self.h, self._ph(), int(k)))

    def end_step(self):
        self._ok(self.L.pgas_end_step(self.h, self._ph()))

    def field(self, name: str) -> np.ndarray:
        g = self.n + 2
        out = np.empty((g, g, g))
        self._ok(self.L.pgas_get_field(self.h, FIELDS.index(name), out.ctypes.data, 0))
        return out

    def field_to(self, name: str, device_ptr: int):
        self._ok(self.L.pgas_get_field(self.h, FIELDS.index(name), device_ptr, 1))

    def p0(self) -> float:
        v = C.c_double()
        self._ok(self.L.pgas_p0(self.h, C.byref(v)))
        return v.value

    def iterations(self) -> int:
        return int(self.L.pgas_last_iterations(self.h))
