"""numpy front end of libpstep_gen.so (seeded synthetic fields and particles)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


def _gen():
    lib = _lib.load_gen()
    if not getattr(lib, "_typed", False):
        lib.pstep_gen_velocity.argtypes = [C.c_int, C.c_uint64, _D, _D, _D]
        lib.pstep_gen_temperature.argtypes = [C.c_int, C.c_uint64, C.c_double, _D]
        lib.pstep_gen_positions.argtypes = [C.c_int, C.c_double, C.c_uint64, C.c_int64, C.c_int, C.c_int,
                                            C.c_double, _D, _D, _D]
        lib.pstep_gen_interp_velocity.argtypes = [C.c_int, C.c_double, C.c_int64, _D, _D, _D, _D, _D, _D, _D, _D, _D]
        lib.pstep_gen_ghost.argtypes = [C.c_int, _D, _D]
        lib.pstep_gen_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, C.c_double, C.c_double, _D]
        lib.pstep_gen_loguniform.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, C.c_double, C.c_double, _D]
        lib.pstep_gen_normal.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        lib.pstep_gen_normal.restype = C.c_double
        lib._typed = True
    return lib


def ptr(a: np.ndarray):
    if a.dtype == np.float64:
        return a.ctypes.data_as(_D)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_I)
    return C.c_void_p(a.ctypes.data)


def velocity(n: int, seed: int):
    """Interior face velocities (u on x-faces, v on y-faces, w on z-faces), each (n,n,n) [k,j,i]."""
    u, v, w = (np.empty((n, n, n)) for _ in range(3))
    _gen().pstep_gen_velocity(n, seed, ptr(u), ptr(v), ptr(w))
    return u, v, w


def temperature(n: int, seed: int, amp: float = 0.05):
    t = np.empty((n, n, n))
    _gen().pstep_gen_temperature(n, seed, amp, ptr(t))
    return t


def ghost(a: np.ndarray) -> np.ndarray:
    """Interior (n,n,n) -> ghosted (n+2)^3 with periodic ghost layers."""
    n = a.shape[0]
    a = np.ascontiguousarray(a)
    out = np.empty((n + 2, n + 2, n + 2))
    _gen().pstep_gen_ghost(n, ptr(a), ptr(out))
    return out


def positions(n: int, l: float, seed: int, count: int, clustered: bool, nblobs: int = 64, sigma_cells: float = 4.0):
    x, y, z = (np.empty(count) for _ in range(3))
    _gen().pstep_gen_positions(n, l, seed, count, 1 if clustered else 0, nblobs, sigma_cells, ptr(x), ptr(y), ptr(z))
    return x, y, z


def interp_velocity(n, l, x, y, z, ux, uy, uz):
    cnt = x.shape[0]
    u, v, w = (np.empty(cnt) for _ in range(3))
    _gen().pstep_gen_interp_velocity(n, l, cnt, ptr(x), ptr(y), ptr(z), ptr(np.ascontiguousarray(ux)),
                                     ptr(np.ascontiguousarray(uy)), ptr(np.ascontiguousarray(uz)),
                                     ptr(u), ptr(v), ptr(w))
    return u, v, w


def uniform(seed: int, stream: int, count: int, lo: float, hi: float) -> np.ndarray:
    out = np.empty(count)
    _gen().pstep_gen_uniform(seed, stream, count, lo, hi, ptr(out))
    return out


def loguniform(seed: int, stream: int, count: int, lo: float, hi: float) -> np.ndarray:
    out = np.empty(count)
    _gen().pstep_gen_loguniform(seed, stream, count, lo, hi, ptr(out))
    return out


def make_case(n: int, count: int, seed: int, clustered: bool, l: float = 2 * 3.141592653589793, nblobs: int = 64):
    """Fields (interior) and particles of one synthetic case: u_p = interpolated gas velocity, T_p = 1."""
    ux, uy, uz = velocity(n, seed)
    tf = temperature(n, seed + 7)
    x, y, z = positions(n, l, seed + 13, count, clustered, nblobs=nblobs)
    u, v, w = interp_velocity(n, l, x, y, z, ux, uy, uz)
    t = np.ones(count)
    flag = np.arange(count, dtype=np.int32)
    return {"ux": ux, "uy": uy, "uz": uz, "T": tf, "x": x, "y": y, "z": z, "u": u, "v": v, "w": w, "t": t,
            "flag": flag}
