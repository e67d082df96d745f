"""ctypes binding of libpstep.so, mirroring the reference's `class particle`
(particle.h:12-155) and the particle part of `grid` (grid.cpp:207-226,
315-325, 659-680, 705-712).

The library runs the step on the GPU; this module only marshals arguments.
There is no CPU fallback: if libpstep.so or a CUDA device is missing, the
constructor raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .config import RK4_POST, RK4_PRE

FP64, FP32 = 0, 1
TRACK_ORDER, CHECK_INPUTS, REFERENCE_SUMS, KEEP_GAS = 1, 2, 4, 8

ARRAY_IDS = {n: i for i, n in enumerate(
    ["x", "y", "z", "u", "v", "w", "T",
     "x_int", "y_int", "z_int", "u_int", "v_int", "w_int", "T_int",
     "x_new", "y_new", "z_new", "u_new", "v_new", "w_new", "T_new",
     "x_np1", "y_np1", "z_np1", "u_np1", "v_np1", "w_np1", "T_np1",
     "RHS_T", "flag", "ug", "vg", "wg", "Tg"])}
FIELD_IDS = {"C": 0, "RHS_RU_x": 1, "RHS_RU_y": 2, "RHS_RU_z": 3, "RHS_Part_Temp": 4}

STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported configuration", 3: "capacity exceeded",
          4: "call out of sequence", 5: "CUDA error", 6: "non-finite value", 7: "position out of range",
          8: "particle moved more than one cell", 9: "device memory exhausted", 10: "device wait timed out",
          11: "snapshot file error"}


class PstepError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"pstep status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class Props(C.Structure):
    _fields_ = [("tau_p", C.c_void_p), ("mass_ratio", C.c_void_p), ("itth", C.c_void_p), ("heat_is", C.c_void_p),
                ("alpha", C.c_void_p), ("accel", C.c_void_p * 3)]


class Correction(C.Structure):
    _fields_ = [("params", C.POINTER(C.c_float)), ("shift", C.c_float * 10), ("scale", C.c_float * 10),
                ("lo", C.c_float * 4), ("hi", C.c_float * 4), ("prior_re", C.c_float), ("nu_gas", C.c_double),
                ("every_stage", C.c_int32), ("drive_cap", C.c_float)]


class Config(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("bs", C.c_int32),
                ("twc", C.c_int32), ("particle_gravity", C.c_int32), ("precision", C.c_int32),
                ("flags", C.c_int32), ("capacity", C.c_int64),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double), ("dt", C.c_double),
                ("tp", C.c_double), ("mp", C.c_double), ("dp", C.c_double), ("nu", C.c_double),
                ("k", C.c_double), ("epsilonp", C.c_double), ("i0", C.c_double), ("cvp", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double)]


_D = C.POINTER(C.c_double)
_VP = C.c_void_p
_H = C.c_void_p

EXPORTS = ["pstep_create", "pstep_destroy", "pstep_set_stream", "pstep_update_params", "pstep_upload_particles", "pstep_download_particles", "pstep_set_tau_p", "pstep_set_particle_props", "pstep_set_correction", "pstep_set_wait_limit",
           "pstep_num_particles", "pstep_bind_velocity", "pstep_bind_temperature", "pstep_prime",
           "pstep_stage_interp_advance_deposit", "pstep_wrap", "pstep_stage_temp", "pstep_stage",
           "pstep_end_stage", "pstep_end_step", "pstep_run", "pstep_get_field", "pstep_energy_mean", "pstep_momentum_sums",
           "pstep_get_particle_array", "pstep_last_error", "pstep_status_string", "pstep_check",
           "pstep_last_run_ms", "pstep_launch_count", "pstep_profile", "pstep_profile_read"]
PHASES = ["advance", "deposit_int", "order", "sort", "deposit_temp", "reorder", "network"]


def lib():
    L = _lib.load_pstep()
    if getattr(L, "_typed", False):
        return L
    L.pstep_create.argtypes = [C.POINTER(Config), C.POINTER(_H)]
    L.pstep_destroy.argtypes = [_H]
    L.pstep_set_stream.argtypes = [_H, _VP]
    L.pstep_update_params.argtypes = [_H, C.POINTER(Config)]
    L.pstep_upload_particles.argtypes = [_H, C.c_int64] + [_VP] * 8 + [C.c_int]
    L.pstep_set_tau_p.argtypes = [_H, _VP, C.c_int]
    L.pstep_download_particles.argtypes = [_H] + [_VP] * 8 + [C.c_int]
    L.pstep_set_particle_props.argtypes = [_H, C.POINTER(Props), C.c_int]
    L.pstep_set_correction.argtypes = [_H, C.POINTER(Correction)]
    L.pstep_set_wait_limit.argtypes = [_H, C.c_uint32, C.c_int]
    L.pstep_num_particles.argtypes = [_H]
    L.pstep_num_particles.restype = C.c_int64
    L.pstep_bind_velocity.argtypes = [_H, _VP, _VP, _VP, C.c_int]
    L.pstep_bind_temperature.argtypes = [_H, _VP, C.c_int]
    L.pstep_prime.argtypes = [_H]
    L.pstep_stage_interp_advance_deposit.argtypes = [_H, C.c_int, C.c_double, C.c_double]
    L.pstep_wrap.argtypes = [_H]
    L.pstep_stage_temp.argtypes = [_H]
    L.pstep_stage.argtypes = [_H, C.c_int, C.c_double, C.c_double]
    L.pstep_end_stage.argtypes = [_H]
    L.pstep_end_step.argtypes = [_H]
    L.pstep_run.argtypes = [_H, C.c_int]
    L.pstep_get_field.argtypes = [_H, C.c_int, _VP, C.c_int]
    L.pstep_energy_mean.argtypes = [_H, _D]
    L.pstep_momentum_sums.argtypes = [_H, _D]
    L.pstep_get_particle_array.argtypes = [_H, C.c_int, _VP, C.c_int]
    L.pstep_last_error.argtypes = [_H]
    L.pstep_last_error.restype = C.c_char_p
    L.pstep_status_string.argtypes = [C.c_int]
    L.pstep_status_string.restype = C.c_char_p
    L.pstep_check.argtypes = [_H, C.POINTER(C.c_int32)]
    L.pstep_last_run_ms.argtypes = [_H, _D]
    L.pstep_launch_count.argtypes = [_H]
    L.pstep_launch_count.restype = C.c_int64
    L.pstep_profile.argtypes = [_H, C.c_int]
    L.pstep_profile_read.argtypes = [_H, _D, C.POINTER(C.c_int64), C.c_int]
    L.pstep_np_tot.argtypes = [_H, C.POINTER(C.c_int64)]
    L.pstep_max.argtypes = [_H, C.c_int, _D]
    L.pstep_balance_index.argtypes = [_H, _D]
    L.pstep_field_stats.argtypes = [_H, C.c_int, _D, _D, _D]
    L.pstep_find_tags.argtypes = [_H, _VP, C.c_int32, _VP, _VP]
    L.pstep_store_all.argtypes = [_H, C.c_char_p, C.c_int]
    L.pstep_load_all.argtypes = [_H, C.c_char_p, C.c_int64, C.c_int]
    L._typed = True
    return L


def _ptr(a):
    """numpy array -> (address, on_device=0); int -> device address (on_device=1)."""
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data, 0
    if hasattr(a, "data_ptr"):  # torch tensor on the device
        return int(a.data_ptr()), 1
    return int(a), 1


def make_config(step_cfg: dict, capacity: int, precision: int = FP64, flags: int = TRACK_ORDER) -> Config:
    c = Config()
    n = int(step_cfg["n"])
    c.nx = c.ny = c.nz = n
    c.bs = 1
    c.twc = int(step_cfg.get("twc", 1))
    c.particle_gravity = int(step_cfg.get("particle_gravity", 0))
    c.precision = precision
    c.flags = flags
    c.capacity = capacity
    c.lx = c.ly = c.lz = float(step_cfg["l"])
    for k in ("dt", "tp", "mp", "dp", "nu", "k", "epsilonp", "i0", "cvp", "gx", "gy", "gz"):
        setattr(c, k, float(step_cfg.get(k, 0.0)))
    return c


class ParticleStep:
    """One device-resident particle population with the reference's call surface."""

    def __init__(self, step_cfg: dict, capacity: int, precision: int = FP64, flags: int = TRACK_ORDER):
        self.L = lib()
        self.cfg = make_config(step_cfg, capacity, precision, flags)
        self.n = int(step_cfg["n"])
        h = _H()
        rc = self.L.pstep_create(C.byref(self.cfg), C.byref(h))
        if rc != 0:
            raise PstepError(rc, "pstep_create failed (no CUDA device, or unsupported configuration)")
        self.h = h
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.L.pstep_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc: int):
        if rc != 0:
            msg = self.L.pstep_last_error(self.h)
            raise PstepError(rc, msg.decode() if msg else "")

    # particle.cpp load_random / Load_All stand-in + grid.cpp:207-221
    def load(self, x, y, z, u, v, w, t, flag):
        ps = [_ptr(a) for a in (x, y, z, u, v, w, t, flag)]
        on_dev = ps[0][1]
        n = len(flag) if isinstance(flag, np.ndarray) else int(flag.numel())
        self._keep = [x, y, z, u, v, w, t, flag]
        self._ok(self.L.pstep_upload_particles(self.h, n, *[p for p, _ in ps], on_dev))

    def download(self, x, y, z, u, v, w, t, flag):
        """the base state and ids into preallocated arrays (pstep_download_particles)"""
        ps = [_ptr(a) for a in (x, y, z, u, v, w, t, flag)]
        self._ok(self.L.pstep_download_particles(self.h, *[p for p, _ in ps], ps[0][1]))

    def set_tau_p(self, tau):
        if tau is None:
            self._ok(self.L.pstep_set_tau_p(self.h, None, 0))
        else:
            p, d = _ptr(tau)
            self._ok(self.L.pstep_set_tau_p(self.h, p, d))

    def set_props(self, tau_p=None, mass_ratio=None, itth=None, heat_is=None, alpha=None, accel=None):
        """Per-particle properties in upload order (pstep_set_particle_props); None keeps
        the config's scalar. accel is a sequence of three arrays (or None)."""
        pr = Props()
        keep = []
        on_dev = None

        def addr(a):
            nonlocal on_dev
            if a is None:
                return None
            if isinstance(a, np.ndarray):
                a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            p, d = _ptr(a)
            if on_dev is not None and on_dev != d:
                raise ValueError("mix of host and device property arrays")
            on_dev = d
            return p

        pr.tau_p = addr(tau_p)
        pr.mass_ratio = addr(mass_ratio)
        pr.itth = addr(itth)
        pr.heat_is = addr(heat_is)
        pr.alpha = addr(alpha)
        if accel is not None:
            for d in range(3):
                pr.accel[d] = addr(accel[d])
        self._ok(self.L.pstep_set_particle_props(self.h, C.byref(pr), int(on_dev or 0)))

    def set_correction(self, model, nu_gas: float | None = None, every_stage: bool = False):
        """Learned correction (pstep_set_correction): model = dict(params, shift, scale, lo, hi)
        as made by first_repo_gb300.learn, nu_gas the gas kinematic viscosity; None: off.
        every_stage: run the network at every stage (default: stage 0, output kept for the step)."""
        if model is None:
            self._ok(self.L.pstep_set_correction(self.h, None))
            return
        c = Correction()
        self._corr_params = np.ascontiguousarray(model["params"], dtype=np.float32)
        c.params = self._corr_params.ctypes.data_as(C.POINTER(C.c_float))
        for name, n in (("shift", 10), ("scale", 10), ("lo", 4), ("hi", 4)):
            vals = np.asarray(model[name], dtype=np.float64)
            arr = getattr(c, name)
            for i in range(n):
                arr[i] = float(vals[i])
        c.prior_re = float(model.get("prior_re", 0.0))
        c.nu_gas = float(nu_gas if nu_gas is not None else model["nu_gas"])
        c.every_stage = 1 if every_stage else 0
        c.drive_cap = float(model.get("drive_cap", 0.0))
        self._ok(self.L.pstep_set_correction(self.h, C.byref(c)))

    def set_stream(self, stream: int):
        """the CUDA stream (cudaStream_t as an int; 0 = the default stream) this handle
        enqueues its work on (pstep_set_stream)"""
        self._ok(self.L.pstep_set_stream(self.h, C.c_void_p(int(stream))))

    def set_wait_limit(self, polls: int = 0, idle_first: bool = False):
        """bound of the fused inference's tensor-core completion waits (0: default); idle_first
        makes each warpgroup's first wait poll a barrier that nothing signals (timeout test)"""
        self._ok(self.L.pstep_set_wait_limit(self.h, int(polls), 1 if idle_first else 0))

    @property
    def np(self) -> int:
        return int(self.L.pstep_num_particles(self.h))

    def bind_velocity(self, ux, uy, uz):
        ps = [_ptr(a) for a in (ux, uy, uz)]
        self._ok(self.L.pstep_bind_velocity(self.h, ps[0][0], ps[1][0], ps[2][0], ps[0][1]))

    def bind_temperature(self, t):
        p, d = _ptr(t)
        self._ok(self.L.pstep_bind_temperature(self.h, p, d))

    def prime(self):
        self._ok(self.L.pstep_prime(self.h))

    def interp_advance_deposit(self, k: int):
        self._ok(self.L.pstep_stage_interp_advance_deposit(self.h, k, RK4_PRE[k], RK4_POST[k]))

    def wrap(self):
        self._ok(self.L.pstep_wrap(self.h))

    def stage_temp(self):
        self._ok(self.L.pstep_stage_temp(self.h))

    def stage(self, k: int):
        self._ok(self.L.pstep_stage(self.h, k, RK4_PRE[k], RK4_POST[k]))

    def end_stage(self):
        self._ok(self.L.pstep_end_stage(self.h))

    def end_step(self):
        self._ok(self.L.pstep_end_step(self.h))

    def run(self, nsteps: int):
        self._ok(self.L.pstep_run(self.h, nsteps))

    def last_run_ms(self) -> float:
        v = C.c_double()
        self._ok(self.L.pstep_last_run_ms(self.h, C.byref(v)))
        return v.value

    def field(self, name: str, out=None):
        g = self.n + 2
        if out is None:
            out = np.empty((g, g, g))
        p, d = _ptr(out)
        self._ok(self.L.pstep_get_field(self.h, FIELD_IDS[name], p, d))
        return out

    def energy_mean(self) -> float:
        v = C.c_double()
        self._ok(self.L.pstep_energy_mean(self.h, C.byref(v)))
        return v.value

    def momentum_sums(self) -> np.ndarray:
        """interior sums of the three deposited momentum fields of the last stage (fp64)"""
        out = np.zeros(3)
        self._ok(self.L.pstep_momentum_sums(self.h, out.ctypes.data_as(_D)))
        return out

    def array(self, name: str, out=None):
        """One particle array as fp64 (int32 ids). out: a preallocated numpy array, or a
        device buffer (a torch tensor, or an address) of np elements to fill in place."""
        n = self.np
        if out is None:
            out = np.empty(n, dtype=np.int32 if name == "flag" else np.float64)
        p, d = _ptr(out)
        if n:
            self._ok(self.L.pstep_get_particle_array(self.h, ARRAY_IDS[name], p, d))
        return out

    def check(self) -> int:
        f = C.c_int32()
        rc = self.L.pstep_check(self.h, C.byref(f))
        return rc, f.value

    def profile(self, enable: bool = True):
        self._ok(self.L.pstep_profile(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        ms = (C.c_double * len(PHASES))()
        cnt = (C.c_int64 * len(PHASES))()
        self._ok(self.L.pstep_profile_read(self.h, ms, cnt, len(PHASES)))
        return {p: (ms[i], cnt[i]) for i, p in enumerate(PHASES)}

    def launches(self) -> int:
        return int(self.L.pstep_launch_count(self.h))

    # ---- diagnostics (particle.cpp:662-741, tensor0.cpp:418-503) ----
    def np_tot(self) -> int:
        v = C.c_int64()
        self._ok(self.L.pstep_np_tot(self.h, C.byref(v)))
        return v.value

    def max(self, name: str) -> float:
        v = C.c_double()
        self._ok(self.L.pstep_max(self.h, ARRAY_IDS[name], C.byref(v)))
        return v.value

    def balance_index(self) -> float:
        v = C.c_double()
        self._ok(self.L.pstep_balance_index(self.h, C.byref(v)))
        return v.value

    def field_stats(self, name: str) -> tuple[float, float, float]:
        """(max, min, mean) of a deposited field over the interior"""
        mx, mn, me = C.c_double(), C.c_double(), C.c_double()
        self._ok(self.L.pstep_field_stats(self.h, FIELD_IDS[name], C.byref(mx), C.byref(mn), C.byref(me)))
        return mx.value, mn.value, me.value

    def find_tags(self, tags) -> tuple[np.ndarray, np.ndarray]:
        """positions (n, 3) of the particles with the given ids, and found flags"""
        t = np.ascontiguousarray(tags, dtype=np.int32)
        xyz = np.zeros((t.size, 3))
        found = np.zeros(t.size, dtype=np.int32)
        self._ok(self.L.pstep_find_tags(self.h, t.ctypes.data, t.size, xyz.ctypes.data, found.ctypes.data))
        return xyz, found.astype(bool)

    # ---- snapshot files (particle.cpp:867-1025) ----
    def store_all(self, data_dir: str, num_ts: int):
        self._ok(self.L.pstep_store_all(self.h, data_dir.encode(), int(num_ts)))

    def load_all(self, directory: str, n0: int, box: bool = True):
        self._ok(self.L.pstep_load_all(self.h, directory.encode(), int(n0), 1 if box else 0))
