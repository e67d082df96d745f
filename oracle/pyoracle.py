"""Python access to the checkers. TEST INFRASTRUCTURE: imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg.

  Oracle      ctypes wrapper of oracle/_build/libpstep_oracle.so (the C restatement)
  run_ref     runs oracle/_ref/ref_harness (the reference's own sources, built here)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libpstep_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
REFDIR = "/root/reference"

ARRAYS = ["x", "y", "z", "x_int", "y_int", "z_int", "x_new", "y_new", "z_new", "x_np1", "y_np1", "z_np1",
          "u", "v", "w", "u_int", "v_int", "w_int", "u_new", "v_new", "w_new", "u_np1", "v_np1", "w_np1",
          "T", "T_int", "T_new", "T_np1", "RHS_u", "RHS_v", "RHS_w", "RHS_T", "ug", "vg", "wg", "Tg"]
FIELDS = ["C", "Ax", "Ay", "Az", "E"]


def build_port() -> str:
    r = subprocess.run(["make", "-s", "-C", HERE, "port"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + r.stdout + r.stderr)
    return PORT_SO


def ref_available() -> bool:
    return os.path.isdir(REFDIR) and os.path.exists(os.path.join(REFDIR, "particle.cpp"))


def build_ref() -> str | None:
    """Compile the reference's particle path from its sources (only where they exist)."""
    if not ref_available():
        return None
    r = subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFDIR={REFDIR}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return REF_BIN


class _Cfg(C.Structure):
    _fields_ = [("n", C.c_int32), ("particle_gravity", C.c_int32), ("twc", C.c_int32), ("pad", C.c_int32),
                ("l", C.c_double), ("dt", C.c_double), ("tp", C.c_double), ("mp", C.c_double),
                ("dp", C.c_double), ("nu", C.c_double), ("k", C.c_double), ("epsilonp", C.c_double),
                ("i0", C.c_double), ("cvp", C.c_double), ("gx", C.c_double), ("gy", C.c_double),
                ("gz", C.c_double)]


_D = C.POINTER(C.c_double)


def _p(a):
    return a.ctypes.data_as(_D)


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(PORT_SO):
            build_port()
        lib = C.CDLL(PORT_SO)
        lib.pso_create.restype = C.c_void_p
        lib.pso_create.argtypes = [C.POINTER(_Cfg), C.c_int64]
        lib.pso_destroy.argtypes = [C.c_void_p]
        lib.pso_load.argtypes = [C.c_void_p, C.c_int64] + [_D] * 7 + [C.POINTER(C.c_int32)]
        lib.pso_prime.argtypes = [C.c_void_p, _D, _D]
        lib.pso_stage.argtypes = [C.c_void_p, C.c_int] + [_D] * 4 + [_D] * 5
        lib.pso_end_stage.argtypes = [C.c_void_p]
        lib.pso_end_step.argtypes = [C.c_void_p]
        lib.pso_array.restype = _D
        lib.pso_array.argtypes = [C.c_void_p, C.c_int]
        lib.pso_flag.restype = C.POINTER(C.c_int32)
        lib.pso_flag.argtypes = [C.c_void_p]
        lib.pso_np.restype = C.c_int64
        lib.pso_np.argtypes = [C.c_void_p]
        lib.pso_edge_hits.restype = C.c_int64
        lib.pso_edge_hits.argtypes = [C.c_void_p]
        lib.pso_mean.restype = C.c_double
        lib.pso_mean.argtypes = [_D, C.c_int32]
        lib.pso_run.argtypes = [C.c_void_p, C.c_int] + [_D] * 4 + [_D] * 5
        _lib = lib
    return _lib


class Oracle:
    """The C restatement driven in the reference's call order."""

    def __init__(self, cfg: dict, capacity: int):
        lib = _load()
        c = _Cfg()
        for k in ("n", "particle_gravity", "twc"):
            setattr(c, k, int(cfg[k]))
        for k in ("l", "dt", "tp", "mp", "dp", "nu", "k", "epsilonp", "i0", "cvp", "gx", "gy", "gz"):
            setattr(c, k, float(cfg[k]))
        self.n = int(cfg["n"])
        self.h = lib.pso_create(C.byref(c), capacity)
        g = self.n + 2
        self.fields = {f: np.zeros((g, g, g)) for f in FIELDS}

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pso_destroy(self.h)
            self.h = None

    def load(self, x, y, z, u, v, w, t, flag):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, u, v, w, t)]
        fl = np.ascontiguousarray(flag, dtype=np.int32)
        rc = _lib.pso_load(self.h, len(fl), *[_p(a) for a in arrs], fl.ctypes.data_as(C.POINTER(C.c_int32)))
        assert rc == 0

    def prime(self, tfield_g):
        _lib.pso_prime(self.h, _p(tfield_g), _p(self.fields["E"]))

    def stage(self, k, ux_g, uy_g, uz_g, tf_g):
        f = self.fields
        rc = _lib.pso_stage(self.h, k, _p(ux_g), _p(uy_g), _p(uz_g), _p(tf_g), _p(f["C"]), _p(f["Ax"]),
                            _p(f["Ay"]), _p(f["Az"]), _p(f["E"]))
        assert rc == 0

    def end_stage(self):
        _lib.pso_end_stage(self.h)

    def end_step(self):
        _lib.pso_end_step(self.h)

    def run(self, nsteps, ux_g, uy_g, uz_g, tf_g):
        f = self.fields
        _lib.pso_run(self.h, nsteps, _p(ux_g), _p(uy_g), _p(uz_g), _p(tf_g), _p(f["C"]), _p(f["Ax"]),
                     _p(f["Ay"]), _p(f["Az"]), _p(f["E"]))

    @property
    def np(self) -> int:
        return int(_lib.pso_np(self.h))

    @property
    def edge_hits(self) -> int:
        return int(_lib.pso_edge_hits(self.h))

    def array(self, name: str) -> np.ndarray:
        i = ARRAYS.index(name)
        p = _lib.pso_array(self.h, i)
        return np.ctypeslib.as_array(p, shape=(self.np,)).copy()

    def flag(self) -> np.ndarray:
        return np.ctypeslib.as_array(_lib.pso_flag(self.h), shape=(self.np,)).copy()

    def mean(self, field: np.ndarray) -> float:
        return float(_lib.pso_mean(_p(np.ascontiguousarray(field)), self.n))


def write_case(dirname: str, bp, case: dict) -> tuple[str, str]:
    """params.in + input.bin for ref_harness."""
    pfile = os.path.join(dirname, "params.in")
    with open(pfile, "w") as f:
        f.write(bp.params_file())
    ifile = os.path.join(dirname, "input.bin")
    n = case["x"].shape[0]
    with open(ifile, "wb") as f:
        f.write(np.int64(n).tobytes())
        f.write(np.int32(bp.n).tobytes())
        for k in ("ux", "uy", "uz", "T"):
            f.write(np.ascontiguousarray(case[k], dtype=np.float64).tobytes())
        for k in ("x", "y", "z", "u", "v", "w", "t"):
            f.write(np.ascontiguousarray(case[k], dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(case["flag"], dtype=np.int32).tobytes())
    return pfile, ifile


def read_records(path: str, n_cells: int) -> list[dict]:
    """Parse ref_harness output: per record the 32 particle arrays, flag, 5 ghosted fields, mean(E)."""
    g3 = (n_cells + 2) ** 3
    raw = open(path, "rb").read()
    off = 0
    recs = []
    names = ARRAYS[:32]
    while off < len(raw):
        tag, np_ = np.frombuffer(raw, dtype=np.int32, count=2, offset=off)
        off += 8
        rec = {"tag": int(tag), "np": int(np_)}
        for nm in names:
            rec[nm] = np.frombuffer(raw, dtype=np.float64, count=np_, offset=off).copy()
            off += 8 * np_
        rec["flag"] = np.frombuffer(raw, dtype=np.int32, count=np_, offset=off).copy()
        off += 4 * np_
        g = n_cells + 2
        for nm in FIELDS:
            rec[nm] = np.frombuffer(raw, dtype=np.float64, count=g3, offset=off).reshape(g, g, g).copy()
            off += 8 * g3
        rec["mean_E"] = float(np.frombuffer(raw, dtype=np.float64, count=1, offset=off)[0])
        off += 8
        recs.append(rec)
    return recs


def run_ref(bp, case: dict, nsteps: int, dump_all: bool = True, timing: bool = False, workdir: str | None = None):
    """Run the reference's own particle step (oracle/_ref/ref_harness) on a case."""
    if not os.path.exists(REF_BIN):
        if build_ref() is None:
            raise RuntimeError("reference sources are not available here")
    own = workdir is None
    d = workdir or tempfile.mkdtemp(prefix="pstep_ref_")
    pfile, ifile = write_case(d, bp, case)
    ofile = os.path.join(d, "output.bin")
    r = subprocess.run([REF_BIN, pfile, ifile, ofile, str(nsteps), "1" if dump_all else "0",
                        "1" if timing else "0"], capture_output=True, text=True, cwd=d)
    if r.returncode != 0:
        raise RuntimeError("ref_harness failed:\n" + r.stdout + r.stderr)
    recs = read_records(ofile, bp.n)
    if own:
        for f in os.listdir(d):
            os.remove(os.path.join(d, f))
        os.rmdir(d)
    return recs, r.stdout
