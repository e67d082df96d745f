"""Python access to the checkers. TEST INFRASTRUCTURE: imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg.

  Oracle      ctypes wrapper of oracle/_build/libpstep_oracle.so (the C restatement)
  run_ref     runs oracle/_ref/ref_harness (the reference's own sources, built here)
  store_all, load_all, stats restatements   the snapshot files and statistics
              (particle.cpp:662-741, 867-1025; tensor0.cpp:418-503)
  run_ref_snapshot   the harness's Store_All / Load_All / statistics mode
"""
from __future__ import annotations

import json
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libpstep_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
# where the reference's sources lie: PSTEP_REFERENCE_DIR, else this build container's
# mount point; everything that needs them is skipped where the directory is absent
REFDIR = os.environ.get("PSTEP_REFERENCE_DIR", "/root/reference")

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
        lib.pso_set_props.argtypes = [C.c_void_p, C.c_int64] + [_D] * 8
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

    PROPS = ("tau_p", "mass_ratio", "itth", "heat_is", "alpha", "ax", "ay", "az")

    def set_props(self, n, **props):
        """per-particle properties indexed by particle id (flag); omitted ones keep the scalar"""
        unknown = set(props) - set(self.PROPS)
        if unknown:
            raise ValueError(f"unknown properties {unknown}")
        self._props = [None if props.get(k) is None else np.ascontiguousarray(props[k], dtype=np.float64)
                       for k in self.PROPS]
        ptrs = [None if a is None else _p(a) for a in self._props]
        assert _lib.pso_set_props(self.h, int(n), *ptrs) == 0

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


def run_ref_digests(bp, case: dict, nsteps: int, dump_mode: int = 2, chunk: int = 1 << 24) -> list[dict]:
    """Run the reference harness and digest its records as they stream out of a pipe
    (SHA-256 of every particle array, the flags and the five ghosted fields, first 32
    hex digits; mean(E) as a hex float), so that cases whose records are gigabytes each
    never touch the disk. dump_mode 2: a record after every step."""
    import hashlib
    import threading
    if build_ref() is None:
        raise RuntimeError("reference sources are not available here")
    d = tempfile.mkdtemp(prefix="pstep_refdig_")
    pfile, ifile = write_case(d, bp, case)
    fifo = os.path.join(d, "records.fifo")
    os.mkfifo(fifo)
    g3 = (bp.n + 2) ** 3
    recs: list[dict] = []
    err: list[BaseException] = []

    def reader():
        try:
            with open(fifo, "rb", buffering=0) as f:
                def take(nbytes: int) -> bytes:
                    out = bytearray()
                    while len(out) < nbytes:
                        b = f.read(min(chunk, nbytes - len(out)))
                        if not b:
                            raise EOFError("harness output ended inside a record")
                        out += b
                    return bytes(out)

                def digest_of(nbytes: int) -> str:
                    h = hashlib.sha256()
                    left = nbytes
                    while left:
                        b = f.read(min(chunk, left))
                        if not b:
                            raise EOFError("harness output ended inside an array")
                        h.update(b)
                        left -= len(b)
                    return h.hexdigest()[:32]

                while True:
                    hdr = f.read(8)
                    if not hdr:
                        break
                    if len(hdr) < 8:
                        hdr += take(8 - len(hdr))
                    tag, np_ = np.frombuffer(hdr, dtype=np.int32)
                    rec = {"tag": int(tag), "np": int(np_), "digests": {}}
                    for nm in ARRAYS[:32]:
                        rec["digests"][nm] = digest_of(8 * int(np_))
                    rec["digests"]["flag"] = digest_of(4 * int(np_))
                    for nm in FIELDS:
                        rec["digests"][nm] = digest_of(8 * g3)
                    rec["mean_E"] = float(np.frombuffer(take(8), dtype=np.float64)[0])
                    recs.append(rec)
        except BaseException as e:  # reported after the harness ends
            err.append(e)

    t = threading.Thread(target=reader)
    t.start()
    try:
        r = subprocess.run([REF_BIN, pfile, ifile, fifo, str(nsteps), str(dump_mode), "0"], capture_output=True,
                           text=True, cwd=d)
        t.join()
        if r.returncode != 0:
            raise RuntimeError("ref_harness failed:\n" + r.stdout + r.stderr)
        if err:
            raise err[0]
    finally:
        for f in os.listdir(d):
            os.remove(os.path.join(d, f))
        os.rmdir(d)
    return recs


# ---------------------------------------------------------------- snapshots and statistics
SNAP_NAMES = ["Part_x", "Part_y", "Part_z", "Part_u", "Part_v", "Part_w", "Part_T", "Part_flag"]
SNAP_KEYS = ["x", "y", "z", "u", "v", "w", "T", "flag"]


def store_all(data_dir: str, num_ts: int, arrays: dict) -> None:
    """particle::Store_All on one rank (particle.cpp:867-919): each quantity as raw
    native-endian values (double; int32 for the ids) in <data_dir><name>_<num_ts>.bin,
    offset 0, refusing an existing file (MPI_MODE_EXCL)."""
    for name, key in zip(SNAP_NAMES, SNAP_KEYS):
        dt = np.int32 if key == "flag" else np.float64
        with open(f"{data_dir}{name}_{num_ts}.bin", "xb") as f:
            f.write(np.ascontiguousarray(arrays[key], dtype=dt).tobytes())


def load_all(directory: str, n0: int, box: bool = True) -> dict:
    """particle::Load_All on one rank (particle.cpp:948-1025): n0 values of each
    quantity from <dir>Restart_<name>.bin (the IO duct's files with _IO)."""
    out = {}
    for name, key in zip(SNAP_NAMES, SNAP_KEYS):
        dt = np.int32 if key == "flag" else np.float64
        a = np.fromfile(f"{directory}Restart_{name}{'' if box else '_IO'}.bin", dtype=dt, count=n0)
        if a.size != n0:
            raise IOError(f"short restart file for {name}")
        out[key] = a
    return out


def array_max(v: np.ndarray) -> float:
    """particle::max (particle.cpp:671-685): -1e9 without particles, else the first
    element raised by every strictly larger one"""
    if v.size == 0:
        return -1e9
    m = v[0]
    larger = v[v > m]
    return float(max(m, larger.max())) if larger.size else float(m)


def field_stats(f: np.ndarray, n: int) -> tuple[float, float, float]:
    """tensor0::max, ::min (tensor0.cpp:452-463, 492-503) over the interior and ::mean
    (:418-435): the interior sum in the reference's i-j-k loop order over size_tot"""
    interior = f[1:n + 1, 1:n + 1, 1:n + 1]  # [k][j][i]
    s = 0.0
    for v in np.ascontiguousarray(interior.transpose(2, 1, 0)).ravel():  # i outermost, k innermost
        s += float(v)
    return float(interior.max()), float(interior.min()), s / float(n * n * n)


def trajectory_ids(n0: int, np_track: int) -> list[int]:
    """ids particle::trajectory reports (particle.cpp:687-719): 0, K, 2K, ... < N0,
    K = ceil(N0 / Np_track)"""
    if np_track == 0:
        return []
    k = (n0 + np_track - 1) // np_track
    return list(range(0, n0, k))


def run_ref_snapshot(bp, case: dict, nsteps: int, workdir: str, store_ts: int = -1, load: bool = False,
                     np_track: int = 0) -> tuple[list[dict], dict | None, list[list[float]]]:
    """Run the harness with Store_All (store_ts >= 0), statistics and trajectory
    (np_track > 0, statistics on) and/or Load_All (load: Restart_Part_*.bin in workdir).
    Returns the records, the STATS line and the trajectory rows (time, then x y z per id)."""
    if build_ref() is None:  # incremental: rebuilds only when the harness or its sources changed
        raise RuntimeError("reference sources are not available here")
    pfile, ifile = write_case(workdir, bp, case)
    if np_track:
        lines = open(pfile).read().split("\n")
        lines[4] = str(np_track)  # Np_track
        lines[6] = "1 0"          # Statistics Stat_print
        with open(pfile, "w") as f:
            f.write("\n".join(lines))
    ofile = os.path.join(workdir, "output.bin")
    r = subprocess.run([REF_BIN, pfile, ifile, ofile, str(nsteps), "0", "0", str(store_ts), "1" if load else "0"],
                       capture_output=True, text=True, cwd=workdir)
    if r.returncode != 0:
        raise RuntimeError("ref_harness failed:\n" + r.stdout + r.stderr)
    stats = None
    for line in r.stdout.splitlines():
        if line.startswith("STATS "):
            stats = json.loads(line[6:])
    traj = []
    tpath = os.path.join(workdir, "Part_trajectory.dat")
    if os.path.exists(tpath):
        traj = [[float(v) for v in ln.split()] for ln in open(tpath) if ln.strip()]
    return read_records(ofile, bp.n), stats, traj


def run_ref(bp, case: dict, nsteps: int, dump_all: bool = True, timing: bool = False, workdir: str | None = None):
    """Run the reference's own particle step (oracle/_ref/ref_harness) on a case."""
    if build_ref() is None:  # incremental: rebuilds only when the harness or its sources changed
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


# ---------------------------------------------------------------- gas step
GAS_REF_BIN = os.path.join(HERE, "_ref", "gas_harness")
GAS_FIELDS = ["RU_x", "RU_y", "RU_z", "Rho", "P", "T", "U_x", "U_y", "U_z", "C", "RHS_RU_x", "RHS_RU_y", "RHS_RU_z",
              "RHS_Part_Temp", "divergence", "Rho_new"]
GAS_REC_FIELDS = ["RU_x", "RU_y", "RU_z", "Rho", "P", "T", "RHS_Part_Temp", "C", "RHS_RU_x", "RHS_RU_y", "RHS_RU_z"]


class _GasCfg(C.Structure):
    _fields_ = [("n", C.c_int32), ("cooling", C.c_int32), ("iterations", C.c_int32), ("twc", C.c_int32),
                ("l", C.c_double), ("dt", C.c_double), ("mu0", C.c_double), ("k", C.c_double), ("cp", C.c_double),
                ("cv", C.c_double), ("rho0", C.c_double), ("u0", C.c_double), ("a_force", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double), ("mp", C.c_double),
                ("epsilon", C.c_double)]


def _gas_lib():
    lib = _load()
    if not getattr(lib, "_gas", False):
        lib.pgo_create.restype = C.c_void_p
        lib.pgo_create.argtypes = [C.POINTER(_GasCfg), C.c_void_p]
        lib.pgo_destroy.argtypes = [C.c_void_p]
        lib.pgo_init.argtypes = [C.c_void_p] + [_D] * 4 + [C.c_double]
        lib.pgo_step.argtypes = [C.c_void_p]
        lib.pgo_field.restype = _D
        lib.pgo_field.argtypes = [C.c_void_p, C.c_int]
        lib.pgo_scalar.restype = C.c_double
        lib.pgo_scalar.argtypes = [C.c_void_p, C.c_int]
        lib.gas_fft3d.argtypes = [_D, C.c_int, C.c_int]
        lib._gas = True
    return lib


class GasOracle:
    """The C restatement of the box gas step (oracle/gas_oracle.c), optionally
    coupled to a particle-step Oracle (which it drives)."""

    def __init__(self, gcfg: dict, particles: "Oracle | None" = None):
        lib = _gas_lib()
        c = _GasCfg()
        for k in ("n", "cooling", "iterations", "twc"):
            setattr(c, k, int(gcfg[k]))
        for k in ("l", "dt", "mu0", "k", "cp", "cv", "rho0", "u0", "a_force", "gx", "gy", "gz", "mp", "epsilon"):
            setattr(c, k, float(gcfg[k]))
        self.n = int(gcfg["n"])
        self.particles = particles
        self.h = lib.pgo_create(C.byref(c), particles.h if particles is not None else None)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.pgo_destroy(self.h)
            self.h = None

    def init(self, ru_x, ru_y, ru_z, rho, p0):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ru_x, ru_y, ru_z, rho)]
        assert _lib.pgo_init(self.h, *[_p(a) for a in arrs], float(p0)) == 0

    def step(self):
        assert _lib.pgo_step(self.h) == 0

    def field(self, name: str) -> np.ndarray:
        g = self.n + 2
        p = _lib.pgo_field(self.h, GAS_FIELDS.index(name))
        return np.ctypeslib.as_array(p, shape=(g, g, g)).copy()

    def p0(self) -> float:
        return float(_lib.pgo_scalar(self.h, 0))

    def iterations(self) -> int:
        return int(_lib.pgo_scalar(self.h, 3))


def fft3d(data: np.ndarray, sign: int) -> np.ndarray:
    """oracle's radix-2 complex FFT on an (n, n, n) complex array (copy)."""
    a = np.ascontiguousarray(data, dtype=np.complex128).copy()
    _gas_lib().gas_fft3d(a.ctypes.data_as(_D), a.shape[0], int(sign))
    return a


def build_gas_ref() -> str | None:
    if not ref_available():
        return None
    r = subprocess.run(["make", "-s", "-C", HERE, "gasref", f"REFDIR={REFDIR}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference gas build failed:\n" + r.stdout + r.stderr)
    return GAS_REF_BIN


def run_gas_ref(bp, fields: dict, particles: dict, nsteps: int, p0: float) -> list[dict]:
    """Run the reference's own box gas step (oracle/_ref/gas_harness). fields: interior
    RU_x, RU_y, RU_z, Rho; particles: x y z u v w t flag."""
    if not os.path.exists(GAS_REF_BIN):
        if build_gas_ref() is None:
            raise RuntimeError("reference sources are not available here")
    d = tempfile.mkdtemp(prefix="pstep_gasref_")
    try:
        pfile = os.path.join(d, "params.in")
        with open(pfile, "w") as f:
            f.write(bp.params_file())
        ifile = os.path.join(d, "input.bin")
        n = len(particles["flag"])
        with open(ifile, "wb") as f:
            f.write(np.int64(n).tobytes())
            f.write(np.int32(bp.n).tobytes())
            f.write(np.float64(p0).tobytes())
            for k in ("RU_x", "RU_y", "RU_z", "Rho"):
                f.write(np.ascontiguousarray(fields[k], dtype=np.float64).tobytes())
            for k in ("x", "y", "z", "u", "v", "w", "t"):
                f.write(np.ascontiguousarray(particles[k], dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(particles["flag"], dtype=np.int32).tobytes())
        ofile = os.path.join(d, "output.bin")
        r = subprocess.run([GAS_REF_BIN, pfile, ifile, ofile, str(nsteps)], capture_output=True, text=True, cwd=d)
        if r.returncode != 0:
            raise RuntimeError("gas_harness failed:\n" + r.stdout + r.stderr)
        raw = open(ofile, "rb").read()
    finally:
        for f in os.listdir(d):
            os.remove(os.path.join(d, f))
        os.rmdir(d)
    g = bp.n + 2
    g3 = g ** 3
    recs, off = [], 0
    while off < len(raw):
        step, np_ = np.frombuffer(raw, dtype=np.int32, count=2, offset=off)
        off += 8
        rec = {"step": int(step), "np": int(np_)}
        for nm in GAS_REC_FIELDS:
            rec[nm] = np.frombuffer(raw, dtype=np.float64, count=g3, offset=off).reshape(g, g, g).copy()
            off += 8 * g3
        rec["P0"] = float(np.frombuffer(raw, dtype=np.float64, count=1, offset=off)[0])
        off += 12
        for nm in ("x", "y", "z", "u", "v", "w", "T"):
            rec[nm] = np.frombuffer(raw, dtype=np.float64, count=np_, offset=off).copy()
            off += 8 * np_
        rec["flag"] = np.frombuffer(raw, dtype=np.int32, count=np_, offset=off).copy()
        off += 4 * np_
        recs.append(rec)
    return recs
