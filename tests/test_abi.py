"""The drop-in boundary: libpstep.so builds, loads without a GPU, and exports
every entry point include/pstep.h declares (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import pytest

import helpers  # noqa: F401  (sets sys.path)
import pyoracle
from first_repo_gb300 import _lib, gas, mlp, pstep

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix="pstep_"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_binding_surface():
    names = declared("pstep.h")
    assert set(pstep.EXPORTS) <= set(names)


def test_library_exports_every_declared_symbol(built_cuda):
    lib = ctypes.CDLL(_lib.path("libpstep.so"))
    for name in declared("pstep.h"):
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.path("libpstep.so")], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(pstep_[a-z0-9_]+)\b", out))
    for name in declared("pstep.h"):
        assert name in exported, name


def test_mlp_header_matches_binding_and_exports(built_cuda):
    names = declared("pstep_mlp.h", "pmlp_")
    assert set(mlp.EXPORTS) == set(names)
    lib = ctypes.CDLL(_lib.path("libpstep.so"))
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.path("libpstep.so")], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(pmlp_[a-z0-9_]+)\b", out))
    for name in names:
        assert hasattr(lib, name), name
        assert name in exported, name


def test_gas_header_matches_binding_and_exports(built_cuda):
    names = declared("pstep_gas.h", "pgas_")
    assert set(gas.EXPORTS) == set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.path("libpstep.so")], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(pgas_[a-z0-9_]+)\b", out))
    for name in names:
        assert name in exported, name


def test_status_strings_without_device(built_cuda):
    L = pstep.lib()
    assert L.pstep_status_string(0) == b"ok"
    assert L.pstep_status_string(3) == b"capacity exceeded"


def test_create_rejects_bad_config_without_touching_device(built_cuda):
    L = pstep.lib()
    c = pstep.Config()
    c.nx = c.ny = c.nz = 8
    c.bs = 2  # the reference's box uses bs = 1
    c.lx = c.ly = c.lz = 1.0
    c.dt = 1e-3
    h = ctypes.c_void_p()
    assert L.pstep_create(ctypes.byref(c), ctypes.byref(h)) == 2
    c.bs = 1
    c.nx = 1
    assert L.pstep_create(ctypes.byref(c), ctypes.byref(h)) == 2
    assert L.pstep_create(None, ctypes.byref(h)) == 1


def test_null_handle_is_an_error(built_cuda):
    L = pstep.lib()
    assert L.pstep_prime(None) == 1
    assert L.pstep_end_step(None) == 1
    assert L.pstep_num_particles(None) == -1
    # statistics and snapshot files (no device is touched for these argument checks)
    v64, d = ctypes.c_int64(), ctypes.c_double()
    assert L.pstep_np_tot(None, ctypes.byref(v64)) == 1
    assert L.pstep_max(None, 0, ctypes.byref(d)) == 1
    assert L.pstep_balance_index(None, ctypes.byref(d)) == 1
    assert L.pstep_field_stats(None, 0, None, None, None) == 1
    assert L.pstep_find_tags(None, None, 0, None, None) == 1
    assert L.pstep_store_all(None, b"./", 0) == 1
    assert L.pstep_load_all(None, b"./", 1, 1) == 1
    assert L.pstep_status_string(11) == b"snapshot file error"


REFDIR = pyoracle.REFDIR  # PSTEP_REFERENCE_DIR, skipped where absent


@pytest.mark.skipif(not os.path.exists(os.path.join(REFDIR, "particle.h")), reason="reference headers not present")
def test_adapter_compiles_and_links_against_reference_headers(built_cuda, tmp_path):
    """first_repo_gb300/adapter/particle_gpu.cpp builds in place of the reference's
    particle.cpp against its unchanged particle.h, and links with the reference's
    other sources and libpstep.so (running it needs a GPU)."""
    obj = tmp_path / "particle_gpu.o"
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I", os.path.join(ROOT, "oracle", "mpi_stub"), "-I", REFDIR,
           "-I", os.path.join(ROOT, "include"), "-c", os.path.join(ROOT, "first_repo_gb300", "adapter", "particle_gpu.cpp"),
           "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    main = tmp_path / "main.cpp"
    main.write_text('#include "mpi.h"\n#include "params.h"\n#include "proc.h"\n#include "gridsize.h"\n'
                    '#include "particle.h"\nint main(int c, char **v) { if (c < 2) return 0; MPI_Init(&c, &v);\n'
                    'params p(v[1]); proc pc; gridsize s(&p, &pc); particle part(&p, &pc, &s); return 0; }\n')
    srcs = [os.path.join(REFDIR, f) for f in ("tensor0.cpp", "tensor1.cpp", "communicator.cpp", "gridsize.cpp",
                                              "proc.cpp", "params.cpp")]
    exe = tmp_path / "app"
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I", os.path.join(ROOT, "oracle", "mpi_stub"), "-I", REFDIR,
           str(main), str(obj), *srcs, "-L", os.path.dirname(_lib.path("libpstep.so")), "-lpstep",
           "-L/usr/local/cuda/lib64", "-lcudart", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
