"""In-tree build of the native libraries (no cmake; nvcc and gcc only).

  libpstep_gen.so  host C: seeded synthetic fields and particles (gcc, OpenMP)
  libpstep.so      the C-ABI and the sm_103a kernels (nvcc -gencode arch=compute_103a,code=sm_103a)

Every translation unit is compiled in parallel; outputs go to first_repo_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# FP64 drop-in kernels must not contract a*b+c into FMA: the reference's
# expressions are evaluated as separate IEEE operations, and the GPU must
# reproduce them bit for bit.
CU_UNITS = {
    "pstep_api.cu": ["-fmad=true"],
    "stage_f64.cu": ["-fmad=false"],
    "stage_f32.cu": ["-fmad=true"],
    "sort.cu": ["-fmad=true"],
    "deposit.cu": ["-fmad=false"],
    "order.cu": ["-fmad=true"],
    "mlp.cu": ["-fmad=true"],
    "gas.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "stats_io.cu": ["-fmad=false"],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpstep.so")
    return p


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build_gen(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, "pstep_gen.c")
    so = os.path.join(OUT, "libpstep_gen.so")
    if force or not _newer(so, [src]):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-std=c11", "-Wall",
              "-fPIC", "-shared", "-o", so, src, "-lm"])
    return so


def build_cuda(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libpstep.so")
    units = [u for u in CU_UNITS if os.path.exists(os.path.join(CSRC, u))]
    hdrs = _headers()
    objs = []
    jobs = []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + hdrs):
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", INCLUDE, "-I", CSRC, *CU_UNITS[u], "-c", src, "-o", obj]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or not _newer(so, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", so, *objs, "-lcudart"])
    return so


def build_all(force: bool = False) -> dict:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fg = ex.submit(build_gen, force)
        fc = ex.submit(build_cuda, force)
        return {"gen": fg.result(), "cuda": fc.result()}


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
