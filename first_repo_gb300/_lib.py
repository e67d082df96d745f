"""Locate and load the in-tree native libraries. There is no fallback: a missing
library is an error, so the CUDA path is always the one that runs."""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

_cache: dict = {}


def _load(name: str):
    if name in _cache:
        return _cache[name]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        raise RuntimeError(f"{name} is not built ({path} missing); run "
                           "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    _cache[name] = lib
    return lib


def load_gen():
    return _load("libpstep_gen.so")


def load_pstep():
    return _load("libpstep.so")


def path(name: str) -> str:
    return os.path.join(BUILD, name)
