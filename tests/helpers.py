"""Shared helpers for the parity tests: case construction, digests and the
oracle driven in the reference's call order."""
import hashlib
import json
import os

import numpy as np

from first_repo_gb300 import config, gen

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

PART = ["x", "y", "z", "u", "v", "w", "T", "x_int", "y_int", "z_int", "u_int", "v_int", "w_int", "T_int",
        "x_new", "y_new", "z_new", "u_new", "v_new", "w_new", "T_new",
        "x_np1", "y_np1", "z_np1", "u_np1", "v_np1", "w_np1", "T_np1", "RHS_T"]
FIELD_MAP = {"C": "C", "Ax": "RHS_RU_x", "Ay": "RHS_RU_y", "Az": "RHS_RU_z", "E": "RHS_Part_Temp"}


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def golden():
    with open(os.path.join(GOLDEN, "reference_digests.json")) as f:
        return json.load(f)


def golden_case(name):
    for c in golden()["cases"]:
        if c["name"] == name:
            return c
    raise KeyError(name)


def make_bp(n, count, extra=None):
    extra = extra or {}
    bp = config.box_params(n, count, twc=extra.get("twc", 1))
    bp.particle_gravity = extra.get("particle_gravity", 0)
    bp.gx, bp.gy, bp.gz = extra.get("gx", 0.0), extra.get("gy", 0.0), extra.get("gz", 0.0)
    return bp


def ghosted_fields(case):
    return [gen.ghost(case[k]) for k in ("ux", "uy", "uz", "T")]


def bits_equal(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def max_rel_to_max(a, b) -> float:
    """max|a-b| / max|b| (0 when both are zero)."""
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    m = float(np.max(np.abs(b))) if b.size else 0.0
    return 0.0 if d == 0.0 else d / (m if m > 0 else 1.0)
