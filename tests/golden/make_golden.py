"""Generate the golden fixtures from the REFERENCE's own particle step.

Runs oracle/_ref/ref_harness (the reference's particle.cpp, tensor0/1.cpp,
communicator.cpp, gridsize.cpp, proc.cpp, params.cpp compiled from source with
the single-rank MPI stub) on seeded synthetic cases and records, per call of
the harness (prime, every stage, final state), SHA-256 digests of every array,
plus the full final state of the smallest case.

The configuration-sized case (box256_clustered: 256^3 cells, 2^24 clustered
particles, 10 steps -- the plain FP64 drop-in's named configuration) records a
digest of every array after the prime, after every step and at the end; its
records (about 5 GB each) are digested as they stream out of the harness and
written to reference_digests_box256.json.

usage: python tests/golden/make_golden.py [--sized]    (needs the reference sources)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from first_repo_gb300 import build, config, gen  # noqa: E402
import pyoracle  # noqa: E402

CASES = [
    # name, cells, particles, seed, clustered, steps, extra box_params
    ("box12_small", 12, 1024, 11, False, 3, {}),
    ("box16_twc_off_gravity", 16, 3000, 12, True, 2, {"twc": 0, "particle_gravity": 1, "gz": -0.5, "gx": 0.25}),
    ("box32_clustered", 32, 20000, 13, True, 2, {}),
    ("box64_uniform", 64, 1 << 15, 1001, False, 1, {}),
]

STATE = ["x", "y", "z", "x_int", "y_int", "z_int", "x_new", "y_new", "z_new", "x_np1", "y_np1", "z_np1",
         "u", "v", "w", "u_int", "v_int", "w_int", "u_new", "v_new", "w_new", "u_np1", "v_np1", "w_np1",
         "T", "T_int", "T_new", "T_np1", "RHS_T", "flag", "C", "Ax", "Ay", "Az", "E"]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def case_inputs(n, count, seed, clustered):
    return gen.make_case(n, count, seed, clustered)


def make_bp(n, count, extra):
    bp = config.box_params(n, count, twc=extra.get("twc", 1))
    bp.particle_gravity = extra.get("particle_gravity", 0)
    bp.gx, bp.gy, bp.gz = extra.get("gx", 0.0), extra.get("gy", 0.0), extra.get("gz", 0.0)
    return bp


# name, workload (config.WORKLOADS), steps
SIZED_CASES = [("box256_clustered", "box256_clustered", 10)]
SIZED_FILE = os.path.join(HERE, "reference_digests_box256.json")


def main_sized():
    import time
    build.build_gen()
    if pyoracle.build_ref() is None:
        sys.exit("reference sources not found; golden fixtures come from the reference itself")
    out = {"generator": "first_repo_gb300/csrc/pstep_gen.c", "cases": []}
    for name, wname, steps in SIZED_CASES:
        wl = config.WORKLOADS[wname]
        bp = config.box_params(wl.n, wl.n_particles, dp_over_dx=wl.dp_over_dx, mass_loading=wl.mass_loading)
        case = gen.make_case(wl.n, wl.n_particles, wl.seed, wl.clustered, nblobs=wl.nblobs)
        t0 = time.time()
        recs = pyoracle.run_ref_digests(bp, case, steps, dump_mode=2)
        entry = {
            "name": name, "workload": wname, "n": wl.n, "count": wl.n_particles, "seed": wl.seed,
            "clustered": wl.clustered, "nblobs": wl.nblobs, "steps": steps, "step_config": bp.step_config(),
            "inputs": {k: digest(case[k]) for k in ("ux", "uy", "uz", "T", "x", "y", "z", "u", "v", "w", "t", "flag")},
            "reference_seconds": round(time.time() - t0, 1),
            "records": [{"tag": r["tag"], "np": r["np"], "mean_E": r["mean_E"].hex(),
                         "digests": {k: r["digests"][k] for k in STATE}} for r in recs],
        }
        out["cases"].append(entry)
        print(name, "records", len(recs), f"{time.time() - t0:.0f} s")
    with open(SIZED_FILE, "w") as f:
        json.dump(out, f, indent=1)


def main():
    build.build_gen()
    if pyoracle.build_ref() is None:
        sys.exit("reference sources not found; golden fixtures come from the reference itself")
    out = {"generator": "first_repo_gb300/csrc/pstep_gen.c", "cases": []}
    for name, n, count, seed, clustered, steps, extra in CASES:
        bp = make_bp(n, count, extra)
        case = case_inputs(n, count, seed, clustered)
        recs, _ = pyoracle.run_ref(bp, case, steps, dump_all=True)
        entry = {
            "name": name, "n": n, "count": count, "seed": seed, "clustered": clustered, "steps": steps,
            "extra": extra, "step_config": bp.step_config(),
            "inputs": {k: digest(case[k]) for k in ("ux", "uy", "uz", "T", "x", "y", "z", "u", "v", "w", "t", "flag")},
            "records": [],
        }
        for r in recs:
            entry["records"].append({"tag": r["tag"], "np": r["np"], "mean_E": r["mean_E"].hex(),
                                     "digests": {k: digest(r[k]) for k in STATE}})
        out["cases"].append(entry)
        if name == "box12_small":
            fin = recs[-1]
            keep = ["x", "y", "z", "u", "v", "w", "T", "RHS_T", "flag", "C", "Ax", "Ay", "Az", "E"]
            np.savez_compressed(os.path.join(HERE, "box12_small_final.npz"),
                                **{k: fin[k] for k in keep}, mean_E=np.float64(fin["mean_E"]))
        print(name, "records", len(recs))
    with open(os.path.join(HERE, "reference_digests.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if "--sized" in sys.argv:
        main_sized()
    else:
        main()
