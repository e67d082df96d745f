"""Parity at the named configurations' own sizes.

box256_clustered (256^3 cells, 2^24 particles, 50% in 64 Gaussian blobs, 10 steps):
the FP64 drop-in against the reference's own particle step, compiled from its
sources, on identical inputs. The reference's record after every step is committed
as SHA-256 digests of every array (tests/golden/reference_digests_box256.json, made
by tests/golden/make_golden.py --sized); with PSTEP_TRACK_ORDER |
PSTEP_REFERENCE_SUMS every particle array in the reference's order, the ids and the
five ghosted deposited fields must be bit-identical after every step, and the
energy mean within 1e-12 (a different fixed summation order). The default mode
(order tracking, fast deposit) runs beside it: bit-identical particle states, and
deposited fields within 1e-12 of max|field| of the exact run's.

box512_mixed (512^3 cells, 2^27 particles, tau_p log-uniform in [0.01, 1]): the FP32
form against the FP64 drop-in -- itself pinned to the reference above and in
tests/test_parity_gpu.py -- on the same inputs, one step. The reference cannot
hold per-particle tau_p or be constructed at this size (particle.cpp:23-26), so the
FP64 drop-in is the FP64 run the configuration names. Bound 1e-5, measured per
particle (positions in cell units, velocity vectors and temperatures relative to
their own magnitude, RHS_T relative to its maximum) over all but a fraction 1e-6 of
the particles, and for the deposited concentration and energy norm-wise. The
excluded few sit on cell faces: the reference's face-normal interpolation
(particle.cpp:340-360) is piecewise constant across the other two axes, so a
particle within the fp32 resolution of a face (about 1e-7 cells) can take the
neighbouring cell's transverse velocity -- measured: 17 of 2^27 particles move more
than 1e-6 cells apart, at most 4e-5 cells, every one a particle that crossed a cell
face during the step (also with scalar tau_p).
The deposited momentum is the drag RHS_u = (u_gas - u_p) / tau_p, a difference of two
velocities of size u_rms. The particles start at the gas velocity, so after one step
the slip is about 1e-3 u_rms, and fp32 velocities (relative resolution 6e-8) carry it
to about 1e-4; tau_p down to 0.01 puts those particles' drag among the largest deposits.
Measured: RHS_RU fields within 2.5e-4 in the L2 norm and 1e-2 of the maximum (the face
cases), their totals -- the momentum balance -- within 5e-7 of the sum of magnitudes.
The momentum fields are bounded at 1e-3 (L2) and 2e-2 (max) accordingly, their totals
at 1e-5. The measured report is printed.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import helpers
from first_repo_gb300 import config, gen, pstep

pytestmark = pytest.mark.gpu

SIZED = os.path.join(helpers.GOLDEN, "reference_digests_box256.json")
FIELD_TOL = 1e-12
MEAN_RTOL = 1e-12
REL_TOL = 1e-5
RU_L2_TOL, RU_MAX_TOL = 1e-3, 2e-2  # momentum fields after one step from zero slip (see above)


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def sized_case(name):
    with open(SIZED) as f:
        for c in json.load(f)["cases"]:
            if c["name"] == name:
                return c
    raise KeyError(name)


def test_box256_fp64_dropin_matches_reference_every_step(built_cuda):
    gold = sized_case("box256_clustered")
    wl = config.WORKLOADS[gold["workload"]]
    case = gen.make_case(wl.n, wl.n_particles, wl.seed, wl.clustered, nblobs=wl.nblobs)
    for k, d in gold["inputs"].items():
        assert digest(case[k]) == d, f"input {k} differs from the one the reference ran"
    bp = config.box_params(wl.n, wl.n_particles, dp_over_dx=wl.dp_over_dx, mass_loading=wl.mass_loading)
    assert bp.step_config() == gold["step_config"]
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    fields = helpers.ghosted_fields(case)
    del case
    handles = {}
    for mode, flags in (("exact", pstep.TRACK_ORDER | pstep.REFERENCE_SUMS), ("fast", pstep.TRACK_ORDER)):
        g = pstep.ParticleStep(bp.step_config(), wl.n_particles, pstep.FP64, flags)
        g.load(*arrs)
        g.bind_velocity(*fields[:3])
        g.bind_temperature(fields[3])
        g.prime()
        handles[mode] = g
    exact, fast = handles["exact"], handles["fast"]
    recs = {r["tag"]: r for r in gold["records"]}

    def check(tag, where):
        rec = recs[tag]
        assert exact.np == rec["np"]
        for name in helpers.PART:
            assert digest(exact.array(name)) == rec["digests"][name], f"{where}: {name} differs from the reference"
        assert digest(exact.array("flag")) == rec["digests"]["flag"], f"{where}: particle order differs"
        for f, gname in helpers.FIELD_MAP.items():
            assert digest(exact.field(gname)) == rec["digests"][f], f"{where}: field {f} differs"
        want = float.fromhex(rec["mean_E"])
        assert abs(exact.energy_mean() - want) <= MEAN_RTOL * abs(want), f"{where}: energy mean"
        # default mode: states bit-identical, deposits within 1e-12 of max of the exact run's
        for name in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
            assert digest(fast.array(name)) == rec["digests"][name], f"{where}: fast-mode {name} differs"
        assert digest(fast.array("flag")) == rec["digests"]["flag"], f"{where}: fast-mode order differs"
        for gname in helpers.FIELD_MAP.values():
            assert helpers.max_rel_to_max(fast.field(gname), exact.field(gname)) <= FIELD_TOL, (where, gname)

    check(-1, "prime")
    for s in range(gold["steps"]):
        exact.run(1)
        fast.run(1)
        check(100000 + s, f"step {s}")
    for g in (exact, fast):
        rc, flags = g.check()
        assert rc == 0 and flags == 0, flags
        g.close()


def test_box512_mixed_fp32_error_against_fp64(built_cuda):
    pytest.importorskip("torch")
    import bench
    wl = config.WORKLOADS["box512_mixed"]
    n = wl.n_particles
    case = gen.make_case(wl.n, n, wl.seed, wl.clustered, nblobs=wl.nblobs)
    tau = wl.tau_p()
    bp = config.box_params(wl.n, n, dp_over_dx=wl.dp_over_dx, mass_loading=wl.mass_loading)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    fields = helpers.ghosted_fields(case)
    del case
    hs = []
    for form in (pstep.FP32, pstep.FP64):
        g = pstep.ParticleStep(bp.step_config(), n, form, 0)
        g.load(*arrs)
        g.set_tau_p(tau)
        g.bind_velocity(*fields[:3])
        g.bind_temperature(fields[3])
        g.prime()
        g.run(1)
        rc, flags = g.check()
        assert rc == 0, flags
        hs.append(g)
    rep = bench.fp32_error_report(hs[0], hs[1], bp.l, wl.n)
    print("box512_mixed FP32 vs FP64 after one step:", json.dumps(rep))
    bad = {k: rep[k] for k in ("position_cells_bulk", "velocity_rel_bulk", "temperature_rel_max",
                               "rhs_t_rel_to_max_bulk", "energy_mean_rel")
           if not rep[k] <= REL_TOL}
    bad.update({k: v for k, v in rep["fields"].items() if k in ("C", "RHS_Part_Temp") and not v <= REL_TOL})
    bad.update({"l2_" + k: v for k, v in rep["fields_l2"].items()
                if not v <= (REL_TOL if k in ("C", "RHS_Part_Temp") else RU_L2_TOL)})
    bad.update({k: v for k, v in rep["fields"].items() if k.startswith("RHS_RU") and not v <= RU_MAX_TOL})
    bad.update({k: v for k, v in rep["momentum_rel_to_abs"].items() if not v <= REL_TOL})
    # the face cases are few and stay small
    assert rep["position_cells_count"] <= rep["bulk_excludes"], rep["position_cells_count"]
    assert rep["position_cells_max"] <= 1e-3, rep["position_cells_max"]
    assert not bad, bad
    for g in hs:
        g.close()
