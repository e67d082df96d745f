"""Per-particle properties (pstep_set_particle_props) and the kept gas values
(PSTEP_KEEP_GAS) of the FP32 form, against the FP64 oracle with the same
properties (oracle/pstep_oracle.c, pso_set_props; properties follow particle
ids there, storage order on the GPU).

The log-uniform tau_p in [0.01, 1] is the mixed-precision workload's particle
set; the reference has a scalar Tp only, so these cases are pinned by the
oracle port, whose scalar path is itself pinned to the reference."""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen, pstep
from test_fp32_gpu import REL_TOL, compare

pytestmark = pytest.mark.gpu


def _setup(n, count, seed, clustered=True):
    bp = helpers.make_bp(n, count)
    case = gen.make_case(n, count, seed, clustered)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    return bp, arrs, helpers.ghosted_fields(case)


def _run_both(bp, arrs, fields, count, props, steps, flags=0):
    cfg = bp.step_config()
    o = pyoracle.Oracle(cfg, count)
    o.load(*arrs)
    o.set_props(count, **{k: v for k, v in props.items() if k != "accel"},
                **({"ax": props["accel"][0], "ay": props["accel"][1], "az": props["accel"][2]}
                   if "accel" in props else {}))
    g = pstep.ParticleStep(cfg, count, pstep.FP32, flags)
    g.load(*arrs)
    g.set_props(**props)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    o.prime(fields[3])
    g.prime()
    errs = []
    for _ in range(steps):
        o.run(1, *fields)
        g.run(1)
        errs.append(compare(o, g, bp.l))
    return errs, g


def test_fp32_log_uniform_tau_p(built_cuda):
    n, count = 64, 1 << 15
    bp, arrs, fields = _setup(n, count, 2001)
    tau = gen.loguniform(2002, 0, count, 0.01, 1.0)
    errs, g = _run_both(bp, arrs, fields, count, {"tau_p": tau}, 3)
    for step, e in enumerate(errs):
        bad = {k: v for k, v in e.items() if not v <= REL_TOL}
        assert not bad, f"step {step}: {bad}"
    assert g.check()[0] == 0


def test_fp32_all_properties(built_cuda):
    n, count = 32, 20000
    bp, arrs, fields = _setup(n, count, 2011)
    rng = np.random.default_rng(2012)
    itth0 = bp.nu * np.pi * bp.dp * bp.k
    is0 = 1.0 / (bp.derived()["mp"] * bp.cvp)
    a0 = 0.25 * bp.epsilonp * np.pi * bp.dp ** 2 * bp.i0
    props = {
        "tau_p": np.exp(rng.uniform(np.log(0.02), np.log(0.5), count)),
        "mass_ratio": rng.uniform(0.2, 3.0, count),
        "itth": itth0 * rng.uniform(0.5, 2.0, count),
        "heat_is": is0 * rng.uniform(0.5, 2.0, count),
        "alpha": a0 * rng.uniform(0.0, 2.0, count),
        "accel": [rng.normal(0, 0.5, count) for _ in range(3)],
    }
    errs, g = _run_both(bp, arrs, fields, count, props, 2)
    for step, e in enumerate(errs):
        bad = {k: v for k, v in e.items() if not v <= REL_TOL}
        assert not bad, f"step {step}: {bad}"


def test_fp64_form_takes_tau_p_only(built_cuda):
    bp, arrs, fields = _setup(16, 500, 2021)
    g = pstep.ParticleStep(bp.step_config(), 500, pstep.FP64, 0)
    g.load(*arrs)
    g.set_props(tau_p=np.full(500, 0.1))
    with pytest.raises(pstep.PstepError) as e:
        g.set_props(mass_ratio=np.ones(500))
    assert e.value.status == 2
    with pytest.raises(pstep.PstepError) as e:
        g.array("ug")
    assert e.value.status == 2




def test_keep_gas_values_are_the_interpolated_fields(built_cuda):
    n, count = 32, 5000
    bp, arrs, fields = _setup(n, count, 2031)
    g = pstep.ParticleStep(bp.step_config(), count, pstep.FP32, pstep.KEEP_GAS)
    g.load(*arrs)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    g.stage(0)
    idx = n / bp.l
    xi = [g.array(k) * idx for k in ("x_int", "y_int", "z_int")]
    xn = [g.array(k) * idx for k in ("x_new", "y_new", "z_new")]
    ux, uy, uz, tf = fields
    t = [np.floor(a).astype(int) for a in xi]
    fr = [a - b for a, b in zip(xi, t)]
    i, j, k = (b + 1 for b in t)
    ug = fr[0] * ux[k, j, i + 1] + (1 - fr[0]) * ux[k, j, i]
    vg = fr[1] * uy[k, j + 1, i] + (1 - fr[1]) * uy[k, j, i]
    wg = fr[2] * uz[k + 1, j, i] + (1 - fr[2]) * uz[k, j, i]
    r = [np.floor(a + 0.5).astype(int) for a in xn]
    tx, ty, tz = (a - b + 0.5 for a, b in zip(xn, r))
    ni, nj, nk = (b + 1 for b in r)
    tg = (tx * ty * tz * tf[nk, nj, ni] + (1 - tx) * ty * tz * tf[nk, nj, ni - 1] +
          tx * (1 - ty) * tz * tf[nk, nj - 1, ni] + tx * ty * (1 - tz) * tf[nk - 1, nj, ni] +
          (1 - tx) * (1 - ty) * tz * tf[nk, nj - 1, ni - 1] + (1 - tx) * ty * (1 - tz) * tf[nk - 1, nj, ni - 1] +
          tx * (1 - ty) * (1 - tz) * tf[nk - 1, nj - 1, ni] + (1 - tx) * (1 - ty) * (1 - tz) * tf[nk - 1, nj - 1, ni - 1])
    for name, ref in (("ug", ug), ("vg", vg), ("wg", wg)):
        assert helpers.max_rel_to_max(g.array(name), ref) <= 2e-6, name
    assert np.max(np.abs(g.array("Tg") - tg)) <= 2e-6 * np.max(np.abs(tg))
