"""The oracle (C restatement of the reference's particle step) against the
reference itself: bit-for-bit, per call of the step.

 - against the golden digests in tests/golden (made by tests/golden/make_golden.py
   from the reference's own sources), everywhere;
 - against the reference built from source (oracle/_ref), where the sources exist.
"""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen

STATE = ["x", "y", "z", "x_int", "y_int", "z_int", "x_new", "y_new", "z_new", "x_np1", "y_np1", "z_np1",
         "u", "v", "w", "u_int", "v_int", "w_int", "u_new", "v_new", "w_new", "u_np1", "v_np1", "w_np1",
         "T", "T_int", "T_new", "T_np1", "RHS_T"]
FIELDS = ["C", "Ax", "Ay", "Az", "E"]


def port_records(case_def, case):
    """Drive the port exactly as the reference harness does; digest every record."""
    bp = helpers.make_bp(case_def["n"], case_def["count"], case_def["extra"])
    o = pyoracle.Oracle(bp.step_config(), case_def["count"])
    o.load(case["x"], case["y"], case["z"], case["u"], case["v"], case["w"], case["t"], case["flag"])
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    out = []

    def rec(tag):
        d = {k: helpers.digest(o.array(k)) for k in STATE}
        d["flag"] = helpers.digest(o.flag())
        for f in FIELDS:
            d[f] = helpers.digest(o.fields[f])
        out.append({"tag": tag, "np": o.np, "mean_E": o.mean(o.fields["E"]).hex(), "digests": d})

    o.prime(tf)
    rec(-1)
    for s in range(case_def["steps"]):
        for k in range(4):
            o.stage(k, ux, uy, uz, tf)
            rec(s * 4 + k)
            o.end_stage()
        o.end_step()
    rec(1000000 + case_def["steps"])
    assert o.edge_hits == 0
    return out


@pytest.mark.parametrize("name", ["box12_small", "box16_twc_off_gravity", "box32_clustered", "box64_uniform"])
def test_port_matches_reference_golden(built, name):
    cdef = helpers.golden_case(name)
    case = gen.make_case(cdef["n"], cdef["count"], cdef["seed"], cdef["clustered"])
    # the generator reproduces the inputs the fixtures were made from (x86 and Arm alike)
    for k, dg in cdef["inputs"].items():
        assert helpers.digest(case[k]) == dg, f"generated input {k} differs from the fixture"
    got = port_records(cdef, case)
    assert len(got) == len(cdef["records"])
    for g, r in zip(got, cdef["records"]):
        assert g["tag"] == r["tag"] and g["np"] == r["np"]
        bad = [k for k, v in r["digests"].items() if g["digests"][k] != v]
        assert not bad, f"record {r['tag']}: arrays differ from the reference: {bad}"
        assert g["mean_E"] == r["mean_E"]


def test_port_final_state_matches_fixture(built):
    cdef = helpers.golden_case("box12_small")
    case = gen.make_case(cdef["n"], cdef["count"], cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(cdef["n"], cdef["count"], cdef["extra"])
    o = pyoracle.Oracle(bp.step_config(), cdef["count"])
    o.load(case["x"], case["y"], case["z"], case["u"], case["v"], case["w"], case["t"], case["flag"])
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    o.prime(tf)
    o.run(cdef["steps"], ux, uy, uz, tf)
    fx = np.load(helpers.GOLDEN + "/box12_small_final.npz")
    for k in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
        assert helpers.bits_equal(o.array(k), fx[k]), k
    assert np.array_equal(o.flag(), fx["flag"])
    for f in FIELDS:
        assert helpers.bits_equal(o.fields[f], fx[f]), f


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("n,count,steps,clustered,seed", [(8, 700, 4, True, 21), (20, 5000, 2, False, 22)])
def test_port_matches_reference_binary(built, n, count, steps, clustered, seed):
    """Fresh cases (not in the fixtures) through the reference built from source."""
    bp = helpers.make_bp(n, count)
    case = gen.make_case(n, count, seed, clustered)
    recs, _ = pyoracle.run_ref(bp, case, steps, dump_all=True)
    cdef = {"n": n, "count": count, "extra": {}, "steps": steps}
    got = port_records(cdef, case)
    for g, r in zip(got, recs):
        for k in STATE + ["flag"] + FIELDS:
            assert g["digests"][k] == helpers.digest(r[k]), (r["tag"], k)


def test_known_answer_uniform_temperature(built):
    """Uniform gas T and zero gas velocity: T_p follows RK4 of dT/dt = (Tg - T)/tau_T + Q
    and u_p of du/dt = -u/tau_p; the deposits conserve particle count, momentum and
    energy (known answers from the mathematics)."""
    n, count = 8, 64
    bp = helpers.make_bp(n, count)
    cfg = bp.step_config()
    g = n + 2
    zero = np.zeros((g, g, g))
    tgas = np.full((g, g, g), 1.3)
    rng = np.random.default_rng(0)
    x, y, z = (rng.uniform(0.1, 0.9, count) * bp.l for _ in range(3))
    u0 = rng.normal(size=count)
    o = pyoracle.Oracle(cfg, count)
    o.load(x, y, z, u0, np.zeros(count), np.zeros(count), np.ones(count), np.arange(count, dtype=np.int32))
    o.prime(tgas)
    o.run(1, zero, zero, zero, tgas)
    dt = bp.dt
    from first_repo_gb300 import config
    tau_t = config.tau_t(bp)
    q = config.heating_rate(bp)
    tp = cfg["tp"]

    def rk4(f, y0):
        k1 = f(y0); k2 = f(y0 + dt / 2 * k1); k3 = f(y0 + dt / 2 * k2); k4 = f(y0 + dt * k3)
        return y0 + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)

    t_expect = rk4(lambda T: (1.3 - T) / tau_t + q, 1.0)
    u_expect = rk4(lambda u: -u / tp, u0)
    flag = o.flag()
    assert np.allclose(o.array("T"), t_expect, rtol=1e-12, atol=0)
    assert np.allclose(o.array("u")[np.argsort(flag)], u_expect, rtol=1e-12, atol=1e-15)
    # deposited concentration sums to the particle count; energy to the sum of RHS_T
    c = o.fields["C"][1:-1, 1:-1, 1:-1]
    assert abs(c.sum() - count) < 1e-10
    e = o.fields["E"][1:-1, 1:-1, 1:-1]
    assert abs(e.sum() - o.array("RHS_T").sum()) < 1e-12 * max(1.0, abs(e).sum())
    # deposited momentum sums to the sum of RHS_u per component (the face weights of a
    # particle add to one: x_l + (1 - x_l), particle.cpp:498-524)
    for comp, key in (("Ax", "RHS_u"), ("Ay", "RHS_v"), ("Az", "RHS_w")):
        a, r = o.fields[comp][1:-1, 1:-1, 1:-1], o.array(key)
        assert abs(a.sum() - r.sum()) < 1e-12 * max(1.0, np.abs(r).sum()), comp
    assert np.abs(o.array("RHS_u")).sum() > 0
