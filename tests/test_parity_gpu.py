"""GPU parity: the FP64 drop-in through the C ABI against the oracle.

With PSTEP_TRACK_ORDER | PSTEP_REFERENCE_SUMS the device path must reproduce
the reference exactly: every particle array in the reference's order (the
permutation Send_Recv leaves), the flags, and all five deposited fields
including their ghost layers, bit for bit, at every call. The interior mean of
RHS_Part_Temp is a different summation order (a fixed tree): relative
tolerance 1e-12. With the fast deposit (no REFERENCE_SUMS) particle states and
order stay bit-exact and the deposits match to 1e-12 of the field's maximum
(a different, fixed summation order).
"""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen, pstep

pytestmark = pytest.mark.gpu

FIELDS = ["C", "Ax", "Ay", "Az", "E"]
MEAN_RTOL = 1e-12
DEPOSIT_TOL = 1e-12  # max|gpu - oracle| / max|oracle| without order tracking


EXACT = pstep.TRACK_ORDER | pstep.REFERENCE_SUMS


def setup_pair(cdef, flags=EXACT):
    case = gen.make_case(cdef["n"], cdef["count"], cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(cdef["n"], cdef["count"], cdef.get("extra"))
    cfg = bp.step_config()
    o = pyoracle.Oracle(cfg, cdef["count"])
    o.load(case["x"], case["y"], case["z"], case["u"], case["v"], case["w"], case["t"], case["flag"])
    g = pstep.ParticleStep(cfg, cdef["count"], pstep.FP64, flags)
    g.load(*(np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")))
    fields = helpers.ghosted_fields(case)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    return case, o, g, fields


def compare_exact(o, g, where, exact_fields=True):
    for name in helpers.PART:
        a, b = g.array(name), o.array(name)
        assert helpers.bits_equal(a, b), f"{where}: {name} differs (max abs {np.max(np.abs(a - b))})"
    assert np.array_equal(g.array("flag"), o.flag()), f"{where}: particle order differs"
    for f in FIELDS:
        a, b = g.field(helpers.FIELD_MAP[f]), o.fields[f]
        if exact_fields:
            assert helpers.bits_equal(a, b), f"{where}: field {f} differs (max rel {helpers.max_rel_to_max(a, b):.3e})"
        else:
            assert helpers.max_rel_to_max(a, b) <= DEPOSIT_TOL, f"{where}: field {f} {helpers.max_rel_to_max(a, b):.3e}"
    me, mo = g.energy_mean(), o.mean(o.fields["E"])
    assert abs(me - mo) <= MEAN_RTOL * max(abs(mo), 1e-300), f"{where}: energy mean {me} vs {mo}"
    check_momentum_sums(o, g, where)


def check_momentum_sums(o, g, where, rtol=MEAN_RTOL):
    """The per-stage momentum balance (pstep_momentum_sums): interior sums of the three
    deposited momentum fields, within rtol of the sum of their magnitudes (the sums
    cancel, so a relative bound on the sum itself would be meaningless)."""
    got = g.momentum_sums()
    for d, f in enumerate(("Ax", "Ay", "Az")):
        interior = o.fields[f][1:-1, 1:-1, 1:-1]
        want, scale = float(np.sum(interior)), float(np.sum(np.abs(interior)))
        assert abs(got[d] - want) <= rtol * max(scale, 1e-300), f"{where}: momentum sum {f} {got[d]} vs {want}"


@pytest.mark.parametrize("name", ["box12_small", "box16_twc_off_gravity", "box32_clustered", "box64_uniform"])
def test_fp64_bit_exact_in_reference_order(built_cuda, name):
    cdef = helpers.golden_case(name)
    _, o, g, (ux, uy, uz, tf) = setup_pair(cdef)
    o.prime(tf)
    g.prime()
    compare_exact(o, g, "prime")
    for s in range(cdef["steps"]):
        for k in range(4):
            o.stage(k, ux, uy, uz, tf)
            g.stage(k)
            compare_exact(o, g, f"step {s} stage {k}")
            o.end_stage()
            g.end_stage()
        o.end_step()
        g.end_step()
    compare_exact(o, g, "end")
    rc, flags = g.check()
    assert rc == 0 and flags == 0


@pytest.mark.parametrize("name", ["box16_twc_off_gravity", "box32_clustered", "box64_uniform"])
def test_fp64_fast_deposit_reference_order(built_cuda, name):
    """Default drop-in mode: bit-exact states and order, deposits to 1e-12 of max."""
    cdef = helpers.golden_case(name)
    _, o, g, (ux, uy, uz, tf) = setup_pair(cdef, flags=pstep.TRACK_ORDER)
    o.prime(tf)
    g.prime()
    compare_exact(o, g, "prime", exact_fields=False)
    for s in range(cdef["steps"]):
        for k in range(4):
            o.stage(k, ux, uy, uz, tf)
            g.stage(k)
            compare_exact(o, g, f"step {s} stage {k}", exact_fields=False)
            o.end_stage()
            g.end_stage()
        o.end_step()
        g.end_step()


def test_fp64_split_calls_and_late_temperature(built_cuda):
    """The three-call stage (interp_advance_deposit, wrap, stage_temp) with the
    temperature bound after the wrap, as the reference forms it (grid.cpp:676)."""
    cdef = helpers.golden_case("box32_clustered")
    _, o, g, (ux, uy, uz, tf) = setup_pair(cdef)
    tf2 = tf * 1.01
    o.prime(tf)
    g.prime()
    for k in range(4):
        o.stage(k, ux, uy, uz, tf2)
        g.bind_temperature(tf)
        g.interp_advance_deposit(k)
        g.wrap()
        g.bind_temperature(tf2)
        g.stage_temp()
        compare_exact(o, g, f"stage {k}")
        o.end_stage()
        g.end_stage()
    o.end_step()
    g.end_step()


def test_fp64_without_order_tracking(built_cuda):
    cdef = helpers.golden_case("box32_clustered")
    _, o, g, (ux, uy, uz, tf) = setup_pair(cdef, flags=0)
    o.prime(tf)
    g.prime()
    o.run(cdef["steps"], ux, uy, uz, tf)
    g.run(cdef["steps"])
    fo, fg = o.flag(), g.array("flag")
    io, ig = np.argsort(fo), np.argsort(fg)
    assert np.array_equal(fo[io], fg[ig])
    for name in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
        assert helpers.bits_equal(g.array(name)[ig], o.array(name)[io]), name
    for f in FIELDS:
        a, b = g.field(helpers.FIELD_MAP[f]), o.fields[f]
        assert helpers.max_rel_to_max(a, b) <= DEPOSIT_TOL, f


def test_fp64_deterministic(built_cuda):
    cdef = helpers.golden_case("box32_clustered")
    outs = []
    for _ in range(2):
        _, _, g, _ = setup_pair(cdef, flags=0)
        g.prime()
        g.run(2)
        outs.append([g.field(helpers.FIELD_MAP[f]).copy() for f in FIELDS] + [g.array("x")])
        g.close()
    for a, b in zip(*outs):
        assert helpers.bits_equal(a, b)


def test_state_machine_errors(built_cuda):
    cdef = helpers.golden_case("box12_small")
    _, _, g, _ = setup_pair(cdef)
    with pytest.raises(pstep.PstepError) as e:
        g.stage(0)  # before prime
    assert e.value.status == 4
    g.prime()
    with pytest.raises(pstep.PstepError):
        g.stage(1)  # out of sequence
    g.stage(0)
    with pytest.raises(pstep.PstepError):
        g.stage(1)  # end_stage missing
    g.end_stage()
    with pytest.raises(pstep.PstepError):
        g.end_step()  # only after stage 3


def test_capacity_and_input_checks(built_cuda):
    cdef = helpers.golden_case("box12_small")
    case = gen.make_case(cdef["n"], cdef["count"], cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(cdef["n"], cdef["count"])
    g = pstep.ParticleStep(bp.step_config(), 10, pstep.FP64, pstep.TRACK_ORDER | pstep.CHECK_INPUTS)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    with pytest.raises(pstep.PstepError) as e:
        g.load(*arrs)
    assert e.value.status == 3
    small = [a[:10].copy() for a in arrs]
    small[0][3] = np.nan
    with pytest.raises(pstep.PstepError) as e:
        g.load(*small)
    assert e.value.status == 6
    small[0][3] = bp.l * 1.5
    with pytest.raises(pstep.PstepError) as e:
        g.load(*small)
    assert e.value.status == 7
