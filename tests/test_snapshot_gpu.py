"""Snapshot files and statistics of the device-resident particle state against the
oracle (whose restatements are pinned to the reference's Store_All, Load_All and
statistics in test_snapshot_oracle.py).

FP64 drop-in with the reference's particle order: Store_All's files are
byte-identical to the oracle's state written in the reference's format. FP32
form: the files hold what pstep_get_particle_array returns, and Load_All reads
them back. Maxima and minima are exact; the field mean is a fixed-order sum
(relative difference from the reference's loop order below 1e-13).
"""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen, pstep

pytestmark = pytest.mark.gpu

N, COUNT = 32, 20000
KEYS = ("x", "y", "z", "u", "v", "w", "T")


def _state(precision, flags, steps=2, seed=17):
    case = gen.make_case(N, COUNT, seed, True)
    bp = helpers.make_bp(N, COUNT)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    g = pstep.ParticleStep(bp.step_config(), COUNT, precision, flags)
    g.load(*arrs)
    g.bind_velocity(ux, uy, uz)
    g.bind_temperature(tf)
    g.prime()
    g.run(steps)
    o = None
    if precision == pstep.FP64:
        o = pyoracle.Oracle(bp.step_config(), COUNT)
        o.load(*arrs)
        o.prime(tf)
        o.run(steps, ux, uy, uz, tf)
    return g, o


def _check_field_stats(g):
    for name in ("C", "RHS_Part_Temp"):
        mx, mn, me = g.field_stats(name)
        rmx, rmn, rme = pyoracle.field_stats(g.field(name), N)
        assert (mx, mn) == (rmx, rmn), name
        assert abs(me - rme) <= 1e-13 * max(abs(rme), 1e-300), name


def test_fp64_store_all_is_the_reference_files(built_cuda, tmp_path):
    g, o = _state(pstep.FP64, pstep.TRACK_ORDER)
    g.store_all(str(tmp_path) + "/", 7)
    ref_dir = tmp_path / "oracle"
    ref_dir.mkdir()
    arrays = {k: o.array(k) for k in KEYS}
    arrays["flag"] = o.flag()
    pyoracle.store_all(str(ref_dir) + "/", 7, arrays)
    for name in pyoracle.SNAP_NAMES:
        assert (tmp_path / f"{name}_7.bin").read_bytes() == (ref_dir / f"{name}_7.bin").read_bytes(), name
    with pytest.raises(pstep.PstepError) as e:  # never overwrites (MPI_MODE_EXCL)
        g.store_all(str(tmp_path) + "/", 7)
    assert e.value.status == 11
    # statistics
    assert g.np_tot() == COUNT
    assert g.balance_index() == 1.0
    for k in KEYS:
        assert g.max(k) == pyoracle.array_max(o.array(k)), k
    # max u and max ug (grid::Statistics) come from the last stage's epilogue: no kernel
    # launch, equal to the oracle's (its ug is the gas velocity of the last stage)
    before = g.launches()
    assert g.max("u") == pyoracle.array_max(o.array("u"))
    assert g.max("ug") == pyoracle.array_max(o.array("ug"))
    assert g.launches() == before
    _check_field_stats(g)
    for name, key in (("C", "C"), ("RHS_Part_Temp", "E")):  # the oracle's fields, within the deposit bound
        mx, mn, me = g.field_stats(name)
        rmx, rmn, rme = pyoracle.field_stats(o.fields[key], N)
        scale = max(abs(rmx), abs(rmn))
        assert abs(mx - rmx) <= 1e-12 * scale and abs(mn - rmn) <= 1e-12 * scale, name
    ids = pyoracle.trajectory_ids(COUNT, 9) + [COUNT + 3]
    xyz, found = g.find_tags(ids)
    flag = o.flag()
    where = {int(f): i for i, f in enumerate(flag)}
    for i, t in enumerate(ids):
        assert found[i] == (t in where)
        if found[i]:
            assert [xyz[i, d] for d in range(3)] == [o.array(k)[where[t]] for k in ("x", "y", "z")]
    g.close()


def test_fp32_snapshot_round_trip_and_statistics(built_cuda, tmp_path):
    g, _ = _state(pstep.FP32, 0)
    d = str(tmp_path) + "/"
    g.store_all(d, 3)
    got = {k: g.array(k) for k in KEYS}
    got["flag"] = g.array("flag")
    for name, key in zip(pyoracle.SNAP_NAMES, pyoracle.SNAP_KEYS):
        dt = np.int32 if key == "flag" else np.float64
        assert np.array_equal(np.fromfile(tmp_path / f"{name}_3.bin", dtype=dt), got[key]), name
        (tmp_path / f"{name}_3.bin").rename(tmp_path / f"Restart_{name}.bin")
    assert g.np_tot() == COUNT
    for k in KEYS:
        assert g.max(k) == pyoracle.array_max(got[k]), k
    # after the step, the extrema come from its last deposit (no kernel launch) ...
    before = g.launches()
    _check_field_stats(g)
    assert g.launches() == before
    tags = [0, 11, COUNT - 1, -5, 11]  # an absent id and a repeated one
    xyz, found = g.find_tags(tags)
    where = {int(f): i for i, f in enumerate(got["flag"])}
    assert list(found) == [True, True, True, False, True]
    for i, t in enumerate(tags):
        if found[i]:
            assert [xyz[i, dd] for dd in range(3)] == [got[k][where[t]] for k in ("x", "y", "z")]
    bp = helpers.make_bp(N, COUNT)
    g2 = pstep.ParticleStep(bp.step_config(), COUNT, pstep.FP32, 0)
    g2.load_all(d, COUNT)
    assert np.array_equal(g2.array("flag"), got["flag"])
    for k in ("u", "v", "w"):
        assert np.array_equal(g2.array(k), got[k]), k
    assert np.max(np.abs(g2.array("T") - got["T"])) <= 1e-6 * np.max(np.abs(got["T"]))
    L, dx = bp.l, bp.l / N
    for k in ("x", "y", "z"):
        dd = (g2.array(k) - got[k] + L / 2) % L - L / 2
        assert np.max(np.abs(dd)) <= dx * 2.0 ** -22, k
    with pytest.raises(pstep.PstepError) as e:
        g2.load_all(d, COUNT, box=False)  # no _IO files
    assert e.value.status == 11
    # ... after a stage that is not a step's last, from a pass over the fields
    g.stage(0)
    before = g.launches()
    _check_field_stats(g)
    assert g.launches() > before
    g.close()
    g2.close()


def test_fp32_particle_maxima_fused_into_the_last_stage(built_cuda):
    """grid::Statistics' particle maxima (grid.cpp:726-727: max u and max ug) come out of
    the FP32 step's last stage without a pass over the particles (the FP64 form's are
    checked against the oracle above): pstep_max launches no
    kernel then, and equals the maximum of the arrays the step left (ug kept with
    PSTEP_KEEP_GAS here to compare), plain and with the learned correction. After an
    upload (no step yet) the call falls back to a pass."""
    from first_repo_gb300 import learn
    case = gen.make_case(N, COUNT, 23, True)
    bp = helpers.make_bp(N, COUNT)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    for corrected in (False, True):
        g = pstep.ParticleStep(bp.step_config(), COUNT, pstep.FP32, pstep.KEEP_GAS)
        g.load(*arrs)
        if corrected:
            g.set_correction(learn.load_model(), bp.mu0 / bp.rho0)
        g.bind_velocity(ux, uy, uz)
        g.bind_temperature(tf)
        g.prime()
        before = g.launches()
        assert g.max("u") == float(np.max(g.array("u")))  # after the upload: a pass
        assert g.launches() > before
        g.run(2)
        for name in ("u", "ug"):
            before = g.launches()
            got = g.max(name)
            assert g.launches() == before, name  # read from the last stage's epilogue
            assert got == float(np.max(g.array(name))), (corrected, name)
        assert g.max("v") == float(np.max(g.array("v")))  # other arrays: a pass
        g.close()
