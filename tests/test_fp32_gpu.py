"""The FP32 mixed form against the FP64 oracle.

Bound (uncorrected FP32 step vs the FP64 oracle): relative error <= 1e-5,
measured norm-wise per quantity as max|fp32 - fp64| / max|fp64| (positions as
max|dx| / L), after every step; and per particle, for every particle: position
within 1e-6 cells, velocity vector within 2e-6 and temperature within 1e-8 of
their own size. The concentration's ghost layer is excluded:
the reference leaves unfolded partial sums there (no refresh), the FP32 form
periodic copies. Deposits are exact 64-bit fixed-point sums, so two runs give
bit-identical fields and per-particle states (compared by particle id; the
storage order inside a cell is not fixed in this form).
"""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen, pstep

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
# per-particle bounds: positions in cells, velocity vectors and temperatures relative to
# their own size
PER_PARTICLE_TOL = {"position_cells": 1e-6, "velocity_rel": 2e-6, "temperature_rel": 1e-8}
FIELDS = ["C", "Ax", "Ay", "Az", "E"]


def run_pair(name, steps=None):
    cdef = helpers.golden_case(name)
    steps = steps or cdef["steps"]
    case = gen.make_case(cdef["n"], cdef["count"], cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(cdef["n"], cdef["count"], cdef.get("extra"))
    cfg = bp.step_config()
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    o = pyoracle.Oracle(cfg, cdef["count"])
    o.load(*arrs)
    g = pstep.ParticleStep(cfg, cdef["count"], pstep.FP32, 0)
    g.load(*arrs)
    g.bind_velocity(ux, uy, uz)
    g.bind_temperature(tf)
    o.prime(tf)
    g.prime()
    errs, parts = [], []
    for _ in range(steps):
        o.run(1, ux, uy, uz, tf)
        g.run(1)
        errs.append(compare(o, g, bp.l))
        parts.append(per_particle(o, g, bp.l, cdef["n"]))
    return errs, g, parts


def per_particle(o, g, L, n):
    """Per-particle errors of the FP32 form against the oracle: positions in cells (the
    largest component), velocity vectors and temperatures relative to their own size."""
    fo, fg = o.flag(), g.array("flag")
    io, ig = np.argsort(fo), np.argsort(fg)
    dpos = np.stack([(g.array(k)[ig] - o.array(k)[io] + L / 2) % L - L / 2 for k in ("x", "y", "z")], 1)
    cells = np.max(np.abs(dpos), 1) * n / L
    vo = np.stack([o.array(k)[io] for k in ("u", "v", "w")], 1)
    vg = np.stack([g.array(k)[ig] for k in ("u", "v", "w")], 1)
    vel = np.linalg.norm(vg - vo, axis=1) / np.maximum(np.linalg.norm(vo, axis=1), 1e-300)
    to = o.array("T")[io]
    temp = np.abs(g.array("T")[ig] - to) / np.maximum(np.abs(to), 1e-300)
    return {"position_cells": cells, "velocity_rel": vel, "temperature_rel": temp}


def compare(o, g, L):
    fo, fg = o.flag(), g.array("flag")
    io, ig = np.argsort(fo), np.argsort(fg)
    assert np.array_equal(fo[io], fg[ig])
    out = {}
    for k in ("x", "y", "z"):
        d = g.array(k)[ig] - o.array(k)[io]
        d = (d + L / 2) % L - L / 2  # periodic images
        out[k] = float(np.max(np.abs(d)) / L)
    for k in ("u", "v", "w", "T", "RHS_T"):
        a, b = g.array(k)[ig], o.array(k)[io]
        out[k] = helpers.max_rel_to_max(a, b)
    for f in FIELDS:
        a, b = g.field(helpers.FIELD_MAP[f]), o.fields[f]
        if f == "C":
            a, b = a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]
        out[f] = helpers.max_rel_to_max(a, b)
    me, mo = g.energy_mean(), o.mean(o.fields["E"])
    out["mean_E"] = abs(me - mo) / max(abs(mo), 1e-300)
    # the momentum balance against the oracle's deposits, relative to the sum of magnitudes,
    # and against the form's own deposited fields (the exact integer totals, rounded once)
    mom = g.momentum_sums()
    for d, f in enumerate(("Ax", "Ay", "Az")):
        ref = o.fields[f][1:-1, 1:-1, 1:-1]
        own = g.field(helpers.FIELD_MAP[f])[1:-1, 1:-1, 1:-1]
        scale = max(float(np.sum(np.abs(ref))), 1e-300)
        out["mom_" + f] = abs(mom[d] - float(np.sum(ref))) / scale
        assert abs(mom[d] - float(np.sum(own))) <= 1e-12 * scale
    return out


@pytest.mark.parametrize("name", ["box16_twc_off_gravity", "box32_clustered", "box64_uniform"])
def test_fp32_error_against_fp64_oracle(built_cuda, name):
    errs, g, parts = run_pair(name, steps=3)
    for step, e in enumerate(errs):
        bad = {k: v for k, v in e.items() if not v <= REL_TOL}
        assert not bad, f"step {step}: {bad}"
    report = [{k: {"max": float(v.max()), "p99.9": float(np.quantile(v, 0.999))} for k, v in p.items()}
              for p in parts]
    print(name, "per-particle FP32 error after each step:", report)
    # per particle, every particle: measured after 3 steps 2.9e-7 cells, 4.9e-7 and 8.8e-10
    # (no particle of these cases sits within fp32 resolution of a cell face)
    for step, p in enumerate(parts):
        for k, tol in PER_PARTICLE_TOL.items():
            assert p[k].max() <= tol, (step, k, float(p[k].max()))
    rc, flags = g.check()
    assert rc == 0, flags


def test_fp32_deterministic(built_cuda):
    cdef = helpers.golden_case("box32_clustered")
    case = gen.make_case(cdef["n"], cdef["count"], cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(cdef["n"], cdef["count"])
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    outs = []
    for _ in range(2):
        g = pstep.ParticleStep(bp.step_config(), cdef["count"], pstep.FP32, 0)
        g.load(*arrs)
        g.bind_velocity(ux, uy, uz)
        g.bind_temperature(tf)
        g.prime()
        g.run(2)
        order = np.argsort(g.array("flag"))
        outs.append([g.field(helpers.FIELD_MAP[f]).copy() for f in FIELDS] +
                    [g.array(k)[order] for k in ("x", "y", "z", "u", "v", "w", "T", "RHS_T")])
        g.close()
    for a, b in zip(*outs):
        assert helpers.bits_equal(a, b)


def test_fp32_rejects_unsupported_grid(built_cuda):
    bp = helpers.make_bp(12, 100)
    with pytest.raises(pstep.PstepError) as e:
        pstep.ParticleStep(bp.step_config(), 100, pstep.FP32, 0)
    assert e.value.status == 2


def window_max(x, y, z, n, L, br):
    """most particles in one deposit brick's source window (the br^3 brick and two
    cells around it, periodic)"""
    idx = [np.floor(a / (L / n)).astype(np.int64) for a in (x, y, z)]
    cnt = np.bincount((idx[2] * n + idx[1]) * n + idx[0], minlength=n ** 3).reshape(n, n, n)
    best = 0
    for bz in range(0, n, br):
        for by in range(0, n, br):
            for bx in range(0, n, br):
                r = [np.arange(b - 2, b + br + 2) % n for b in (bz, by, bx)]
                best = max(best, int(cnt[np.ix_(*r)].sum()))
    return best


# the deposit splits a brick into slices of at most this many window particles
CHUNK_MAX = 1 << 16


@pytest.mark.parametrize("n,count,br", [(32, 300000, 16), (24, 200000, 8)])
def test_fp32_dense_blob_split_bricks(built_cuda, n, count, br):
    """A single tight blob puts more particles into one deposit brick's source window
    than one work item takes, so the deposit splits the brick into slices combined in
    global memory; still within the bound and bit-identical across runs. Both brick
    edges (16 where every side is a multiple of 16 and at least 32, else 8)."""
    bp = helpers.make_bp(n, count)
    L = bp.l
    ux, uy, uz = gen.velocity(n, 41)
    tf = gen.temperature(n, 42)
    x, y, z = gen.positions(n, L, 43, count, True, nblobs=1, sigma_cells=1.5)
    assert window_max(x, y, z, n, L, br) > CHUNK_MAX
    u, v, w = gen.interp_velocity(n, L, x, y, z, ux, uy, uz)
    t = np.ones(count)
    flag = np.arange(count, dtype=np.int32)
    arrs = [np.ascontiguousarray(a) for a in (x, y, z, u, v, w, t, flag)]
    fields = [gen.ghost(a) for a in (ux, uy, uz, tf)]
    o = pyoracle.Oracle(bp.step_config(), count)
    o.load(*arrs)
    o.prime(fields[3])
    o.run(2, *fields)
    outs = []
    for _ in range(2):
        g = pstep.ParticleStep(bp.step_config(), count, pstep.FP32, 0)
        g.load(*arrs)
        g.bind_velocity(*fields[:3])
        g.bind_temperature(fields[3])
        g.prime()
        g.run(2)
        e = compare(o, g, L)
        bad = {k: v for k, v in e.items() if not v <= REL_TOL}
        assert not bad, bad
        outs.append([g.field(helpers.FIELD_MAP[f]).copy() for f in FIELDS])
        g.close()
    for a, b in zip(*outs):
        assert helpers.bits_equal(a, b)


def test_fp32_empty_population(built_cuda):
    """No particles: the step runs, every deposited field is zero, the arrays are empty."""
    n = 16
    bp = helpers.make_bp(n, 100)
    ux, uy, uz = gen.velocity(n, 41)
    tf = gen.temperature(n, 42)
    fields = [gen.ghost(a) for a in (ux, uy, uz, tf)]
    g = pstep.ParticleStep(bp.step_config(), 16, pstep.FP32, 0)
    empty = np.zeros(0)
    g.load(empty, empty, empty, empty, empty, empty, empty, np.zeros(0, dtype=np.int32))
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    g.run(2)
    rc, flags = g.check()
    assert rc == 0, flags
    for f in FIELDS:
        assert not np.any(g.field(helpers.FIELD_MAP[f])), f
    assert g.array("x").size == 0 and g.array("flag").size == 0
    assert g.np_tot() == 0 and g.max("u") == -1e9
    g.close()


def test_fp32_prime_keeps_an_upload_already_in_cell_order(built_cuda):
    """A population uploaded in the order a step left it (a host round trip) is not
    permuted again: the prime finds the storage in cell order and only rebuilds the
    cell-start table (fewer launches). The following steps equal, by id and bit for bit,
    those of the same population uploaded in a shuffled order (fully sorted by the prime)."""
    cdef = helpers.golden_case("box32_clustered")
    n = cdef["count"]
    case = gen.make_case(cdef["n"], n, cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(cdef["n"], n)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    ux, uy, uz, tf = helpers.ghosted_fields(case)

    def start(a):
        g = pstep.ParticleStep(bp.step_config(), n, pstep.FP32, 0)
        g.load(*a)
        g.bind_velocity(ux, uy, uz)
        g.bind_temperature(tf)
        return g

    g = start(arrs)
    g.prime()
    g.run(1)
    back = [np.empty(n) for _ in range(7)] + [np.empty(n, dtype=np.int32)]
    g.download(*back)  # storage order: the cell order the step's sort left
    g.close()
    # (the first particle stays first: the FP32 form keeps temperatures as offsets from the
    # first uploaded particle's, so both handles get the same reference temperature)
    perm = np.concatenate([[0], 1 + np.random.default_rng(5).permutation(n - 1)])
    shuffled = [np.ascontiguousarray(a[perm]) for a in back]
    a, b = start(back), start(shuffled)
    l0 = a.launches()
    a.prime()
    la = a.launches() - l0
    l0 = b.launches()
    b.prime()
    lb = b.launches() - l0
    assert la < lb, (la, lb)
    a.run(2)
    b.run(2)
    ia, ib = np.argsort(a.array("flag")), np.argsort(b.array("flag"))
    for name in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
        assert helpers.bits_equal(a.array(name)[ia], b.array(name)[ib]), name
    for f in FIELDS:
        assert helpers.bits_equal(a.field(helpers.FIELD_MAP[f]), b.field(helpers.FIELD_MAP[f])), f
    a.close()
    b.close()
