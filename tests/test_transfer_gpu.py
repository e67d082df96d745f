"""Host upload and read-back of the FP32 form through its staged, chunked copies.

Host arrays move in chunks of 2^22 particles through two device staging slots
(copy of one chunk overlapping the conversion of the other). A round trip of
more particles than two chunks checks every chunk lands at its own offset:
velocities come back as their float32 rounding, temperatures as the float32
rounding of T - T_ref plus T_ref, positions within the float32 resolution of the
in-cell offset, ids exactly.
"""
import numpy as np
import pytest

import helpers
from first_repo_gb300 import pstep

pytestmark = pytest.mark.gpu

STAGE_CHUNK = 1 << 22


def test_fp32_host_round_trip_over_several_chunks(built_cuda):
    n, count = 64, 2 * STAGE_CHUNK + 123457  # three chunks, the last partial
    bp = helpers.make_bp(n, count)
    L = bp.l
    rng = np.random.default_rng(7)
    x, y, z = (rng.uniform(0.0, L, count) for _ in range(3))
    u, v, w = (rng.normal(0.0, 1.0, count) for _ in range(3))
    t = rng.uniform(0.5, 2.0, count)
    flag = rng.permutation(count).astype(np.int32)
    g = pstep.ParticleStep(bp.step_config(), count, pstep.FP32, 0)
    g.load(x, y, z, u, v, w, t, flag)
    assert np.array_equal(g.array("flag"), flag)
    for name, a in (("u", u), ("v", v), ("w", w)):
        assert np.array_equal(g.array(name), a.astype(np.float32).astype(np.float64)), name
    tref = float(np.float32(t[0]))
    assert np.array_equal(g.array("T"), (t - tref).astype(np.float32).astype(np.float64) + tref)
    dx = L / n
    for name, a in (("x", x), ("y", y), ("z", z)):
        got = g.array(name)
        d = (got - a + L / 2) % L - L / 2
        assert np.max(np.abs(d)) <= dx * 2.0 ** -23, name
    g.close()


def test_fp32_back_to_back_host_uploads(built_cuda):
    """Two uploads in a row (the second's copies must wait for the first's conversions
    still running on the handle's stream), then a read-back: the second population."""
    n, count = 64, STAGE_CHUNK + 77
    bp = helpers.make_bp(n, count)
    L = bp.l
    rng = np.random.default_rng(11)
    pops = []
    for _ in range(2):
        x, y, z = (rng.uniform(0.0, L, count) for _ in range(3))
        u, v, w = (rng.normal(0.0, 1.0, count) for _ in range(3))
        t = rng.uniform(0.5, 2.0, count)
        flag = rng.permutation(count).astype(np.int32)
        pops.append((x, y, z, u, v, w, t, flag))
    g = pstep.ParticleStep(bp.step_config(), count, pstep.FP32, 0)
    for pop in pops:
        g.load(*pop)
    x, y, z, u, v, w, t, flag = pops[1]
    assert np.array_equal(g.array("flag"), flag)
    assert np.array_equal(g.array("u"), u.astype(np.float32).astype(np.float64))
    dx = L / n
    d = (g.array("x") - x + L / 2) % L - L / 2
    assert np.max(np.abs(d)) <= dx * 2.0 ** -23
    g.close()


@pytest.mark.parametrize("form", [pstep.FP32, pstep.FP64])
def test_download_particles_equals_the_array_reads(built_cuda, form):
    """pstep_download_particles (one pass over every chunk, all arrays) returns exactly what
    pstep_get_particle_array returns for PSTEP_X .. PSTEP_T and PSTEP_FLAG, into host and
    into device memory, after a step (over three staging chunks for the FP32 form)."""
    torch = pytest.importorskip("torch")
    n = 64
    count = 2 * STAGE_CHUNK + 4321 if form == pstep.FP32 else 50000
    bp = helpers.make_bp(n, count)
    rng = np.random.default_rng(13)
    x, y, z = (rng.uniform(0.0, bp.l, count) for _ in range(3))
    u, v, w = (rng.normal(0.0, 1.0, count) for _ in range(3))
    t = rng.uniform(0.9, 1.1, count)
    flag = rng.permutation(count).astype(np.int32)
    g = pstep.ParticleStep(bp.step_config(), count, form, pstep.TRACK_ORDER if form == pstep.FP64 else 0)
    g.load(x, y, z, u, v, w, t, flag)
    zf = np.zeros((n + 2,) * 3)
    g.bind_velocity(zf, zf, zf)
    g.bind_temperature(zf + 1.0)
    g.prime()
    g.run(1)
    names = ["x", "y", "z", "u", "v", "w", "T", "flag"]
    want = [g.array(k) for k in names]
    host = [np.empty(count, dtype=np.int32 if k == "flag" else np.float64) for k in names]
    g.download(*host)
    for k, a, b in zip(names, host, want):
        assert helpers.bits_equal(a, b), k
    dev = [torch.empty(count, dtype=torch.int32 if k == "flag" else torch.float64, device="cuda") for k in names]
    g.download(*dev)
    for k, a, b in zip(names, dev, want):
        assert helpers.bits_equal(a.cpu().numpy(), b), k
    g.close()
