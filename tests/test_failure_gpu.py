"""Device-side failure reporting, injected from the host: nothing faults, traps or
hangs the GPU, and the handle stays usable afterwards.

- PSTEP_ERR_MOVE: particles uploaded with a velocity that carries them three cells in
  the first stage (the FP32 form's deposit windows hold moves of at most one cell per
  stage). The check word reports it and the next, well-formed population steps cleanly.
- PSTEP_ERR_TIMEOUT: the fused inference's first tensor-core completion wait polls a
  barrier that nothing signals (pstep_set_wait_limit with idle_first), so it runs out
  after a short bound as a lost completion would. The kernel drains its own MMA,
  frees its tensor memory and returns; the check word reports the timeout, and the
  same handle then runs a step whose results equal a fresh handle's bit for bit (no
  tensor memory was left allocated, or the next allocation would wait).
"""
import numpy as np
import pytest

import helpers
from first_repo_gb300 import gen, learn, pstep

pytestmark = pytest.mark.gpu

ERR_MOVE_BIT, ERR_TIMEOUT_BIT = 1 << 2, 1 << 3


def small_case(n=16, count=3000, seed=21):
    case = gen.make_case(n, count, seed, True)
    bp = helpers.make_bp(n, count)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    return bp, arrs, helpers.ghosted_fields(case)


def start(bp, arrs, fields, corrected=False):
    g = pstep.ParticleStep(bp.step_config(), len(arrs[-1]), pstep.FP32, 0)
    g.load(*arrs)
    if corrected:
        g.set_correction(learn.load_model(), bp.mu0 / bp.rho0)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    return g


def test_move_of_more_than_one_cell_is_reported(built_cuda):
    bp, arrs, fields = small_case()
    fast = [a.copy() for a in arrs]
    dx = bp.l / bp.n
    fast[3][::7] = 6.0 * dx / bp.dt  # stage 0 moves x by dt * 0.5 * u = 3 cells
    g = start(bp, fast, fields)
    g.run(1)
    rc, flags = g.check()
    assert rc == 8 and flags & ERR_MOVE_BIT, (rc, flags)
    # the same handle, a well-formed population: clean
    g.load(*arrs)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    g.run(1)
    rc, flags = g.check()
    assert rc == 0 and flags == 0, (rc, flags)
    g.close()


def test_inference_wait_timeout_is_reported_and_recovers(built_cuda):
    bp, arrs, fields = small_case()
    g = start(bp, arrs, fields, corrected=True)
    g.set_wait_limit(1000, idle_first=True)
    g.interp_advance_deposit(0)  # stage 0 runs the network: its first wait runs out
    rc, flags = g.check()
    assert rc == 10 and flags & ERR_TIMEOUT_BIT, (rc, flags)
    # back to the default bound on the same handle: a full step equals a fresh handle's
    g.set_wait_limit(0, idle_first=False)
    g.load(*arrs)
    g.set_correction(learn.load_model(), bp.mu0 / bp.rho0)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    g.run(1)
    rc, flags = g.check()
    assert rc == 0 and flags == 0, (rc, flags)
    ref = start(bp, arrs, fields, corrected=True)
    ref.run(1)
    io, ig = np.argsort(ref.array("flag")), np.argsort(g.array("flag"))
    for name in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
        assert helpers.bits_equal(g.array(name)[ig], ref.array(name)[io]), name
    for name in pstep.FIELD_IDS:
        assert helpers.bits_equal(g.field(name), ref.field(name)), name
    g.close()
    ref.close()
