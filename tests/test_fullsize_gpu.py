"""The corrected FP32 step at the headline workload's full size (box512_corrected:
512^3 cells x 2^27 clustered particles, d_p/dx 0.5, mass loading 1.0), checked
through size-independent properties: the deposited concentration sums to the
particle count and the deposited energy to the particles' RHS_T (the trilinear
weights of a particle add to one), the device check word is clear, and two runs
give bit-identical fields and particle states (a digest of every array)."""
import hashlib

import numpy as np
import pytest

from first_repo_gb300 import config, gen, learn, pstep

pytestmark = pytest.mark.gpu


def test_corrected_step_at_full_size(built_cuda):
    wl = config.WORKLOADS["box512_corrected"]
    n = wl.n_particles
    case = gen.make_case(wl.n, n, wl.seed, wl.clustered, nblobs=wl.nblobs)
    bp = config.box_params(wl.n, n, dp_over_dx=wl.dp_over_dx, mass_loading=wl.mass_loading)
    fields = [gen.ghost(case[k]) for k in ("ux", "uy", "uz", "T")]
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    del case
    digests = []
    for _ in range(2):
        g = pstep.ParticleStep(bp.step_config(), n, pstep.FP32, 0)
        g.load(*arrs)
        g.set_correction(learn.load_model(), bp.mu0 / bp.rho0)
        g.bind_velocity(*fields[:3])
        g.bind_temperature(fields[3])
        g.prime()
        g.run(1)
        rc, flags = g.check()
        assert rc == 0, flags
        c = g.field("C")[1:-1, 1:-1, 1:-1]
        assert abs(c.sum() - n) <= 1e-5 * n
        rt = g.array("RHS_T")
        e = g.field("RHS_Part_Temp")[1:-1, 1:-1, 1:-1]
        assert abs(e.sum() - rt.sum()) <= 1e-5 * np.abs(rt).sum()
        h = hashlib.sha256()
        for name in pstep.FIELD_IDS:
            h.update(g.field(name).tobytes())
        order = np.argsort(g.array("flag"))
        for name in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
            h.update(g.array(name)[order].tobytes())
        digests.append(h.hexdigest())
        g.close()
    assert digests[0] == digests[1]
