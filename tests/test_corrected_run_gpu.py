"""The corrected step (FP32 form, learned correction on the tensor cores) over 100
steps at 1/8 of the headline workload (box256_dense: 256^3 cells, 2^24 particles,
d_p/dx 0.5, mass loading 1.0, blob-centre occupancy as at full size), with the gas
fields held fixed: after every 10 steps the device check word is clear, every
particle array is finite, the deposited concentration sums to the particle count,
the deposited energy to the particles' RHS_T, and the momentum balance
(pstep_momentum_sums) equals the sums of the deposited momentum fields. The slip-
velocity and particle-temperature statistics against the plain FP64 drop-in after
the same 100 steps are reported (the configuration's required report)."""
import json

import numpy as np
import pytest

import helpers
from first_repo_gb300 import config, gen, learn, pstep

pytestmark = pytest.mark.gpu


def test_corrected_step_100_steps_eighth_size(built_cuda):
    torch = pytest.importorskip("torch")
    import bench
    wl = config.WORKLOADS["box256_dense"]
    n = wl.n_particles
    case = gen.make_case(wl.n, n, wl.seed, wl.clustered, nblobs=wl.nblobs)
    bp = config.box_params(wl.n, n, dp_over_dx=wl.dp_over_dx, mass_loading=wl.mass_loading)
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    fields = helpers.ghosted_fields(case)
    del case
    g = pstep.ParticleStep(bp.step_config(), n, pstep.FP32, 0)
    g.load(*arrs)
    g.set_correction(learn.load_model(), bp.mu0 / bp.rho0)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    for block in range(10):
        g.run(10)
        rc, flags = g.check()
        assert rc == 0, (block, flags)
        for name in ("x", "y", "z", "u", "v", "w", "T", "RHS_T"):
            assert np.all(np.isfinite(g.array(name))), (block, name)
        c = g.field("C")[1:-1, 1:-1, 1:-1]
        assert abs(c.sum() - n) <= 1e-5 * n, block
        rt = g.array("RHS_T")
        e = g.field("RHS_Part_Temp")[1:-1, 1:-1, 1:-1]
        assert abs(e.sum() - rt.sum()) <= 1e-5 * np.abs(rt).sum(), block
        mom = g.momentum_sums()
        for d, name in enumerate(("RHS_RU_x", "RHS_RU_y", "RHS_RU_z")):
            f = g.field(name)[1:-1, 1:-1, 1:-1]
            assert abs(mom[d] - f.sum()) <= 1e-12 * max(np.abs(f).sum(), 1e-300), (block, name)
    u_dev = [torch.from_numpy(np.ascontiguousarray(fields[d]).ravel()).to("cuda") for d in range(3)]
    stats_corr = bench.particle_stats(g, u_dev, bp.l, wl.n)
    g.close()
    g64 = pstep.ParticleStep(bp.step_config(), n, pstep.FP64, 0)
    g64.load(*arrs)
    g64.bind_velocity(*fields[:3])
    g64.bind_temperature(fields[3])
    g64.prime()
    g64.run(100)
    rc, flags = g64.check()
    assert rc == 0, flags
    stats64 = bench.particle_stats(g64, u_dev, bp.l, wl.n)
    g64.close()
    for st in (stats_corr, stats64):
        assert all(np.isfinite(v) for v in st.values()), st
    print("box256_dense after 100 steps: corrected FP32", json.dumps(stats_corr), "plain FP64", json.dumps(stats64),
          "difference", json.dumps(bench.stats_difference(stats_corr, stats64)))
