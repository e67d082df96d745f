"""The GPU machine gas step (first_repo_gb300/csrc/gas.cu) against its C
restatement (oracle/gas_oracle.c, itself bit-for-bit with the reference's
grid.cpp): gas alone, and coupled to the FP64 and FP32 particle steps.

Elementwise and stencil kernels repeat the restatement's arithmetic exactly
(no FMA, same operand order, same FFT butterflies and tables); the interior
mean and maximum reductions sum in a different order, so fields agree to a
few ulps that grow slowly: the bound is 1e-10 relative to the field's range
after 3 steps. The FP32 particle step's coupling is held to its own 1e-5."""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gas, pstep
from test_gas_oracle import gas_case

pytestmark = pytest.mark.gpu

FIELDS = ["RU_x", "RU_y", "RU_z", "Rho", "P", "T", "RHS_Part_Temp", "C", "RHS_RU_x"]


def _port(bp, fields, parts, nsteps, with_particles=True):
    o = None
    if with_particles:
        o = pyoracle.Oracle(bp.step_config(), len(parts["flag"]) + 16)
        o.load(*[parts[k] for k in ("x", "y", "z", "u", "v", "w", "t", "flag")])
    g = pyoracle.GasOracle(bp.gas_config(), o)
    g.init(fields["RU_x"], fields["RU_y"], fields["RU_z"], fields["Rho"], bp.gas_config()["p0"])
    out = []
    for _ in range(nsteps):
        g.step()
        rec = {k: g.field(k) for k in FIELDS}
        rec["P0"] = g.p0()
        if o is not None:
            fl = o.flag()
            order = np.argsort(fl)
            for k in ("x", "u", "T"):
                rec["p_" + k] = o.array(k)[order]
        out.append(rec)
    return out


def _gpu(bp, fields, parts, nsteps, precision=None, flags=0):
    ps = None
    if precision is not None:
        ps = pstep.ParticleStep(bp.step_config(), len(parts["flag"]) + 16, precision, flags)
        ps.load(*[parts[k] for k in ("x", "y", "z", "u", "v", "w", "t", "flag")])
    g = gas.GasStep(bp.gas_config(), ps)
    g.init(fields["RU_x"], fields["RU_y"], fields["RU_z"], fields["Rho"])
    out = []
    for _ in range(nsteps):
        g.step()
        rec = {k: g.field(k) for k in FIELDS}
        rec["P0"] = g.p0()
        if ps is not None:
            order = np.argsort(ps.array("flag"))
            for k in ("x", "u", "T"):
                rec["p_" + k] = ps.array(k)[order]
        out.append(rec)
    return out, g


def _rel(a, b):
    a, b = a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


def test_gas_only_matches_restatement(built_cuda):
    bp, fields, parts = gas_case(32, 10, 21)
    ref = _port(bp, fields, parts, 3, with_particles=False)
    got, g = _gpu(bp, fields, parts, 3)
    for s in range(3):
        for k in ("RU_x", "RU_y", "RU_z", "Rho", "P", "T"):
            assert _rel(got[s][k], ref[s][k]) <= 1e-10, (s, k, _rel(got[s][k], ref[s][k]))
        assert abs(got[s]["P0"] - ref[s]["P0"]) <= 1e-14
    assert g.iterations() >= 1


@pytest.mark.parametrize("cooling", [0, 1])
def test_coupled_fp64_matches_restatement(built_cuda, cooling):
    bp, fields, parts = gas_case(16, 300, 11, cooling)
    ref = _port(bp, fields, parts, 3)
    got, _ = _gpu(bp, fields, parts, 3, pstep.FP64, pstep.TRACK_ORDER | pstep.REFERENCE_SUMS)
    for s in range(3):
        for k in FIELDS:
            assert _rel(got[s][k], ref[s][k]) <= 1e-10, (s, k, _rel(got[s][k], ref[s][k]))
        for k in ("p_x", "p_u", "p_T"):
            assert helpers.max_rel_to_max(got[s][k], ref[s][k]) <= 1e-10, (s, k)
        assert abs(got[s]["P0"] - ref[s]["P0"]) <= 1e-13


def test_coupled_fp32_within_its_bound(built_cuda):
    bp, fields, parts = gas_case(32, 2000, 31)
    ref = _port(bp, fields, parts, 2)
    got, _ = _gpu(bp, fields, parts, 2, pstep.FP32)
    for s in range(2):
        for k in ("RU_x", "Rho", "P", "T", "RHS_Part_Temp", "RHS_RU_x"):
            assert _rel(got[s][k], ref[s][k]) <= 1e-5, (s, k, _rel(got[s][k], ref[s][k]))
        for k in ("p_u", "p_T"):
            assert helpers.max_rel_to_max(got[s][k], ref[s][k]) <= 1e-5, (s, k)
