"""pstep_field_mean_noalloc: the interior mean of a deposited field with no
device allocation, for callers that cannot call cudaMalloc (work recorded
during stream capture, an application's own memory pool, loops that must not
synchronise the device). Checked through the C ABI against the handle's own
pstep_energy_mean (tolerance 1e-12 relative, a different fixed summation
order) on two calls in a row. Collected last on purpose: it must pass alone in
a fresh process (its first call looks up the scratch array's address) and
after every other test."""
import ctypes as C

import numpy as np
import pytest

import helpers
from first_repo_gb300 import gen, pstep

pytestmark = pytest.mark.gpu

MEAN_RTOL = 1e-12


def test_field_mean_noalloc_matches_energy_mean(built_cuda):
    torch = pytest.importorskip("torch")
    L = pstep.lib()
    L.pstep_field_mean_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    L.pstep_noalloc_last_error.restype = C.c_char_p
    cdef = helpers.golden_case("box32_clustered")
    n = cdef["n"]
    case = gen.make_case(n, cdef["count"], cdef["seed"], cdef["clustered"])
    bp = helpers.make_bp(n, cdef["count"])
    g = pstep.ParticleStep(bp.step_config(), cdef["count"], pstep.FP64, pstep.TRACK_ORDER)
    g.load(*(np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")))
    ux, uy, uz, tf = helpers.ghosted_fields(case)
    g.bind_velocity(ux, uy, uz)
    g.bind_temperature(tf)
    g.prime()
    field = torch.empty((n + 2) ** 3, dtype=torch.float64, device="cuda")
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    means = []
    for _ in range(2):  # two calls in a row, on two different fields
        g.run(1)
        g._ok(L.pstep_get_field(g.h, pstep.FIELD_IDS["RHS_Part_Temp"], C.c_void_p(field.data_ptr()), 1))
        rc = L.pstep_field_mean_noalloc(C.c_void_p(field.data_ptr()), n, n, n, C.c_void_p(out.data_ptr()), None)
        assert rc == 0, L.pstep_noalloc_last_error()
        torch.cuda.synchronize()
        got, want = float(out.item()), g.energy_mean()
        assert abs(got - want) <= MEAN_RTOL * abs(want), (got, want)
        means.append(got)
    assert means[0] != means[1]
    # a non-cubic field with non-zero ghost layers: the interior of a (nz+2, ny+2, nx+2)
    # array, axes in the reference's layout (i fastest), against numpy
    nx, ny, nz = 5, 7, 3
    rng = np.random.default_rng(5)
    host = rng.standard_normal((nz + 2, ny + 2, nx + 2)) + 10.0 * np.arange(nz + 2)[:, None, None]
    host[1:-1, 1:-1, 1:-1] += np.arange(nx)[None, None, :] * 0.25 + np.arange(ny)[None, :, None] * 0.5
    small = torch.from_numpy(host.ravel().copy()).to("cuda")
    rc = L.pstep_field_mean_noalloc(C.c_void_p(small.data_ptr()), nx, ny, nz, C.c_void_p(out.data_ptr()), None)
    assert rc == 0, L.pstep_noalloc_last_error()
    torch.cuda.synchronize()
    want = host[1:-1, 1:-1, 1:-1].mean()
    assert abs(float(out.item()) - want) <= MEAN_RTOL * abs(want), (float(out.item()), want)
    # beyond the fixed scratch: a clear error, nothing launched
    rc = L.pstep_field_mean_noalloc(C.c_void_p(field.data_ptr()), 4, 2048, 1024, C.c_void_p(out.data_ptr()), None)
    assert rc == 3 and b"exceeds" in L.pstep_noalloc_last_error()
    g.close()
