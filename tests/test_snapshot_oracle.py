"""The snapshot files and statistics of the particle state, restated in the oracle
(pyoracle.store_all / load_all / array_max / field_stats / trajectory_ids), pinned
against the reference's own Store_All, Load_All, NP_TOT, max, Balance_Index,
tensor0 max/min/mean and trajectory (particle.cpp:662-741, 867-1025;
tensor0.cpp:418-503), compiled from its sources with the single-rank stub whose
MPI-IO is stdio on one file."""
import numpy as np
import pytest

import helpers
import pyoracle
from first_repo_gb300 import gen

pytestmark = pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not available")

N, COUNT = 16, 2000


def _case(seed=5):
    return helpers.make_bp(N, COUNT), gen.make_case(N, COUNT, seed, True)


def test_store_all_and_statistics_match_the_reference(tmp_path):
    bp, case = _case()
    recs, stats, traj = pyoracle.run_ref_snapshot(bp, case, 2, str(tmp_path), store_ts=2, np_track=7)
    last = recs[-1]
    restated = tmp_path / "restated"
    restated.mkdir()
    pyoracle.store_all(str(restated) + "/", 2, last)
    for name in pyoracle.SNAP_NAMES:
        ref = (tmp_path / f"{name}_2.bin").read_bytes()
        assert ref == (restated / f"{name}_2.bin").read_bytes(), name
        assert len(ref) == COUNT * (4 if name == "Part_flag" else 8)
    # a second Store_All of the same step refuses to overwrite (MPI_MODE_EXCL)
    with pytest.raises(FileExistsError):
        pyoracle.store_all(str(restated) + "/", 2, last)
    assert stats["np_tot"] == COUNT
    assert stats["balance_index"] == 1.0
    for k in ("x", "y", "z", "u", "v", "w", "T"):
        assert stats["max"][k] == pyoracle.array_max(last[k]), k
    assert tuple(stats["C"]) == pyoracle.field_stats(last["C"], N)
    assert tuple(stats["RHS_Part_Temp"]) == pyoracle.field_stats(last["E"], N)
    # trajectory: ids 0, K, 2K, ... located by find_tag; the reference writes 6 significant digits
    ids = pyoracle.trajectory_ids(COUNT, 7)
    assert len(ids) == 7 and traj[-1][0] == 2.0
    where = {int(f): i for i, f in enumerate(last["flag"])}
    pos = np.array([[last[k][where[t]] for k in ("x", "y", "z")] for t in ids])
    np.testing.assert_allclose(np.array(traj[-1][1:]), pos.ravel(), rtol=1e-5, atol=1e-9)


def test_load_all_matches_the_reference(tmp_path):
    bp, case = _case(seed=9)
    rng = np.random.default_rng(3)
    order = rng.permutation(COUNT)  # files in an arbitrary particle order, ids kept
    arrays = {k: np.ascontiguousarray(case["t" if k == "T" else k][order]) for k in pyoracle.SNAP_KEYS}
    for name, key in zip(pyoracle.SNAP_NAMES, pyoracle.SNAP_KEYS):
        dt = np.int32 if key == "flag" else np.float64
        (tmp_path / f"Restart_{name}.bin").write_bytes(arrays[key].astype(dt).tobytes())
    recs, _, _ = pyoracle.run_ref_snapshot(bp, case, 1, str(tmp_path), load=True)
    loaded = pyoracle.load_all(str(tmp_path) + "/", COUNT)
    prime = recs[0]  # the state Load_All produced, before the first stage
    for k in pyoracle.SNAP_KEYS:
        assert np.array_equal(prime[k], loaded[k]), k
        assert np.array_equal(loaded[k], arrays[k]), k
    with pytest.raises(IOError):
        pyoracle.load_all(str(tmp_path) + "/", COUNT + 1)


def test_array_max_edge_cases():
    assert pyoracle.array_max(np.array([])) == -1e9
    assert pyoracle.array_max(np.array([-3.0, -5.0])) == -3.0
    assert pyoracle.array_max(np.array([1.0, 7.0, 2.0])) == 7.0
