"""Host logic of the learned correction (first_repo_gb300/learn.py) on CPU: the
quiescent-gas training boxes (4096 isolated particles on a 16 dx lattice in
128^3 boxes, Re_p log-uniform in [0.1, 50], d_p/dx uniform in [0.05, 1], Q
uniform in [0, 2]), the feature normaliser, the prior, the error metrics and the
committed network's file."""
import math

import numpy as np

from first_repo_gb300 import learn
from first_repo_gb300.mlp import NPARAM as N_PARAMS


def test_training_boxes_follow_the_quiescent_gas_construction():
    spec = learn.Spec()
    runs = learn.sample(spec, 3001)
    assert len(runs) == spec.runs and sum(len(r["q"]) for r in runs) == 4096
    dx = spec.dx
    for r in runs:
        assert np.all((r["dp_dx"] >= 0.05) & (r["dp_dx"] <= 1.0))
        assert np.all((r["re_p"] >= 0.1) & (r["re_p"] <= 50.0))
        assert np.all((r["q"] >= 0.0) & (r["q"] <= 2.0))
        assert np.allclose(np.linalg.norm(r["dir"], axis=1), 1.0)
        # one particle per lattice site, anywhere inside the site's cell
        cell = np.floor(r["pos"] / dx).astype(int)
        assert np.all((cell - spec.lattice // 2) % spec.lattice == 0)
        d = r["pos"][:, None, :] - r["pos"][None, :, :]
        dist = np.linalg.norm(d, axis=2) + np.eye(len(d)) * 1e9
        assert dist.min() > (spec.lattice - 1) * dx
        # the box viscosity keeps the fastest particle at <= cfl_max cells per step and
        # viscous diffusion at <= visc_max dx^2 per step
        visc = r["nu"] * spec.dt / dx ** 2
        assert visc <= spec.visc_max * (1 + 1e-12)
        re_cell = r["re_p"] / r["dp_dx"]
        assert re_cell.max() * visc <= spec.cfl_max * (1 + 1e-12)
    # boxes grouped by Re_p / (d_p/dx): each box's range sits above the previous one's
    tops = [float((r["re_p"] / r["dp_dx"]).max()) for r in runs]
    bots = [float((r["re_p"] / r["dp_dx"]).min()) for r in runs]
    assert all(bots[i + 1] >= tops[i] for i in range(len(runs) - 1))


def test_normaliser_and_prior():
    rng = np.random.default_rng(5)
    m = 1000
    f = np.column_stack([rng.uniform(0, 1, (m, 3)), rng.normal(size=(m, 3)), rng.uniform(0.05, 1, m),
                         np.log(rng.uniform(0.1, 50, m)), rng.uniform(0, 2, m), np.log(rng.uniform(0.01, 1, m))])
    shift, scale, lo, hi = learn.normaliser(f)
    x = (f - shift) * scale
    assert np.all(np.abs(x[:, 6:]) <= 1 + 1e-12)
    assert np.all((x[:, :3] >= -1) & (x[:, :3] < 1))
    assert np.array_equal(x[:, 3:6], f[:, 3:6])
    assert np.allclose(lo, [f[:, 6].min(), math.exp(f[:, 7].min()), f[:, 8].min(), math.exp(f[:, 9].min())])
    assert np.allclose(hi, [f[:, 6].max(), math.exp(f[:, 7].max()), f[:, 8].max(), math.exp(f[:, 9].max())])
    p = learn.prior(f)
    assert np.allclose(p, f[:, 6] / (1 + np.exp(f[:, 7]) / f[:, 6] / learn.PRIOR_RE))


def test_error_metrics():
    spec = learn.Spec()
    slip0 = np.array([[1.0, 0.0, 0.0], [0.0, 2.0, 0.0]])
    rec = {"const": {"slip0": slip0, "q": np.array([1.0, 0.0])}, "flag": np.array([0, 1]),
           "ug": np.array([0.1, 0.0]), "vg": np.array([0.0, 0.4]), "wg": np.zeros(2),
           "Tg": np.array([1.0 + 0.15 * 0.3, 5.0]),
           "final": {"flag": np.array([1, 0]), "u": np.array([0.0, 1.05]), "v": np.array([1.9, 0.0]),
                     "w": np.zeros(2)}}
    e = learn.errors(spec, rec)
    assert math.isclose(e["slip_rms"], math.sqrt((0.1 ** 2 + 0.2 ** 2) / 2))
    assert math.isclose(e["settle_rms"], math.sqrt((0.05 ** 2 + 0.05 ** 2) / 2))
    assert math.isclose(e["temp_rms"], 0.3)  # only the particle with Q > 0.05 counts


def test_committed_network_file(tmp_path):
    model = learn.load_model()
    assert model["params"].size == N_PARAMS and np.all(np.isfinite(model["params"]))
    assert model["shift"].shape == (10,) and model["scale"].shape == (10,)
    assert model["lo"].shape == (4,) and np.all(model["lo"] <= model["hi"])
    assert float(model["prior_re"]) == np.float32(learn.PRIOR_RE)
    path = str(tmp_path / "m.npz")
    learn.save_model(model, path, meta={"note": "round trip"})
    back = learn.load_model(path)
    for k in model:
        assert np.array_equal(np.asarray(back[k]), np.asarray(model[k])), k


def test_slip_error_binned_by_k():
    """slip_by_k: per-particle RMS of |gas used| / terminal slip, binned by the particle's K from
    the plain run (|gas| / |drive slip|); a correction removing 90% of every disturbance
    reduces every bin 10x."""
    rng = np.random.default_rng(0)
    n, steps = 60, 3
    fl = np.tile(np.arange(n), steps)
    slip0 = rng.normal(size=(n, 3))
    k = rng.uniform(0.0, 1.2, n)

    def rec(scale):
        g = slip0[fl] * scale[fl, None]
        u = slip0[fl] + g
        return dict(const=dict(slip0=slip0), flag=fl, ug=g[:, 0], vg=g[:, 1], wg=g[:, 2],
                    u=u[:, 0], v=u[:, 1], w=u[:, 2])

    bins = learn.slip_by_k([(rec(k), rec(0.1 * k))])
    assert sum(b["particles"] for b in bins) == n
    for b in bins:
        assert abs(b["reduction"] - 10.0) < 1e-9
        assert b["k_lo"] <= b["plain"] < max(b["k_hi"], 2.0)


def test_symmetry_images_transform_features_and_targets_together():
    """Each image is one element of the cube's symmetry group applied to a sample: the
    scalar features and the temperature target are unchanged; offsets about the cell
    centre, the slip direction and the velocity target permute and change sign together,
    so every dot product among them and every norm is kept; the images cover the group."""
    rng = np.random.default_rng(11)
    m = 400
    f = np.column_stack([rng.uniform(0, 1, (m, 3)), rng.normal(size=(m, 3)), rng.uniform(size=(m, 4))])
    y = rng.normal(size=(m, 4))
    F, Y = learn.symmetry_images(f, y, 5, 1)
    assert F.shape == (6 * m, 10) and Y.shape == (6 * m, 4)
    assert np.array_equal(F[:m], f) and np.array_equal(Y[:m], y)
    seen = set()
    for c in range(1, 6):
        g, z = F[c * m:(c + 1) * m], Y[c * m:(c + 1) * m]
        assert np.array_equal(g[:, 6:], f[:, 6:]) and np.array_equal(z[:, 3], y[:, 3])
        vecs_f = (f[:, :3] - 0.5, f[:, 3:6], y[:, :3])
        vecs_g = (g[:, :3] - 0.5, g[:, 3:6], z[:, :3])
        for a in range(3):
            for b in range(3):
                assert np.allclose(np.sum(vecs_g[a] * vecs_g[b], 1), np.sum(vecs_f[a] * vecs_f[b], 1))
        assert np.all((g[:, :3] >= 0) & (g[:, :3] <= 1))
        # which group element: the signed permutation mapping d to its image
        for i in range(0, m, 7):
            M = np.round(np.linalg.lstsq(np.stack([f[i, 3:6], y[i, :3], f[i, :3] - 0.5]),
                                         np.stack([g[i, 3:6], z[i, :3], g[i, :3] - 0.5]), rcond=None)[0], 6)
            assert np.allclose(np.abs(M).sum(0), 1) and np.allclose(np.abs(M).sum(1), 1)
            seen.add(tuple(M.ravel()))
    assert len(seen) > 30  # of 48
    assert learn.symmetry_images(f, y, 0, 1)[0] is f
