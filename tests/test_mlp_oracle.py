"""The network oracle (oracle/mlp_oracle.py) on the CPU: its backpropagation
against central finite differences, its bf16 rounding against known values, and
the tensor-core rounding order against the exact fp64 gradient."""
import numpy as np

import helpers  # noqa: F401  (sets sys.path)
import mlp_oracle as mo


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.5, 1.5, (n, mo.N_IN))
    t = rng.normal(0, 0.5, (n, mo.N_OUT))
    return x, t


def test_bf16_rounding_known_values():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 3.0e-5, 0.0], dtype=np.float32)
    r = mo.bf16(v)
    # the bf16 spacing at 1 is 2^-7: 1 + 2^-8 is a tie and rounds to the even 1.0,
    # 1 + 3*2^-9 rounds up to 1 + 2^-7, 1 + 2^-9 rounds down
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == 1.0
    assert r[4] == -2.5 and r[6] == 0.0
    assert abs(r[5] - 3.0e-5) <= 3.0e-5 * 2 ** -8


def test_exact_gradient_matches_finite_differences():
    p = mo.init_params(3).astype(np.float64)
    x, t = _data(40, 4)
    g, _ = mo.gradient_exact(p, x, t)
    rng = np.random.default_rng(5)
    live = np.concatenate([np.arange(mo.OW1, mo.OB1).reshape(64, 16)[:, :10].ravel(), np.arange(mo.OB1, mo.OW3),
                           np.arange(mo.OW3, mo.OW3 + 4 * 64), np.arange(mo.OB3, mo.OB3 + 4)])
    for idx in rng.choice(live, 60, replace=False):
        e = np.zeros_like(p)
        h = 1e-6
        e[idx] = h
        fd = (mo.loss_exact(p + e, x, t) - mo.loss_exact(p - e, x, t)) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-7 + 1e-5 * abs(g[idx]), (idx, fd, g[idx])


def test_padding_has_no_gradient():
    p = mo.init_params(1)
    x, t = _data(16, 2)
    for g in (mo.gradient_exact(p, x, t)[0], mo.gradient_gpu_order(p, x, t)[0]):
        assert not np.any(g[mo.OW1:mo.OB1].reshape(64, 16)[:, 10:])
        assert not np.any(g[mo.OW3:mo.OB3].reshape(16, 64)[4:])
        assert not np.any(g[mo.OB3 + 4:])


def test_tensor_core_order_is_close_to_exact():
    """bf16 operands move the gradient by ~2^-8 relative, never more than a few %."""
    p = mo.init_params(7)
    x, t = _data(512, 8)
    ge, le = mo.gradient_exact(p, x, t)
    gb, lb = mo.gradient_gpu_order(p, x, t)
    assert abs(lb - le) <= 2e-2 * le
    for a, b in [(mo.OW1, mo.OB1), (mo.OW2, mo.OB2), (mo.OW3, mo.OB3)]:
        assert np.linalg.norm(gb[a:b] - ge[a:b]) <= 3e-2 * np.linalg.norm(ge[a:b])


def test_adam_reference_first_step_is_lr_times_sign():
    p = np.ones(5)
    g = np.array([1.0, -2.0, 0.5, 0.0, 3.0])
    q = mo.adam_reference(p, [g], lr=1e-3)
    np.testing.assert_allclose(q, p - 1e-3 * np.sign(g) * (np.abs(g) / (np.abs(g) + 1e-8)), rtol=1e-9, atol=1e-12)
