"""CPU oracle of the learned correction's network -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may use this
module, and only as the checker. The product's network runs on the tensor
cores (first_repo_gb300/csrc/mlp.cu); nothing in the product imports this file.

The network has no reference counterpart (the reference interpolates the
disturbed gas state, particle.cpp:340-360). This restatement pins the GPU
kernels two ways:

* `gradient_exact` is plain fp64 backpropagation of the mean squared error
  through 10 -> 64 SiLU -> 64 SiLU -> 4; it is itself checked against central
  finite differences of `loss_exact` (tests/test_mlp_oracle.py);
* `forward_gpu_order` / `gradient_gpu_order` evaluate the same mathematics with
  the tensor-core kernels' rounding points: every MMA operand (features,
  weights, activations, back-propagated deltas) rounded to bf16 (round to
  nearest even), products summed in high precision (the MMA accumulates in
  fp32), biases, SiLU and its derivative applied to fp32 values, bias gradients
  summed from the unrounded fp32 deltas.

Parameter layout (fp32, PMLP_NPARAM = 6288 floats) as in include/pstep_mlp.h.
"""
from __future__ import annotations

import numpy as np

N_IN, N_IN_PAD, N_HID, N_OUT, N_OUT_PAD = 10, 16, 64, 4, 16
OW1 = 0
OB1 = OW1 + N_HID * N_IN_PAD
OW2 = OB1 + N_HID
OB2 = OW2 + N_HID * N_HID
OW3 = OB2 + N_HID
OB3 = OW3 + N_OUT_PAD * N_HID
NPARAM = OB3 + N_OUT_PAD
assert NPARAM == 6288


def bf16(a) -> np.ndarray:
    """fp32 -> bf16 -> fp32, round to nearest even (finite inputs)."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p: np.ndarray, dtype=np.float32):
    p = np.asarray(p, dtype=dtype)
    w1 = p[OW1:OB1].reshape(N_HID, N_IN_PAD)
    b1 = p[OB1:OW2]
    w2 = p[OW2:OB2].reshape(N_HID, N_HID)
    b2 = p[OB2:OW3]
    w3 = p[OW3:OB3].reshape(N_OUT_PAD, N_HID)
    b3 = p[OB3:NPARAM]
    return w1, b1, w2, b2, w3, b3


def pack(w1, b1, w2, b2, w3, b3) -> np.ndarray:
    p = np.zeros(NPARAM, dtype=np.float64)
    p[OW1:OB1] = np.asarray(w1).reshape(-1)
    p[OB1:OW2] = b1
    p[OW2:OB2] = np.asarray(w2).reshape(-1)
    p[OB2:OW3] = b2
    p[OW3:OB3] = np.asarray(w3).reshape(-1)
    p[OB3:NPARAM] = b3
    return p


def _pad_x(x):
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros((x.shape[0], N_IN_PAD))
    out[:, :N_IN] = x
    return out


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


# ---------------------------------------------------------------- exact fp64
def forward_exact(p, x):
    w1, b1, w2, b2, w3, b3 = unpack(p, np.float64)
    xp = _pad_x(x)
    z1 = xp @ w1.T + b1
    h1 = z1 * _sig(z1)
    z2 = h1 @ w2.T + b2
    h2 = z2 * _sig(z2)
    y = h2 @ w3.T + b3
    return y[:, :N_OUT], (xp, z1, h1, z2, h2)


def loss_exact(p, x, t) -> float:
    y, _ = forward_exact(p, x)
    r = y - np.asarray(t, dtype=np.float64)
    return float(np.mean(r * r))


def gradient_exact(p, x, t):
    """d loss_exact / d p (fp64 backpropagation), and the loss."""
    w1, b1, w2, b2, w3, b3 = unpack(p, np.float64)
    y, (xp, z1, h1, z2, h2) = forward_exact(p, x)
    t = np.asarray(t, dtype=np.float64)
    n = x.shape[0]
    r = y - t
    dy = np.zeros((n, N_OUT_PAD))
    dy[:, :N_OUT] = 2.0 * r / (n * N_OUT)
    s2 = _sig(z2)
    dz2 = (dy @ w3) * s2 * (1.0 + z2 * (1.0 - s2))
    s1 = _sig(z1)
    dz1 = (dz2 @ w2) * s1 * (1.0 + z1 * (1.0 - s1))
    g = pack(dz1.T @ xp, dz1.sum(0), dz2.T @ h1, dz2.sum(0), dy.T @ h2, dy.sum(0))
    g[OW1:OB1].reshape(N_HID, N_IN_PAD)[:, N_IN:] = 0.0
    return g, float(np.mean(r * r))


# --------------------------------------------------- tensor-core rounding points
def forward_gpu_order(p, x):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    w1b, w2b, w3b = (bf16(w).astype(np.float64) for w in (w1, w2, w3))
    xb = bf16(_pad_x(x)).astype(np.float64)
    z1 = (xb @ w1b.T).astype(np.float32) + b1
    s1 = _sig(z1.astype(np.float64))
    h1 = (z1 * s1).astype(np.float32)
    h1b = bf16(h1).astype(np.float64)
    z2 = (h1b @ w2b.T).astype(np.float32) + b2
    s2 = _sig(z2.astype(np.float64))
    h2 = (z2 * s2).astype(np.float32)
    h2b = bf16(h2).astype(np.float64)
    y = (h2b @ w3b.T).astype(np.float32) + b3
    return y[:, :N_OUT].astype(np.float64), (xb, z1, s1, h1b, z2, s2, h2b)


def gradient_gpu_order(p, x, t):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    w2b, w3b = (bf16(w).astype(np.float64) for w in (w2, w3))
    y, (xb, z1, s1, h1b, z2, s2, h2b) = forward_gpu_order(p, x)
    t = np.asarray(t, dtype=np.float64)
    n = x.shape[0]
    r = (y - t).astype(np.float32)
    dy = np.zeros((n, N_OUT_PAD), dtype=np.float32)
    dy[:, :N_OUT] = np.float32(2.0) * r * np.float32(1.0 / (n * N_OUT))
    dyb = bf16(dy).astype(np.float64)
    dh2 = (dyb @ w3b).astype(np.float32)
    dz2 = (dh2 * (s2 * (1.0 + z2 * (1.0 - s2)))).astype(np.float32)
    dz2b = bf16(dz2).astype(np.float64)
    dh1 = (dz2b @ w2b).astype(np.float32)
    dz1 = (dh1 * (s1 * (1.0 + z1 * (1.0 - s1)))).astype(np.float32)
    dz1b = bf16(dz1).astype(np.float64)
    g = pack(dz1b.T @ xb, dz1.astype(np.float64).sum(0), dz2b.T @ h1b, dz2.astype(np.float64).sum(0),
             dyb.T @ h2b, dy.astype(np.float64).sum(0))
    g[OW1:OB1].reshape(N_HID, N_IN_PAD)[:, N_IN:] = 0.0
    g[OW3:OB3].reshape(N_OUT_PAD, N_HID)[N_OUT:, :] = 0.0
    g[OB3 + N_OUT:NPARAM] = 0.0
    return g, float(np.mean(r.astype(np.float64) ** 2))


def init_params(seed: int) -> np.ndarray:
    """Deterministic random parameters for tests (not the library's initialiser)."""
    rng = np.random.default_rng(seed)
    w1 = np.zeros((N_HID, N_IN_PAD))
    w1[:, :N_IN] = rng.uniform(-1, 1, (N_HID, N_IN)) / np.sqrt(N_IN)
    w3 = np.zeros((N_OUT_PAD, N_HID))
    w3[:N_OUT] = rng.uniform(-1, 1, (N_OUT, N_HID)) / np.sqrt(N_HID)
    b3 = np.zeros(N_OUT_PAD)
    b3[:N_OUT] = rng.uniform(-0.1, 0.1, N_OUT)
    return pack(w1, rng.uniform(-0.3, 0.3, N_HID), rng.uniform(-1, 1, (N_HID, N_HID)) / np.sqrt(N_HID),
                rng.uniform(-0.3, 0.3, N_HID), w3, b3).astype(np.float32)


def adam_reference(p, grads, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """Adam over a sequence of gradients (fp64), as the library's update."""
    p = np.asarray(p, dtype=np.float64).copy()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for t, g in enumerate(grads, start=1):
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p -= lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p
