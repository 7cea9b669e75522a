"""FP64 NumPy restatement of the learned-correction network — TEST
INFRASTRUCTURE ONLY (the checker of the tensor-core kernels; nothing in the
product path imports it).

The reference has no learned correction (its far field is the plain monopole
of src/forces.js:680-685), so this file restates the network the C ABI
documents for geon_mlp_forward / geon_mlp_grad: 14 -> 64 -> 64 -> 6, GELU in
its tanh form after both hidden layers, and the loss
    (1/B) sum_s wt_s sum_c (y_sc - y*_sc)^T A_sc (y_sc - y*_sc)
with y_sc the outputs 3c .. 3c+2 and the target row t_s = y*_s[6], then the
two symmetric 3 x 3 forms A_s0, A_s1 as (A00 A11 A22 A01 A02 A12).

With ``bf16=True`` the operands are rounded to BF16 (round to nearest even)
at the points where the device kernels round them — inputs, weights, hidden
activations, the output gradient and the pre-activation gradients — and all
arithmetic is FP64 otherwise, so the only differences left against the
device are its FP32 accumulation order and its tanh approximation.  With
``bf16=False`` it is the plain FP64 network, whose analytic gradient the
tests check by finite differences.
"""
from __future__ import annotations

import numpy as np

LF, LH, LO = 14, 64, 6
LT = LO + 12
NPARAM = 2 * LF + LH * LF + LH + LH * LH + LH + LO * LH + LO
GELU_C = np.sqrt(2.0 / np.pi)
GELU_A = 0.044715


def bf16(a) -> np.ndarray:
    """Rounds to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out[nan] = np.nan
    return out


def unpack(w) -> dict:
    w = np.asarray(w, dtype=np.float64)
    assert w.size == NPARAM
    o = 0
    out = {}
    for name, shape in (("mu", (LF,)), ("isd", (LF,)), ("W1", (LH, LF)), ("b1", (LH,)), ("W2", (LH, LH)), ("b2", (LH,)),
                        ("W3", (LO, LH)), ("b3", (LO,))):
        k = int(np.prod(shape))
        out[name] = w[o:o + k].reshape(shape)
        o += k
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[k], dtype=np.float64).ravel()
                           for k in ("mu", "isd", "W1", "b1", "W2", "b2", "W3", "b3")])


def init_weights(seed: int = 0) -> np.ndarray:
    """nn.Linear's default initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in));
    identity normalisation."""
    rng = np.random.default_rng(seed)
    d = {"mu": np.zeros(LF), "isd": np.ones(LF)}
    for (wn, bn), (o, i) in zip((("W1", "b1"), ("W2", "b2"), ("W3", "b3")), ((LH, LF), (LH, LH), (LO, LH))):
        k = 1.0 / np.sqrt(i)
        d[wn] = rng.uniform(-k, k, (o, i))
        d[bn] = rng.uniform(-k, k, (o,))
    return pack(d).astype(np.float32)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(GELU_C * (x + GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * x * x)


def _r(a, on):
    return bf16(a) if on else np.asarray(a, dtype=np.float64)


def forward(w, x, bf16_ops: bool = True, keep: bool = False):
    p = unpack(w)
    x = np.asarray(x, dtype=np.float64).reshape(-1, LF)
    x = _r((x - p["mu"]) * p["isd"], bf16_ops)
    W1, W2, W3 = (_r(p[k], bf16_ops) for k in ("W1", "W2", "W3"))
    z1 = x @ W1.T + p["b1"]
    h1 = _r(gelu(z1), bf16_ops)
    z2 = h1 @ W2.T + p["b2"]
    h2 = _r(gelu(z2), bf16_ops)
    y = h2 @ W3.T + p["b3"]
    if keep:
        return y, dict(x=x, W1=W1, W2=W2, W3=W3, z1=z1, h1=h1, z2=z2, h2=h2)
    return y


def quad_forms(t):
    """The target rows [B, 18] as (y* [B, 6], A [B, 2, 3, 3])."""
    t = np.asarray(t, dtype=np.float64).reshape(-1, LT)
    A = np.zeros((len(t), 2, 3, 3))
    for c in range(2):
        a = t[:, LO + 6 * c:LO + 6 * c + 6]
        A[:, c] = np.stack([np.stack([a[:, 0], a[:, 3], a[:, 4]], -1), np.stack([a[:, 3], a[:, 1], a[:, 5]], -1),
                            np.stack([a[:, 4], a[:, 5], a[:, 2]], -1)], -2)
    return t[:, :LO], A


def loss_grad(w, x, t, wt=None, bf16_ops: bool = True):
    """(gradient vector, loss) of (1/B) sum_s wt_s sum_c e_sc^T A_sc e_sc,
    e_sc = y_sc - y*_sc."""
    y, c = forward(w, x, bf16_ops, keep=True)
    ys, A = quad_forms(t)
    B = len(y)
    wt = np.ones(B) if wt is None else np.asarray(wt, dtype=np.float64)
    e = (y - ys).reshape(B, 2, 3)
    Ae = np.einsum("bcij,bcj->bci", A, e)
    loss = float(np.sum(wt * np.einsum("bci,bci->b", e, Ae)) / B)
    dy = _r((2.0 * wt[:, None] * Ae.reshape(B, LO)) / B, bf16_ops)
    dh2 = dy @ c["W3"]
    dz2 = _r(dh2 * gelu_grad(c["z2"]), bf16_ops)
    dh1 = dz2 @ c["W2"]
    dz1 = _r(dh1 * gelu_grad(c["z1"]), bf16_ops)
    g = dict(mu=np.zeros(LF), isd=np.zeros(LF), W3=dy.T @ c["h2"], b3=dy.sum(0), W2=dz2.T @ c["h1"], b2=dz2.sum(0),
             W1=dz1.T @ c["x"], b1=dz1.sum(0))
    return pack(g), loss


def random_targets(rng, n, scale=0.1):
    """Target rows with positive definite forms, for tests."""
    t = np.zeros((n, LT))
    t[:, :LO] = rng.normal(size=(n, LO)) * scale
    for c in range(2):
        L = rng.normal(size=(n, 3, 3)) * 0.5 + np.eye(3)
        A = L @ np.transpose(L, (0, 2, 1))
        t[:, LO + 6 * c:LO + 6 * c + 6] = np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], 1)
    return t
