"""Training helpers of the learned far-field correction (host side).

The network, its features and its training run in libgeon_cuda.so
(geon_learn_dataset, geon_mlp_train); this module only draws the initial
weights and strings the calls together.  The reference has no counterpart:
its far field is the plain monopole of src/forces.js:680-685.
"""
from __future__ import annotations

import numpy as np

from . import _native as N

LF, LH, LO = 9, 64, 2


def init_weights(seed: int = 0) -> np.ndarray:
    """FP32 weight vector (W1 b1 W2 b2 W3 b3, W[out][in]) drawn like
    nn.Linear's default: U(-1/sqrt(fan_in), 1/sqrt(fan_in))."""
    rng = np.random.default_rng(seed)
    parts = []
    for o, i in ((LH, LF), (LH, LH), (LO, LH)):
        k = 1.0 / np.sqrt(i)
        parts.append(rng.uniform(-k, k, o * i))
        parts.append(rng.uniform(-k, k, o))
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == N.MLP_NPARAM
    return w


def train_correction(system, targets, steps: int = 20000, batch: int = 65536, lr: float = 2e-3, seed: int = 3,
                     cap: int = 60_000_000, init_seed: int = 1) -> dict:
    """Builds the residual dataset of `targets` on `system` at its current
    theta and trains the network on the device.  Returns the weights, the
    per-step losses and the dataset size."""
    targets = np.asarray(targets, dtype=np.int32)
    ds = system.learn_dataset(targets, cap)
    while ds["count"] > cap:                 # small theta: fewer targets so that the pairs fit
        keep = max(1, int(len(targets) * cap / ds["count"] * 0.9))
        targets = targets[np.linspace(0, len(targets) - 1, keep).astype(np.int64)]
        ds = system.learn_dataset(targets, cap)
    w, hist = system.mlp_train(init_weights(init_seed), ds["feat_mass"], ds["residual"][:, 0:2], steps=steps,
                               batch=batch, lr=lr, seed=seed)
    return {"weights": w, "loss": hist, "pairs": int(ds["count"]), "targets": int(len(targets))}
