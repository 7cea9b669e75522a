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


def pair_weights(system, ds, mass) -> np.ndarray:
    """Loss weight of each pair: its share of its particle's relative force
    error per unit network error, (m_i * scale / |F_i|)^2, normalised to mean
    1 (|F_i| from a Barnes-Hut force pass at the same theta).  This makes the
    loss the mean squared relative force error the correction is judged by."""
    system.compute_forces()
    f = system.forces()
    fmag = np.hypot(f["fx"], f["fy"]).astype(np.float64)
    t = ds["target"]
    w = (mass[t] * ds["scales"][:, 0].astype(np.float64) / np.maximum(fmag[t], 1e-30)) ** 2
    return (w / max(w.mean(), 1e-300)).astype(np.float32)


def train_correction(system, targets, steps: int = 20000, batch: int = 65536, lr: float = 2e-3, seed: int = 3,
                     cap: int = 60_000_000, init_seed: int = 1, mass=None) -> dict:
    """Builds the residual dataset of `targets` on `system` at its current
    theta and trains the network on the device.  With `mass` (the system's
    particle masses) the pairs are weighted by pair_weights.  Returns the
    weights, the per-step losses and the dataset size."""
    targets = np.asarray(targets, dtype=np.int32)
    ds = system.learn_dataset(targets, cap)
    while ds["count"] > cap:                 # small theta: fewer targets so that the pairs fit
        keep = max(1, int(len(targets) * cap / ds["count"] * 0.9))
        targets = targets[np.linspace(0, len(targets) - 1, keep).astype(np.int64)]
        ds = system.learn_dataset(targets, cap)
    wt = pair_weights(system, ds, np.asarray(mass, dtype=np.float64)) if mass is not None else None
    w, hist = system.mlp_train(init_weights(init_seed), ds["feat_mass"], ds["residual"][:, 0:2], steps=steps,
                               batch=batch, lr=lr, seed=seed, wt=wt)
    return {"weights": w, "loss": hist, "pairs": int(ds["count"]), "targets": int(len(targets))}
