"""Training of the learned far-field correction (host side).

The records, the network, its gradients and Adam run in libgeon_cuda.so
(geon_learn_dataset, geon_mlp_train); this module draws the initial weights,
resamples the records and sets the network's input normalisation from them.
The reference has no counterpart: its far field is the plain monopole of
src/forces.js:680-685.
"""
from __future__ import annotations

import numpy as np

from . import _native as N

LF, LH, LO = N.LEARN_FEATURES, 64, N.LEARN_OUTPUTS


def init_weights(seed: int = 0) -> np.ndarray:
    """FP32 weight vector (mu isd W1 b1 W2 b2 W3 b3, W[out][in]) drawn like
    nn.Linear's default, U(-1/sqrt(fan_in), 1/sqrt(fan_in)), with the output
    layer scaled down so that an untrained network corrects little."""
    rng = np.random.default_rng(seed)
    parts = [np.zeros(LF), np.ones(LF)]                      # identity input normalisation
    for o, i, sc in ((LH, LF, 1.0), (LH, LH, 1.0), (LO, LH, 0.1)):
        k = 1.0 / np.sqrt(i)
        parts.append(rng.uniform(-k, k, o * i) * sc)
        parts.append(rng.uniform(-k, k, o) * sc)
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == N.MLP_NPARAM
    return w


def form_trace(target: np.ndarray) -> np.ndarray:
    """Trace of a record's two quadratic forms: its weight in the loss."""
    t = np.asarray(target, dtype=np.float64)
    return t[:, LO + 0] + t[:, LO + 1] + t[:, LO + 2] + t[:, LO + 6] + t[:, LO + 7] + t[:, LO + 8]


def resample(feat, target, size: int, seed: int = 0, alpha: float = 0.5):
    """Records drawn with probability proportional to their loss weight
    raised to alpha, each quadratic form scaled by weight^(1 - alpha) / weight
    (normalised to mean 1): the same expected loss.  alpha = 1 gives the
    lowest variance per sample but, because a few records near the disk
    centre (where the net field nearly cancels) carry most of the weight,
    draws only a few hundred distinct records; alpha < 1 keeps the data
    diverse."""
    tr = form_trace(target)
    keep = tr > 0
    feat, target, tr = feat[keep], target[keep], tr[keep]
    pw = tr ** alpha
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(len(tr), size=int(size), p=pw / pw.sum()))
    x = np.ascontiguousarray(feat[idx], dtype=np.float32)
    t = np.array(target[idx], dtype=np.float64)
    scale = tr[idx] ** (1.0 - alpha) / tr[idx]
    scale /= np.mean(tr[idx] ** (1.0 - alpha))
    t[:, LO:] *= scale[:, None]
    return x, np.ascontiguousarray(t, dtype=np.float32)


def set_normalisation(w: np.ndarray, mu: np.ndarray, sd: np.ndarray) -> np.ndarray:
    """The weight vector with the input normalisation x' = (x - mu) / sd."""
    w = np.array(w, dtype=np.float32, copy=True)
    w[:LF] = mu
    w[LF:2 * LF] = 1.0 / sd
    return w


def train_correction(system, steps: int = 20000, batch: int = 65536, lr: float = 2e-3, seed: int = 3,
                     init_seed: int = 1, group_stride: int = 1, samples: int = 4_000_000, gfloor: float = 0.0,
                     alpha: float = 0.5) -> dict:
    """Builds the training records of `system` (one GeonSystem, or a list of
    snapshots of the same distribution) at its current theta, resamples them
    and trains the network on the device.  Returns the weights (taking raw
    features), the per-step losses and the dataset size."""
    systems = list(system) if isinstance(system, (list, tuple)) else [system]
    parts = [s.learn_dataset(group_stride=group_stride, gfloor=gfloor) for s in systems]
    feat = np.concatenate([d["feat"] for d in parts])
    tg = np.concatenate([d["target"] for d in parts])
    ds = {"count": sum(int(d["count"]) for d in parts)}
    system = systems[0]
    x, t = resample(feat, tg, min(samples, max(len(feat), 1) * 4), seed=seed, alpha=alpha)
    mu = x.astype(np.float64).mean(0)
    sd = x.astype(np.float64).std(0)
    sd = np.where(sd > 1e-6, sd, 1.0)
    w0 = set_normalisation(init_weights(init_seed), mu, sd)
    w, hist = system.mlp_train(w0, x, t, steps=steps, batch=batch, lr=lr, seed=seed)
    return {"weights": w, "loss": hist, "records": int(ds["count"]),
            "samples": int(len(x)), "snapshots": len(systems)}
