"""Learned far-field correction on the GPU, through the C ABI.

* the tensor-core forward pass and gradient against the FP64 oracle of the
  network (oracle/mlp.py, BF16 roundings of training emulated): norm-wise
  relative error <= 5e-3 for outputs and <= 1e-2 for gradients.  Training
  rounds operands to BF16 exactly like the oracle; inference runs FP16
  operands and a packed FP16 GELU, so the output bar also covers the
  difference between the two roundings and the hardware tanh approximation;
* training on the device lowers the loss;
* the dataset: Barnes-Hut force + the exact residuals of every accepted
  (cell, target) pair reproduces the direct sum (<= 2e-5 RMS relative);
* the correction inside the force pass equals BH + sum of m * scale * net
  over the pairs (<= 5e-5 of the particle's force), and a trained net lowers
  the BH force error.
"""
import numpy as np
import pytest

from oracle import mlp as M
from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W
from physsim_gb300.system import GeonSystem
from tests.parity import STATE_KEYS

pytestmark = pytest.mark.gpu


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def feature_like(rng, n):
    """Samples shaped like the pair features (unit direction, small ratios)."""
    ph = rng.uniform(0, 2 * np.pi, n)
    x = np.zeros((n, M.LF))
    x[:, 0], x[:, 1] = np.cos(ph), np.sin(ph)
    x[:, 2] = rng.uniform(0.1, 0.9, n)
    x[:, 3] = rng.uniform(0.0, 0.5, n)
    x[:, 4:7] = rng.normal(0, 0.05, (n, 3))
    x[:, 7] = rng.uniform(0, 0.5, n)
    x[:, 8] = rng.uniform(0, 1, n)
    return x.astype(np.float32)


@pytest.fixture(scope="module")
def sys_small(gpu_lib):
    wl = W.small_disk(256, relativity=False, softening=8.0)
    g = GeonSystem(wl.params, wl.n)
    s = wl.state
    g.upload(*[s[k] for k in STATE_KEYS])
    yield g
    g.close()


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 70000])
def test_forward_matches_oracle(sys_small, n):
    rng = np.random.default_rng(n)
    w = M.init_weights(n)
    x = feature_like(rng, n)
    y = sys_small.mlp_forward(w, x)
    ref = M.forward(w, x, bf16_ops=True)
    assert np.isfinite(y).all()
    assert rel_norm(y, ref) <= 5e-3, rel_norm(y, ref)


@pytest.mark.parametrize("n", [128, 300, 5000])
def test_gradient_matches_oracle(sys_small, n):
    rng = np.random.default_rng(100 + n)
    w = M.init_weights(7)
    x = feature_like(rng, n)
    t = (rng.normal(size=(n, 2)) * 0.05).astype(np.float32)
    wt = rng.uniform(0.5, 2.0, n).astype(np.float32)
    g, loss = sys_small.mlp_grad(w, x, t, wt)
    gr, lr = M.loss_grad(w, x, t, wt, bf16_ops=True)
    assert abs(loss - lr) <= 5e-3 * lr, (loss, lr)
    parts = M.unpack(gr)
    gp = M.unpack(g)
    for k in parts:                        # each layer's gradient block on its own
        assert rel_norm(gp[k], parts[k]) <= 1e-2, (k, rel_norm(gp[k], parts[k]))
    # and against the FP64 network without BF16 roundings: same direction
    g64, _ = M.loss_grad(w, x, t, wt, bf16_ops=False)
    assert g @ g64 / np.linalg.norm(g) / np.linalg.norm(g64) > 0.999


def test_training_lowers_loss(sys_small):
    rng = np.random.default_rng(9)
    n = 20000
    x = feature_like(rng, n)
    # a smooth target of the features
    t = np.stack([0.1 * x[:, 2] ** 2 * x[:, 0] + 0.05 * x[:, 4], 0.1 * x[:, 2] ** 2 * x[:, 1] - 0.05 * x[:, 6]], 1)
    t = t.astype(np.float32)
    w0 = M.init_weights(11)
    _, l0 = M.loss_grad(w0, x, t, bf16_ops=True)
    w, hist = sys_small.mlp_train(w0, x, t, steps=600, batch=4096, lr=3e-3, seed=5)
    assert np.isfinite(hist).all() and np.isfinite(w).all()
    _, l1 = M.loss_grad(w, x, t, bf16_ops=True)
    assert l1 < 0.05 * l0, (l0, l1)
    assert hist[-50:].mean() < 0.1 * hist[:10].mean()


@pytest.fixture(scope="module")
def plummer(gpu_lib):
    wl = W.plummer_disk(65536, theta=0.7)
    s = wl.state
    g = GeonSystem(wl.params, wl.n)
    g.upload(*[s[k] for k in STATE_KEYS])
    test = np.sort(np.random.default_rng(21).choice(wl.n, 2048, replace=False)).astype(np.int32)
    dfx, dfy = g.direct_forces(test)
    yield wl, g, test, np.stack([dfx, dfy], 1).astype(np.float64)
    g.close()


def rms_rel(F, D):
    return float(np.sqrt(np.mean((np.linalg.norm(F - D, axis=1) / np.linalg.norm(D, axis=1)) ** 2)))


def bh_forces(g, test):
    g.compute_forces()
    f = g.forces()
    return np.stack([f["fx"][test], f["fy"][test]], 1).astype(np.float64)


def pair_sum(wl, test, ds, values):
    """sum over the pairs of target mass * scale * values, per test particle."""
    pos = {int(t): k for k, t in enumerate(test)}
    rows = np.array([pos[int(t)] for t in ds["target"]])
    c = values * ds["scales"][:, 0:1] * wl.state["mass"][ds["target"]][:, None]
    out = np.zeros((len(test), 2))
    np.add.at(out, rows, c)
    return out


def test_exact_residuals_recover_direct_sum(plummer):
    wl, g, test, D = plummer
    F = bh_forces(g, test)
    ds = g.learn_dataset(test, 4_000_000)
    assert 0 < ds["count"] <= 4_000_000
    m, q = wl.state["mass"][ds["target"]][:, None], wl.state["charge"][ds["target"]][:, None]
    res = ds["residual"].astype(np.float64)
    corr = res[:, 0:2] * ds["scales"][:, 0:1] * m + res[:, 2:4] * ds["scales"][:, 1:2] * q
    pos = {int(t): k for k, t in enumerate(test)}
    rows = np.array([pos[int(t)] for t in ds["target"]])
    tot = np.zeros((len(test), 2))
    np.add.at(tot, rows, corr)
    plain = rms_rel(F, D)
    exact = rms_rel(F + tot, D)
    assert plain > 1e-2                    # theta 0.7 is coarse
    assert exact <= 2e-5, (plain, exact)


def test_force_pass_correction_and_gain(plummer):
    wl, g, test, D = plummer
    F = bh_forces(g, test)
    plain = rms_rel(F, D)
    # training set from other targets
    train_t = np.sort(np.random.default_rng(22).choice(wl.n, 4096, replace=False)).astype(np.int32)
    tr = g.learn_dataset(train_t, 8_000_000)
    assert tr["count"] <= 8_000_000
    w, hist = g.mlp_train(M.init_weights(1), tr["feat_mass"], tr["residual"][:, 0:2], steps=1500, batch=16384,
                          lr=2e-3, seed=3)
    assert np.isfinite(w).all()
    # the force pass with the correction on
    p = g.params()
    p.flags |= N.FLAG_LEARN
    g.set_params(p)
    g.learn_set_weights(w)
    FL = bh_forces(g, test)
    g.learn_set_weights(None)
    p.flags &= ~N.FLAG_LEARN
    g.set_params(p)
    # the same correction assembled on the host from the dataset of the test targets
    te = g.learn_dataset(test, 4_000_000)
    y = g.mlp_forward(w, te["feat_mass"]).astype(np.float64)
    host = F + pair_sum(wl, test, te, y)
    # the device adds a few hundred corrections per particle with FP32 atomics
    # in no fixed order; relative to particles whose net force nearly
    # cancels, that rounding reaches about 1e-5
    scale = np.linalg.norm(D, axis=1)[:, None]
    assert np.max(np.abs(FL - host) / scale) <= 5e-5, np.max(np.abs(FL - host) / scale)
    learned = rms_rel(FL, D)
    assert learned < 0.5 * plain, (plain, learned)


def test_training_is_reproducible(sys_small):
    """The per-CTA gradients are summed in a fixed order: the same seed gives
    the same weights bit for bit."""
    rng = np.random.default_rng(12)
    x = feature_like(rng, 9000)
    t = (rng.normal(size=(9000, 2)) * 0.05).astype(np.float32)
    w0 = M.init_weights(2)
    a, ha = sys_small.mlp_train(w0, x, t, steps=50, batch=2048, lr=1e-3, seed=9)
    b, hb = sys_small.mlp_train(w0, x, t, steps=50, batch=2048, lr=1e-3, seed=9)
    assert np.array_equal(a, b) and np.array_equal(ha, hb)
