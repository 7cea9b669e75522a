"""CPU checks of the network oracle (oracle/mlp.py): BF16 rounding known
answers and the analytic FP64 gradient against central finite differences."""
import numpy as np

from oracle import mlp as M


def test_bf16_rounding_known_answers():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e38, 1.0e-40, 0.0], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # tie -> even mantissa
    assert r[2] == 1.0 + 2.0 ** -6           # tie -> even mantissa (upwards)
    assert r[3] == -2.5
    assert np.isfinite(r[4]) and abs(r[4] / 3.0e38 - 1) < 2 ** -8
    assert abs(r[5] - 1.0e-40) <= 2.0 ** -133
    assert r[6] == 0.0
    # every BF16 value is a fixed point
    b = M.bf16(np.random.default_rng(0).normal(size=1000))
    assert np.array_equal(M.bf16(b), b)


def test_exact_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    w = M.init_weights(3).astype(np.float64)
    w[:M.LF] = rng.normal(size=M.LF) * 0.1                 # a normalisation that is not the identity
    w[M.LF:2 * M.LF] = rng.uniform(0.5, 2.0, M.LF)
    x = rng.normal(size=(48, M.LF))
    t = M.random_targets(rng, 48)
    wt = rng.uniform(0.5, 2.0, size=48)
    g, loss = M.loss_grad(w, x, t, wt, bf16_ops=False)
    assert np.isfinite(loss) and loss > 0
    idx = rng.choice(np.arange(2 * M.LF, M.NPARAM), 60, replace=False)
    idx = np.concatenate([idx, [M.NPARAM - 1, M.NPARAM - 2, 2 * M.LF + M.LH * M.LF]])   # b3 and b1[0]
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        lp = M.loss_grad(wp, x, t, wt, bf16_ops=False)[1]
        lm = M.loss_grad(wm, x, t, wt, bf16_ops=False)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_gradient_close_to_exact():
    rng = np.random.default_rng(6)
    w = M.init_weights(4)
    x = rng.normal(size=(512, M.LF))
    t = M.random_targets(rng, 512)
    g64, _ = M.loss_grad(w, x, t, bf16_ops=False)
    g16, _ = M.loss_grad(w, x, t, bf16_ops=True)
    cos = g64 @ g16 / np.linalg.norm(g64) / np.linalg.norm(g16)
    assert cos > 0.999
