"""Known answers of the oracle's potential heat map (heatmap.js): one
particle's potentials in closed form, tree walk against the pairwise sum,
and the 3 x 3 box blur."""
import numpy as np

from physsim_gb300 import _native as N

KEYS = ("x", "y", "wx", "wy", "mass", "charge", "angw")


def one_particle(bh):
    from oracle.oracle import OracleSim
    tg = N.GRAVITY | N.COULOMB | N.YUKAWA | (N.BARNES_HUT if bh else 0)
    p = N.make_params(toggles=tg, boundary_mode=N.BOUND_DESPAWN, domain_w=100.0, domain_h=100.0, softening=2.0,
                      yukawa_mu=0.15)
    o = OracleSim(p)
    o.add(*[np.array([v]) for v in (37.5, 61.25, 0.0, 0.0, 2.0, 0.3, 0.0)])
    return o


def test_single_particle_closed_form():
    G = 8
    for bh in (False, True):
        o = one_particle(bh)
        h = o.heatmap(0.0, 0.0, 12.5, 12.5, G, blur=False)
        c = (np.arange(G) + 0.5) * 12.5
        X, Y = np.meshgrid(c, c)
        r2 = (37.5 - X) ** 2 + (61.25 - Y) ** 2 + 4.0
        inv = 1 / np.sqrt(r2)
        r = 1 / inv
        np.testing.assert_allclose(h["gravity"], -2.0 * inv, rtol=1e-14)
        np.testing.assert_allclose(h["electric"], 0.3 * inv, rtol=1e-14)
        yk = -14 * 2.0 * np.exp(-0.15 * r) * inv
        if not bh:                                   # the pairwise branch cuts at (6 / mu)^2 = 40^2
            yk = np.where(r2 < 40.0 ** 2, yk, 0.0)
        np.testing.assert_allclose(h["yukawa"], yk, rtol=1e-13)
        o.close()


def test_tree_walk_close_to_pairwise_at_small_theta():
    from oracle.oracle import OracleSim
    from physsim_gb300 import workloads as W
    wl = W.small_disk(700, relativity=False, softening=8.0)
    out = {}
    for bh in (True, False):
        p = N.make_params(toggles=N.GRAVITY | N.COULOMB | (N.BARNES_HUT if bh else 0), boundary_mode=N.BOUND_DESPAWN,
                          domain_w=100.0, domain_h=100.0, theta=0.05, softening=8.0)
        o = OracleSim(p)
        o.add(*[wl.state[k] for k in KEYS])
        out[bh] = o.heatmap(0.0, 0.0, 100 / 32, 100 / 32, 32, blur=False)
        o.close()
    for k in ("gravity", "electric"):
        err = np.linalg.norm(out[True][k] - out[False][k]) / np.linalg.norm(out[False][k])
        assert err < 1e-3, (k, err)


def test_blur_keeps_constants_and_spreads_a_point():
    from oracle.oracle import OracleSim
    o = one_particle(False)
    G = 16
    raw = o.heatmap(0.0, 0.0, 100 / G, 100 / G, G, blur=False)["gravity"]
    sm = o.heatmap(0.0, 0.0, 100 / G, 100 / G, G, blur=True)["gravity"]
    # interior: mean of the 3 x 3 neighbourhood; corner: clamp to edge
    np.testing.assert_allclose(sm[5, 7], raw[4:7, 6:9].mean(), rtol=1e-13)
    pad = np.pad(raw, 1, mode="edge")
    np.testing.assert_allclose(sm[0, 0], pad[0:3, 0:3].mean(), rtol=1e-13)
    o.close()
