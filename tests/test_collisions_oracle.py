"""Merge collisions in the FP64 oracle (CPU only): known answers for
handleCollisions (src/collisions.js:24-158) as Physics.update runs it after
the tree rebuild (src/integrator.js:1350-1381), and the insertion-order rule
of QuadTreePool leaves that the GPU query reproduces.

Setup of the known-answer cases: no force toggles, so the one substep of a
frame only drifts the particles by w * dt before the tree is rebuilt and the
collisions run.
"""
import numpy as np
import pytest

from physsim_gb300 import _native as N

DT = 1e-6


def merge_sim(x, y, m, wx=None, wy=None, q=None, angw=None, anti=None, boundary=N.BOUND_DESPAWN, W=100.0):
    from oracle.oracle import OracleSim
    n = len(x)
    z = np.zeros(n)
    p = N.make_params(toggles=N.BARNES_HUT, boundary_mode=boundary, domain_w=W, domain_h=W,
                      collision_mode=N.COL_MERGE)
    o = OracleSim(p)
    o.add(np.asarray(x, float), np.asarray(y, float), z if wx is None else np.asarray(wx, float),
          z if wy is None else np.asarray(wy, float), np.asarray(m, float), z if q is None else np.asarray(q, float),
          z if angw is None else np.asarray(angw, float))
    if anti is not None:
        o.set_matter(antimatter=np.asarray(anti, np.int32))
    return o


def ke(m, wx, wy):
    w2 = wx * wx + wy * wy
    return w2 / (np.sqrt(1 + w2) + 1) * m


def test_pass_mode_keeps_overlaps(oracle_mod):
    o = merge_sim([50, 51], [50, 50], [1, 1])
    p = o.params
    p.collision_mode = N.COL_PASS
    o.set_params(p)
    o.update(DT)
    assert o.count() == 2 and len(o.collision_events()) == 0


def test_two_body_merge(oracle_mod):
    x, y, m = np.array([50.0, 52.0]), np.array([50.0, 50.0]), np.array([8.0, 1.0])
    wx, wy = np.array([0.1, -0.2]), np.array([0.0, 0.3])
    q, angw = np.array([0.3, -0.1]), np.array([0.05, -0.2])
    o = merge_sim(x, y, m, wx, wy, q, angw)
    o.update(DT)
    assert o.count() == 1
    s = o.state()
    x1, y1 = x + wx * DT, y + wy * DT                  # drift, relativity off: v = w
    M = m.sum()
    assert s["mass"][0] == M
    assert np.isclose(s["wx"][0], (m * wx).sum() / M, rtol=1e-15)
    assert np.isclose(s["wy"][0], (m * wy).sum() / M, rtol=1e-15)
    cx, cy = (m * x1).sum() / M, (m * y1).sum() / M
    assert np.isclose(s["x"][0], cx, rtol=1e-15) and np.isclose(s["y"][0], cy, rtol=1e-15)
    assert np.isclose(s["charge"][0], 0.2, rtol=1e-15)  # quantised to BOSON_CHARGE multiples
    # orbital + spin angular momentum about the merged centre becomes spin
    lorb = ((x1 - cx) * m * wy - (y1 - cy) * m * wx).sum()
    lspin = (0.4 * m * np.cbrt(m) ** 2 * angw).sum()
    assert np.isclose(s["angw"][0], (lorb + lspin) / (0.4 * M * np.cbrt(M) ** 2), rtol=1e-12)
    assert o.ids().tolist() == [2]
    assert o.matter()["base_mass"][0] == M
    ev = o.collision_events()
    assert ev.shape == (1, 6) and ev[0, 0] == 2
    ke_after = ke(M, s["wx"][0], s["wy"][0])
    assert np.isclose(ev[0, 3], ke(m, wx, wy).sum() - ke_after, rtol=1e-12)
    assert o.collision_counts() == {"merges": 1, "annihilations": 0, "spawned": 1, "removed": 2}


def test_equal_annihilation_removes_both(oracle_mod):
    o = merge_sim([50, 51], [50, 50], [2, 2], wx=[0.1, 0.0], anti=[0, 1])
    o.update(DT)
    assert o.count() == 0
    ev = o.collision_events()
    assert ev.shape == (1, 6) and ev[0, 0] == 1
    assert np.isclose(ev[0, 3], 2 * 2 + ke(2, 0.1, 0.0), rtol=1e-14)
    assert np.isclose(ev[0, 4], 0.1 * 2, rtol=1e-14)


def test_unequal_annihilation_shrinks_the_larger(oracle_mod):
    o = merge_sim([50, 52], [50, 50], [8, 1], anti=[0, 1])
    o.update(DT)
    assert o.count() == 1
    s, mt = o.state(), o.matter()
    assert s["mass"][0] == 7 and mt["base_mass"][0] == 7 and not mt["antimatter"][0]
    assert o.ids().tolist() == [0]


def test_periodic_merge_through_ghost(oracle_mod):
    o = merge_sim([0.5, 99.4], [50, 50], [1, 1], boundary=N.BOUND_LOOP)
    o.update(DT)
    assert o.count() == 1
    s = o.state()
    # min-image offset -1.1: merged centre at -0.05, wrapped into the domain
    assert np.isclose(s["x"][0], 99.95, rtol=0, atol=1e-9)


def test_merged_particle_keeps_merging(oracle_mod):
    """The reference does not re-check p1's mass inside its candidate loop:
    after A merges with B, the dead A 'merges' with C, which spawns a copy of C
    carrying A's charge a second time (collisions.js:37-91, 110-158)."""
    o = merge_sim([50, 50.5, 49.5], [50, 50, 50], [1, 1, 1], q=[0.1, 0.2, 0.3])
    o.update(DT)
    assert o.count() == 2
    s = o.state()
    assert s["mass"].tolist() == [2.0, 1.0]
    assert np.allclose(s["charge"], [0.3, 0.4], rtol=1e-15)
    assert o.ids().tolist() == [3, 4]


def test_dense_merging_conserves_mass_and_momentum(oracle_mod):
    rng = np.random.default_rng(4)
    n = 600
    x, y = rng.uniform(30, 70, n), rng.uniform(30, 70, n)
    m = rng.lognormal(0, 0.5, n)
    wx, wy = rng.normal(0, 0.05, (2, n))
    o = merge_sim(x, y, m, wx, wy)
    o.update(DT)
    c = o.collision_counts()
    assert c["merges"] > 20
    s = o.state()
    assert o.count() == n - c["removed"] + c["spawned"]
    assert np.isclose(s["mass"].sum(), m.sum(), rtol=1e-13)
    # merges conserve proper momentum m * w; only the 'keeps merging' copies break it
    assert np.isclose(o.matter()["base_mass"].sum(), m.sum(), rtol=1e-13)


def _rule_leaf_orders(px, py, cx, cy, hw, hh):
    """Leaf storage orders implied by QuadTreePool.insert (quadtree.js:185-237)
    for points inserted in index order: a node that receives its fifth point
    divides; that point descends first and the four stored points follow
    from the work stack in reverse, so every child sees, in order, the members
    of [a4, a3, a2, a1, a0] and then the later arrivals a5, a6, ..."""
    leaves = []

    def rec(seq, cx, cy, hw, hh):
        if len(seq) <= 4:
            leaves.append(seq)
            return
        order = seq[:5][::-1] + seq[5:]
        kids = [[], [], [], []]
        for q in order:
            kids[(0 if px[q] <= cx else 1) + (0 if py[q] <= cy else 2)].append(q)
        qw, qh = hw / 2, hh / 2
        centres = [(cx - qw, cy - qh), (cx + qw, cy - qh), (cx - qw, cy + qh), (cx + qw, cy + qh)]
        for d in range(4):
            if kids[d]:
                rec(kids[d], centres[d][0], centres[d][1], qw, qh)

    inside = [i for i in range(len(px)) if cx - hw <= px[i] <= cx + hw and cy - hh <= py[i] <= cy + hh]
    rec(inside, cx, cy, hw, hh)
    return leaves


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_leaf_insertion_order_rule(oracle_mod, seed):
    from oracle.oracle import OracleSim
    rng = np.random.default_rng(seed)
    n = 3000
    centres = rng.uniform(20, 80, (12, 2))
    k = rng.integers(0, 12, n)
    x = centres[k, 0] + rng.normal(0, 1.5, n)
    y = centres[k, 1] + rng.normal(0, 1.5, n)
    o = OracleSim(N.make_params(toggles=N.BARNES_HUT | N.GRAVITY))
    z = np.zeros(n)
    o.add(x, y, z, z, np.ones(n), z, z)
    npts, _ = o.build_tree()
    assert npts == n
    slots = o.leaf_slots(n)
    leaves = _rule_leaf_orders(x, y, 50.0, 50.0, 200.0, 200.0)
    multi = 0
    for seq in leaves:
        assert [int(slots[q]) for q in seq] == list(range(len(seq)))
        multi += len(seq) > 1 and seq != sorted(seq)
    assert multi > 50          # many leaves are not in plain index order
