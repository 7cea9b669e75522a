"""Known-answer tests of the FP64 oracle (CPU only).

The reference ships no tests or golden vectors, so the oracle is anchored by
answers derived from first principles for the formulas it restates
(src/forces.js, src/signal-delay.js, src/topology.js, src/quadtree.js,
src/integrator.js), and by structural invariants of the reference tree.
"""
import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W


def sim(params, x, y, wx=None, wy=None, m=None, q=None, angw=None, threads=1):
    from oracle.oracle import OracleSim
    n = len(x)
    z = np.zeros(n)
    o = OracleSim(params, threads=threads)
    o.add(np.asarray(x, float), np.asarray(y, float), z if wx is None else wx, z if wy is None else wy,
          np.ones(n) if m is None else m, z if q is None else q, z if angw is None else angw)
    return o


def test_gravity_two_body_softened(oracle_mod):
    eps = 1.5
    o = sim(N.make_params(toggles=N.GRAVITY, softening=eps), [10, 13], [20, 24], m=[2.0, 3.0])
    o.compute_forces()
    f = o.forces()
    r2 = 25 + eps * eps
    expect = 2 * 3 / r2 ** 1.5 * np.array([3.0, 4.0])
    assert np.allclose([f["fx"][0], f["fy"][0]], expect, rtol=1e-14)
    assert np.allclose([f["fx"][1], f["fy"][1]], -expect, rtol=1e-14)
    assert np.isclose(o.pe(), -6 / np.sqrt(r2), rtol=1e-14)


def test_coulomb_like_charges_repel(oracle_mod):
    o = sim(N.make_params(toggles=N.COULOMB, softening=1.0), [0, 2], [0, 0], q=[0.5, 0.3])
    o.compute_forces()
    f = o.forces()
    assert f["fx"][0] < 0 and f["fx"][1] > 0
    assert np.isclose(f["fx"][0], -0.15 * 2 / 5 ** 1.5, rtol=1e-14)


def test_yukawa_force_and_cutoff(oracle_mod):
    mu, eps = 0.15, 1.0
    for d, inside in ((10.0, True), (6 / mu + 0.5, False)):
        o = sim(N.make_params(toggles=N.YUKAWA, softening=eps, yukawa_mu=mu), [0, d], [0, 0], m=[2.0, 1.5])
        o.compute_forces()
        f = o.forces()
        r = np.sqrt(d * d + eps * eps)
        expect = 14 * 3 * np.exp(-mu * r) * (1 / r ** 2 + mu / r) / r * d if inside else 0.0
        assert np.isclose(f["fx"][0], expect, rtol=1e-13, atol=0.0)


def test_aligned_magnetic_dipoles_repel(oracle_mod):
    p = N.make_params(toggles=N.MAGNETIC, softening=1.0)
    o = sim(p, [0, 3], [0, 0], m=[1.0, 1.0], q=[1.0, 1.0], angw=[0.5, 0.5])
    o.set_forces_init(False)
    o.update(1e-9)            # bootstrap caches angVel and moments, then one tiny substep
    o.compute_forces()
    f = o.forces()
    assert f["mag_x"][0] < 0 < f["mag_x"][1]


def test_min_image_torus_antisymmetric_and_bounded(oracle_mod):
    rng = np.random.default_rng(0)
    W_, H_ = 400.0, 300.0
    for _ in range(200):
        a = rng.random(2) * [W_, H_]
        b = rng.random(2) * [W_, H_]
        d1 = oracle_mod.min_image(a[0], a[1], b[0], b[1], N.TORUS, W_, H_)
        d2 = oracle_mod.min_image(b[0], b[1], a[0], a[1], N.TORUS, W_, H_)
        assert np.allclose(d1, -d2, atol=1e-12)
        assert abs(d1[0]) <= W_ / 2 + 1e-12 and abs(d1[1]) <= H_ / 2 + 1e-12


def test_min_image_klein_rp2_not_longer_than_direct(oracle_mod):
    rng = np.random.default_rng(1)
    for topo in (N.KLEIN, N.RP2):
        for _ in range(100):
            a = rng.random(2) * 100
            b = rng.random(2) * 100
            d = oracle_mod.min_image(a[0], a[1], b[0], b[1], topo, 100.0, 100.0)
            assert np.hypot(*d) <= np.hypot(*(b - a)) + 1e-12


def test_boris_rotation_preserves_speed(oracle_mod):
    """Pure uniform Bz: the Boris rotation keeps |w| exactly (integrator.js:900-915)."""
    p = N.make_params(toggles=N.MAGNETIC | N.RELATIVITY, ext_bz=2.0, boundary_mode=N.BOUND_LOOP,
                      domain_w=1000, domain_h=1000, softening=8.0)
    o = sim(p, [500.0], [500.0], wx=[0.3], wy=[0.1], m=[1.0], q=[1.0])
    w0 = np.hypot(0.3, 0.1)
    for _ in range(50):
        o.update(1 / 60)
    s = o.state()
    assert np.isclose(np.hypot(s["wx"][0], s["wy"][0]), w0, rtol=1e-12)
    assert o.last_substeps() >= 1


def test_light_cone_solution_on_straight_history(oracle_mod):
    """signal-delay.js: the returned point satisfies |x(t_r) - x_obs| = now - t_r."""
    p = N.make_params(toggles=N.GRAVITY | N.RELATIVITY, domain_w=1000, domain_h=1000)
    v = np.array([0.4, -0.2])
    g = 1 / np.sqrt(1 - v @ v)
    o = sim(p, [500.0, 530.0], [500.0, 520.0], wx=[v[0] * g, 0], wy=[v[1] * g, 0])
    times = 100.0 - np.arange(64)[::-1] * 1.0
    X = np.stack([500.0 + v[0] * (times - 100.0), np.full(64, 530.0)])
    Y = np.stack([500.0 + v[1] * (times - 100.0), np.full(64, 520.0)])
    VX = np.stack([np.full(64, v[0]), np.zeros(64)])
    VY = np.stack([np.full(64, v[1]), np.zeros(64)])
    o.upload_history(times, X, Y, VX, VY, np.zeros((2, 64)))
    o.set_sim_time(100.0)
    r = o.delayed_state(0, 530.0, 520.0)
    assert r is not None
    t_r = 100.0 + (r[0] - 500.0) / v[0]
    assert np.isclose(np.hypot(r[0] - 530.0, r[1] - 520.0), 100.0 - t_r, rtol=1e-12)
    assert np.isclose(r[1], 500.0 + v[1] * (t_r - 100.0), rtol=1e-12)
    assert np.allclose(r[2:4], v, rtol=1e-12)


def test_signal_delay_needs_two_samples(oracle_mod):
    p = N.make_params(toggles=N.GRAVITY | N.RELATIVITY | N.BARNES_HUT)
    o = sim(p, [10, 12], [10, 10], m=[1.0, 1.0])
    o.compute_forces()
    # cold history: leaf sources are skipped (forces.js:653)
    assert o.forces()["fx"][0] == 0.0


def _tree_leaves_by_point(o):
    npts, _ = o.build_tree()
    lop, bx, by, bw, lv = o.leaves(npts)
    return [None if l < 0 else (bx[l], by[l], bw[l], lv[l]) for l in lop]


def test_tree_capacity_and_order_independence(oracle_mod):
    wl = W.small_disk(3000, relativity=False, softening=8.0)
    s = wl.state
    keys = ("x", "y", "wx", "wy", "mass", "charge", "angw")
    o = sim(wl.params, *[s[k] for k in keys[:2]])
    sig = _tree_leaves_by_point(o)
    counts = {}
    for t in sig:
        counts[t] = counts.get(t, 0) + 1
    assert max(counts.values()) <= 4
    perm = np.random.default_rng(7).permutation(wl.n)
    o2 = sim(wl.params, s["x"][perm], s["y"][perm])
    sig2 = _tree_leaves_by_point(o2)
    assert [sig[i] for i in perm] == sig2


def test_tree_divided_iff_more_than_four(oracle_mod):
    wl = W.small_disk(1500, relativity=False)
    o = sim(wl.params, wl.state["x"], wl.state["y"], m=wl.state["mass"])
    npts, _ = o.build_tree()
    nodes = o.tree_nodes()
    lop, *_ = o.leaves(npts)
    # a divided node's children hold all its points; leaves hold <= 4
    assert np.all(nodes["count"][nodes["divided"] == 0] <= 4)
    assert np.isclose(nodes["mass"][0], wl.state["mass"].sum(), rtol=1e-12)


def test_points_outside_root_box_are_dropped(oracle_mod):
    p = N.make_params(domain_w=100, domain_h=100)
    # root box is centre (50, 50), half-size 200: [-150, 250]^2
    o = sim(p, [10.0, 260.0, -150.0, 250.0], [10.0, 10.0, 10.0, 10.0])
    npts, _ = o.build_tree()
    lop, *_ = o.leaves(npts)
    assert list(lop >= 0) == [True, False, True, True]


def test_tie_goes_north_west(oracle_mod):
    """quadtree.js:175-179: px <= cx -> west, py <= cy -> north."""
    p = N.make_params(domain_w=100, domain_h=100)
    xs = [50.0, 50.0, 10, 20, 30]
    ys = [50.0, 60.0, 70, 80, 90]
    o = sim(p, xs, ys)
    npts, _ = o.build_tree()
    lop, bx, by, bw, lv = o.leaves(npts)
    assert bx[lop[0]] < 50 and by[lop[0]] < 50      # (50, 50) on both ties -> NW child
    assert bx[lop[1]] < 50 and by[lop[1]] > 50      # x tie -> west, y > cy -> south


def test_despawn_removes_far_particles(oracle_mod):
    p = N.make_params(toggles=N.GRAVITY, domain_w=100, domain_h=100)
    o = sim(p, [50.0, 170.0], [50.0, 50.0])
    o.update(1 / 60)
    assert o.count() == 1
    assert list(o.ids()) == [0]


def test_torus_wrap_keeps_particle_in_box(oracle_mod):
    p = N.make_params(toggles=N.GRAVITY, domain_w=100, domain_h=100, boundary_mode=N.BOUND_LOOP)
    o = sim(p, [99.99], [0.001], wx=[1.0], wy=[-1.0])
    o.update(1 / 60)
    s = o.state()
    assert 0 <= s["x"][0] <= 100 and 0 <= s["y"][0] <= 100


def test_kepler_energy_drift_small(oracle_mod):
    p = N.make_params(toggles=N.GRAVITY, domain_w=1000, domain_h=1000, softening=0.01, flags=N.FLAG_PE)
    m1, m2, a = 100.0, 1.0, 20.0
    v = np.sqrt(m1 / a)
    g = 1.0
    o = sim(p, [500.0, 520.0], [500.0, 500.0], wx=[0.0, 0.0], wy=[-v * m2 / m1, v], m=[m1, m2])
    o.compute_forces()
    s0 = o.stats()
    e0 = s0["linear_ke"] + o.pe()
    for _ in range(120):
        o.update(1 / 30)
    e1 = o.stats()["linear_ke"] + o.pe()
    assert abs(e1 - e0) / abs(e0) < 1e-3


def test_periodic_bh_counts_each_image(oracle_mod):
    """Reference quirk: with ghosts in the tree and min-image in pairForce,
    a source is counted once per copy of it the walk reaches
    (integrator.js:248-257, forces.js:165-167)."""
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, boundary_mode=N.BOUND_LOOP, domain_w=100, domain_h=100,
                      softening=1.0)
    o = sim(p, [40.0, 60.0], [50.0, 50.0], m=[1.0, 1.0])
    o.compute_forces()
    f_bh = o.forces()["fx"][0]
    pd = N.make_params(toggles=N.GRAVITY, boundary_mode=N.BOUND_LOOP, domain_w=100, domain_h=100, softening=1.0)
    od = sim(pd, [40.0, 60.0], [50.0, 50.0], m=[1.0, 1.0])
    od.compute_forces()
    f_direct = od.forces()["fx"][0]
    ghosts = o.ghost_origins()
    copies_of_1 = 1 + int(np.sum(ghosts == 1))
    assert np.isclose(f_bh, copies_of_1 * f_direct, rtol=1e-12)


# ---- hand-traced control flow of the reference ------------------------------------------
# integrator.js:862-870: dtSafe = sqrt(softening / aMax), stepsNeeded =
# min(ceil(dtRemain / dtSafe), budget), dtSub = dtRemain / stepsNeeded.  One
# unit mass in a uniform field g = 4096 (angle 0: force (4096, 0) exactly),
# softening 1, dt = 1/16: dtSafe = 1/64 exactly, dtRemain / dtSafe = 4 exactly,
# so ceil gives 4 (not 5) and the later substeps (lagged aMax, the same field)
# take 3, 2, 1 of the remaining quarters: 4 substeps.  With g = 4096 (1 + 2^-20)
# the ratio is 4 (1 + 2^-21) and ceil gives 5; the next ratio is
# (4/5) / (1 - 2^-21) * 4 = 3.2..., ceil 4, and so on: 5 substeps.
PLANNER_CASES = ((4096.0, 4), (4096.0 * (1 + 2.0 ** -20), 5), (4096.0 * (1 - 2.0 ** -20), 4))


@pytest.mark.parametrize("g,expect", PLANNER_CASES)
def test_planner_ceil_at_exact_multiples(oracle_mod, g, expect):
    p = N.make_params(toggles=N.GRAVITY, softening=1.0, domain_w=1000, domain_h=1000, ext_gravity=g)
    o = sim(p, [100.0], [500.0])
    assert o.update(1 / 16) == expect


# forces.js:82-83, 387: the Yukawa term applies when the unsoftened r^2 is
# strictly below (6 / mu)^2.  mu = 0.75 makes the cutoff 8 exactly: at a
# separation of exactly 8 there is no Yukawa force, one ulp-scale step closer
# (8 - 2^-40) there is the full term.
YUKAWA_TIE_MU, YUKAWA_TIE_EPS = 0.75, 1.0


def yukawa_expect(d, mu=YUKAWA_TIE_MU, eps=YUKAWA_TIE_EPS, m1=2.0, m2=1.5):
    r = np.sqrt(d * d + eps * eps)
    return 14 * m1 * m2 * np.exp(-mu * r) * (1 / r ** 2 + mu / r) / r * d


@pytest.mark.parametrize("d,inside", [(8.0, False), (8.0 - 2.0 ** -40, True), (8.0 + 2.0 ** -40, False)])
def test_yukawa_cutoff_tie(oracle_mod, d, inside):
    p = N.make_params(toggles=N.YUKAWA, softening=YUKAWA_TIE_EPS, yukawa_mu=YUKAWA_TIE_MU,
                      domain_w=1000, domain_h=1000)
    o = sim(p, [100.0, 100.0 + d], [500.0, 500.0], m=[2.0, 1.5])
    o.compute_forces()
    fx = o.forces()["fx"][0]
    if inside:
        assert np.isclose(fx, yukawa_expect(d), rtol=1e-12, atol=0.0)
    else:
        assert fx == 0.0


# integrator.js:866-869: the cyclotron limit dtCyc = (pi/4) / wc, wc = |q| |Bz| / m
# (external Bz 50.25 on a unit charge and mass; no force, so dtSafe starts
# at dtRemain).  dt = 4 dtCyc exactly (a power-of-two multiple): ceil gives 4;
# one ulp-scale step longer gives 5.
CYC_BZ = 50.25
CYC_DT = 4 * (0.7853981633974483 / CYC_BZ)


@pytest.mark.parametrize("dt,expect", [(CYC_DT, 4), (CYC_DT * (1 + 2.0 ** -40), 5)])
def test_planner_cyclotron_limit(oracle_mod, dt, expect):
    p = N.make_params(toggles=N.GRAVITY, softening=1.0, domain_w=1000, domain_h=1000, ext_bz=CYC_BZ)
    o = sim(p, [500.0], [500.0], q=[1.0])
    assert o.update(dt) == expect


@pytest.mark.parametrize("order,dropped,level", [("forward", 5, 67), ("reversed", 0, 69)])
def test_relative_depth_guard_drops_deep_insert(oracle_mod, order, dropped, level):
    """quadtree.js:207-234: the insert's depth count starts at 0 for every
    (node, point) pair popped from its work stack, and a point that is still
    descending after 49 steps is left out of the tree (the loop ends without
    storing it).  Six points one FP64 ulp apart near (0.001, 0.002), root box
    [-150, 250]^2: the first five build a chain of divided nodes by the
    re-insert cascade (each pop descends one or two levels) until level 67
    separates them (level 69 for the last five, inserted in reverse); the
    sixth, inserted from the root, is still descending at step 49 and is
    dropped.  So the leaves hold five points at that level, the root's
    aggregate mass is 5, and the dropped point is whichever comes last in
    insertion order."""
    p = N.make_params(domain_w=100, domain_h=100)
    xs = [0.001]
    for _ in range(5):
        xs.append(float(np.nextafter(xs[-1], 1.0)))
    idx = list(range(6)) if order == "forward" else list(range(5, -1, -1))
    o = sim(p, [xs[i] for i in idx], [0.002] * 6)
    npts, nn = o.build_tree()
    assert npts == 6 and nn == 1 + 4 * level
    lop, bx, by, bw, lv = o.leaves(npts)
    gone = [idx[k] for k in range(6) if lop[k] < 0]
    assert gone == [dropped]
    assert set(lv[lop[lop >= 0]]) == {level}
    assert o.tree_nodes()["mass"][0] == 5.0


# An exact tie of the opening test (forces.js:680, size^2 < theta^2 d^2, strict):
# a cluster of total mass 8 centred at (6.25, 6.25), the centre of the
# level-5 cell [0, 12.5]^2 of the root box [-150, 250]^2 (size 12.5), and a
# target 25 away on the x axis, so at theta 0.5 both sides are 156.25.
TIE_X = [5.25, 7.25, 5.25, 7.25, 6.25, 31.25]
TIE_Y = [5.25, 5.25, 7.25, 7.25, 6.25, 6.25]
TIE_M = [1.0, 1.0, 1.0, 1.0, 4.0, 1.0]


@pytest.mark.parametrize("theta,inter", [(0.4999999, 30), (0.5, 30), (0.5000001, 26)])
def test_opening_test_tie_opens(oracle_mod, theta, inter):
    """At the tie the node is opened: the target takes the cluster's five
    points from four level-6 leaves instead of one aggregate (4 more
    interactions); just above the tie it takes the aggregate.  Every other
    decision of the six walks is far from a tie."""
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, domain_w=100, domain_h=100, theta=theta)
    o = sim(p, TIE_X, TIE_Y, m=np.array(TIE_M))
    o.compute_forces()
    assert o.interactions() == inter
