"""Merge collisions on the GPU (GeonParams.collision_mode = GEON_COL_MERGE)
against the FP64 oracle's restatement of handleCollisions
(src/collisions.js:24-158, src/integrator.js:1350-1381).

Bars:
* the discrete outcome is identical: particle count, ids (spawn ids record
  the order the pairs were resolved in), antimatter flags, event types;
* continuous quantities within FP32 storage: positions 1e-6 of the box, masses
  and base masses 1e-6 of the largest (an annihilation of nearly equal masses
  leaves a small difference of two rounded numbers), proper velocity and spin
  1e-5 of their scale, charges to 1e-6 (multiples of 0.1), event energies
  1e-5 of the largest;
* merge events whose lost energy is at the rounding level of the energies
  (below 1e-12 of the largest event) are left out on both sides: a particle
  that already merged away "merges" again with no velocity change, which
  loses exactly zero in FP32 state and +-1 ulp in the FP64 reference, and
  the reference emits an event only for a positive loss;
* forces after a frame whose last substep merged (removed particles act as
  sources through the tree) within the force-parity bar (1e-5 norm-wise).
The inputs are rounded to FP32 so both sides start from the same numbers.
"""
import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W
from physsim_gb300.system import GeonSystem
from tests.parity import STATE_KEYS, vec_err

pytestmark = pytest.mark.gpu

DT = 1e-6


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def setup(params, st, anti=None, capacity=None, history=None):
    from oracle.oracle import OracleSim
    st = {k: f32(st[k]) for k in STATE_KEYS}
    n = len(st["x"])
    g = GeonSystem(params, capacity or n)
    g.upload(*[st[k] for k in STATE_KEYS])
    o = OracleSim(params, threads=8)
    o.add(*[st[k] for k in STATE_KEYS])
    if anti is not None:
        g.set_matter(antimatter=anti)
        o.set_matter(antimatter=anti)
    if history is not None:
        times, X, Y, VX, VY, A = history
        g.upload_history(times, X, Y, VX, VY, A)
        o.upload_history(times, X, Y, VX, VY, A)
        g.set_sim_time(float(times[-1]))
        o.set_sim_time(float(times[-1]))
    return g, o


def compare(g, o, box=100.0):
    assert g.count() == o.count(), (g.count(), o.count())
    assert np.array_equal(g.ids(), o.ids())
    ci, co = g.collision_info(), o.collision_counts()
    for k in ("merges", "annihilations", "spawned", "removed"):
        assert ci[k] == co[k], (k, ci, co)
    assert ci["order_approx"] == 0
    sg, so = g.state(f64=True), o.state()
    if o.count():
        for k in ("x", "y"):
            assert np.max(np.abs(sg[k] - so[k])) <= 1e-6 * box, k
        assert np.max(np.abs(sg["mass"] - so["mass"])) <= 1e-6 * np.max(so["mass"])
        assert np.allclose(sg["charge"], so["charge"], rtol=0, atol=1e-6)
        for k in ("wx", "wy", "angw"):
            scale = max(np.max(np.abs(so[k])), 1e-12)
            assert np.max(np.abs(sg[k] - so[k])) <= 1e-5 * scale, k
        mg, mo = g.matter(), o.matter()
        assert np.array_equal(mg["antimatter"], mo["antimatter"])
        assert np.max(np.abs(mg["base_mass"] - mo["base_mass"])) <= 1e-6 * np.max(mo["base_mass"])
    eg, eo = significant(g.collision_events()), significant(o.collision_events())
    assert eg.shape == eo.shape
    if len(eo):
        # an annihilation of a particle that already merged away has energy
        # 0/0 in the reference (collisions.js:66-68): NaN on both sides
        assert np.array_equal(eg[:, 0], eo[:, 0])
        assert np.array_equal(np.isnan(eg), np.isnan(eo))
        fin = ~np.isnan(eo[:, 3])
        assert np.max(np.abs(eg[:, 1:3] - eo[:, 1:3])) <= 1e-6 * box
        escale = max(np.max(np.abs(eo[fin, 3]), initial=0.0), 1e-30)
        assert np.max(np.abs(eg[fin, 3] - eo[fin, 3]), initial=0.0) <= 1e-5 * escale
        pscale = max(np.max(np.abs(eo[:, 4:6])), 1e-30)
        assert np.max(np.abs(eg[:, 4:6] - eo[:, 4:6])) <= 1e-5 * pscale
    return ci


def significant(ev):
    if not len(ev):
        return ev
    top = np.nanmax(np.abs(ev[:, 3]), initial=0.0)
    keep = (ev[:, 0] != 2) | (ev[:, 3] > 1e-12 * top)
    return ev[keep]


def params(toggles=N.BARNES_HUT, boundary=N.BOUND_DESPAWN, topology=N.TORUS, W_=100.0, **kw):
    return N.make_params(toggles=toggles, boundary_mode=boundary, topology=topology, domain_w=W_, domain_h=W_,
                         collision_mode=N.COL_MERGE, **kw)


def state_of(x, y, m, wx=None, wy=None, q=None, angw=None):
    n = len(x)
    z = np.zeros(n)
    return {"x": np.asarray(x, float), "y": np.asarray(y, float), "mass": np.asarray(m, float),
            "wx": z if wx is None else np.asarray(wx, float), "wy": z if wy is None else np.asarray(wy, float),
            "charge": z if q is None else np.asarray(q, float), "angw": z if angw is None else np.asarray(angw, float)}


CASES = {
    "two_body": (params(), state_of([50, 52], [50, 50], [8, 1], [0.1, -0.2], [0, 0.3], [0.3, -0.1], [0.05, -0.2]), None),
    "equal_annihilation": (params(), state_of([50, 51], [50, 50], [2, 2], [0.1, 0]), [0, 1]),
    "unequal_annihilation": (params(), state_of([50, 52], [50, 50], [8, 1]), [0, 1]),
    "periodic_ghost": (params(boundary=N.BOUND_LOOP), state_of([0.5, 99.4], [50, 50], [1, 1]), None),
    "klein_edge": (params(boundary=N.BOUND_LOOP, topology=N.KLEIN),
                   state_of([30, 70.2], [0.3, 99.5], [1, 1], [0.05, 0.0], [0.0, 0.02], None, [0.1, 0.0]), None),
    "rp2_corner": (params(boundary=N.BOUND_LOOP, topology=N.RP2),
                   state_of([0.4, 99.3], [30, 70.1], [1, 1], [0.0, 0.03], [0.02, 0.0], None, [0.0, 0.2]), None),
    "keeps_merging": (params(), state_of([50, 50.5, 49.5], [50, 50, 50], [1, 1, 1], q=[0.1, 0.2, 0.3]), None),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_known_cases_match_oracle(gpu_lib, oracle_mod, case):
    p, st, anti = CASES[case]
    g, o = setup(p, st, None if anti is None else np.asarray(anti, np.int32))
    g.update(DT)
    o.update(DT)
    ci = compare(g, o)
    assert ci["merges"] + ci["annihilations"] > 0
    g.close()


def dense(n=600, seed=4, box=40.0, lo=30.0, anti_frac=0.0, W_=100.0, spread_all=False):
    rng = np.random.default_rng(seed)
    if spread_all:
        x, y = rng.uniform(0, W_, n), rng.uniform(0, W_, n)
    else:
        x, y = rng.uniform(lo, lo + box, n), rng.uniform(lo, lo + box, n)
    m = rng.lognormal(0, 0.5, n)
    wx, wy = rng.normal(0, 0.05, (2, n))
    q = rng.integers(-3, 4, n) * 0.1
    angw = rng.normal(0, 0.1, n)
    anti = (rng.random(n) < anti_frac).astype(np.int32)
    return state_of(x, y, m, wx, wy, q, angw), anti


@pytest.mark.parametrize("bh", [True, False])
def test_dense_merging_no_forces(gpu_lib, oracle_mod, bh):
    st, anti = dense(anti_frac=0.2)
    p = params(toggles=N.BARNES_HUT if bh else 0)
    g, o = setup(p, st, anti)
    g.update(DT)
    o.update(DT)
    ci = compare(g, o)
    assert ci["merges"] > 50 and ci["annihilations"] > 10
    # several candidates in one leaf: the insertion-order rule decided the order
    assert ci["candidates"] > ci["merges"] + ci["annihilations"]
    g.close()


@pytest.mark.parametrize("topology", [N.TORUS, N.KLEIN, N.RP2])
def test_periodic_merging_whole_box(gpu_lib, oracle_mod, topology):
    st, anti = dense(n=3000, seed=7, anti_frac=0.1, spread_all=True)
    p = params(boundary=N.BOUND_LOOP, topology=topology)
    g, o = setup(p, st, anti)
    g.update(DT)
    o.update(DT)
    ci = compare(g, o)
    assert ci["merges"] > 20
    g.close()


def test_frames_with_forces(gpu_lib, oracle_mod):
    """Gravity + Coulomb, Barnes-Hut, two frames: merges in several substeps,
    forces from trees holding removed particles, spawns as targets."""
    st, anti = dense(n=800, seed=11, box=60.0, lo=20.0, anti_frac=0.1)
    p = params(toggles=N.BARNES_HUT | N.GRAVITY | N.COULOMB, softening=1.0)
    g, o = setup(p, st, anti)
    for _ in range(2):
        a, b = g.update(1 / 60), o.update(1 / 60)
        assert a == b
    ci = compare(g, o)
    assert ci["merges"] > 0
    fg, fo = g.forces(), o.forces()
    e = vec_err(fg["fx"], fg["fy"], fo["fx"], fo["fy"])
    assert e["norm"] <= 1e-5, e
    g.close()


def test_removed_particles_remain_delayed_sources(gpu_lib, oracle_mod):
    """Relativity on with a warmed history: in the substep of a merge the two
    removed particles still act through their histories (signal delay) and
    the spawn, without history, acts on nothing."""
    st, anti = dense(n=400, seed=13, box=50.0, lo=25.0)
    p = params(toggles=N.BARNES_HUT | N.GRAVITY | N.COULOMB | N.RELATIVITY, softening=1.0)
    st32 = {k: f32(v) for k, v in st.items()}
    hist = W.straight_line_history(st32, 96, 120.0, 64 / 60)
    g, o = setup(p, st32, anti, history=hist)
    a, b = g.update(1 / 600), o.update(1 / 600)
    assert a == b
    ci = compare(g, o)
    assert ci["merges"] > 0
    fg, fo = g.forces(), o.forces()
    e = vec_err(fg["fx"], fg["fy"], fo["fx"], fo["fy"])
    assert e["norm"] <= 1e-5, e
    g.close()


def test_merge_enabled_later_keeps_state(gpu_lib):
    st, _ = dense(n=300, seed=3)
    p = params()
    p.collision_mode = N.COL_PASS
    g = GeonSystem(p, 300)
    g.upload(*[f32(st[k]) for k in STATE_KEYS])
    g.set_matter(antimatter=np.arange(300) % 2, base_mass=np.full(300, 2.5))
    before, mb = g.state(f64=True), g.matter()
    p.collision_mode = N.COL_MERGE
    g.set_params(p)                      # grows the particle slots
    after, ma = g.state(f64=True), g.matter()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    assert np.array_equal(mb["antimatter"], ma["antimatter"]) and np.array_equal(mb["base_mass"], ma["base_mass"])
    g.update(DT)
    assert g.collision_info()["merges"] + g.collision_info()["annihilations"] > 0
    g.close()


def test_unsupported_combinations(gpu_lib):
    p = params()
    p.collision_mode = N.COL_BOUNCE
    with pytest.raises(N.GeonError):
        GeonSystem(p, 16)
    p = params(flags=N.FLAG_LEARN)
    with pytest.raises(N.GeonError):
        GeonSystem(p, 16)


def test_gpu_physics_mirror_merges(gpu_lib):
    """The GPUPhysics mirror: collisionMode 'merge' from the settings string,
    antimatter from addParticle, events and the saved matter fields."""
    from physsim_gb300.gpu_physics import GeonGPUPhysics

    class Phys:
        gravityEnabled = True
        barnesHutEnabled = True
        collisionMode = "merge"

    b = GeonGPUPhysics(domainW=100.0, domainH=100.0, maxParticles=8).init()
    b.setToggles(Phys())
    b.addParticle({"x": 50.0, "y": 50.0, "mass": 8.0, "charge": 0.2})
    b.addParticle({"x": 51.5, "y": 50.0, "mass": 1.0, "antimatter": True})
    b.addParticle({"x": 20.0, "y": 20.0, "mass": 1.0})
    b.addParticle({"x": 21.0, "y": 20.0, "mass": 1.0, "charge": -0.1})
    b.update(1e-4)
    assert b.getParticleCount() == 2                      # one annihilation (8 - 1), one merge
    ev = b.collisionEvents()
    assert 1.0 in ev[:, 0].tolist() and len(ev) <= 2
    saved = b.serialize()
    masses = sorted(p["mass"] for p in saved["particles"])
    assert masses == pytest.approx([2.0, 7.0], rel=1e-6)
    assert saved["settings"]["collision"] == "merge"
    assert not any(p["antimatter"] for p in saved["particles"])
    b.destroy()
