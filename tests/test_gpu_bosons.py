"""The boson-tree walks on the GPU (geon_set_bosons, GEON_FLAG_BOSONS,
geon_boson_kicks) against the FP64 oracle's restatement of
src/forces.js:697-901.

Bars: forces on particles, boson kicks and one-frame trajectories within
1e-5 norm-wise (FP32 sums against FP64; the opening decisions are FP64 on
both sides); no effect without the flag or with an empty pool."""
import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300.system import GeonSystem
from tests.parity import STATE_KEYS, rel_err, vec_err

pytestmark = pytest.mark.gpu


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def particles(rng, n, lo=10.0, hi=90.0):
    return {"x": f32(rng.uniform(lo, hi, n)), "y": f32(rng.uniform(lo, hi, n)),
            "wx": f32(rng.normal(0, 0.02, n)), "wy": f32(rng.normal(0, 0.02, n)),
            "mass": f32(rng.lognormal(0, 0.5, n)), "charge": f32(rng.integers(-3, 4, n) * 0.1),
            "angw": np.zeros(n)}


def pool(rng, nb, lo=5.0, hi=95.0, charged=True):
    kind = (rng.random(nb) < 0.4).astype(float)            # 40 % pions / leptons
    q = np.where(kind > 0, rng.choice([-0.1, 0.1], nb), 0.0) if charged else np.zeros(nb)
    rows = np.stack([rng.uniform(lo, hi, nb), rng.uniform(lo, hi, nb), rng.uniform(0.05, 1.0, nb), q, kind,
                     np.where(kind > 0, rng.uniform(0, 0.5, nb), 0.0)], 1)
    return np.vstack([f32(c) for c in rows.T]).T


def both(p, st, rows):
    from oracle.oracle import OracleSim
    g = GeonSystem(p, len(st["x"]))
    g.upload(*[st[k] for k in STATE_KEYS])
    g.set_bosons(rows)
    o = OracleSim(p, threads=8)
    o.add(*[st[k] for k in STATE_KEYS])
    o.set_bosons(rows)
    return g, o


@pytest.mark.parametrize("boundary,bh", [(N.BOUND_DESPAWN, True), (N.BOUND_LOOP, True), (N.BOUND_DESPAWN, False)])
def test_boson_gravity_on_particles(gpu_lib, oracle_mod, boundary, bh):
    rng = np.random.default_rng(1)
    st = particles(rng, 3000)
    rows = pool(rng, 800)
    p = N.make_params(toggles=N.GRAVITY | (N.BARNES_HUT if bh else 0), flags=N.FLAG_BOSONS | N.FLAG_BREAKDOWN,
                      boundary_mode=boundary, softening=2.0)
    g, o = both(p, st, rows)
    g.compute_forces()
    o.compute_forces()
    fg, fo = g.forces(), o.forces()
    for kx, ky in (("fx", "fy"), ("grav_x", "grav_y")):
        e = vec_err(fg[kx], fg[ky], fo[kx], fo[ky])
        assert e["norm"] <= 1e-5, (kx, e)
    # the bosons' share alone: against the same pass without the flag
    p2 = N.make_params(toggles=N.GRAVITY | (N.BARNES_HUT if bh else 0), boundary_mode=boundary, softening=2.0)
    g.set_params(p2)
    g.compute_forces()
    f0 = g.forces()
    o.set_params(p2)
    o.compute_forces()
    o0 = o.forces()
    e = vec_err(fg["fx"] - f0["fx"], fg["fy"] - f0["fy"], fo["fx"] - o0["fx"], fo["fy"] - o0["fy"])
    assert e["norm"] <= 1e-4, e
    g.close()


@pytest.mark.parametrize("topology", [None, N.TORUS, N.KLEIN])
def test_boson_kicks(gpu_lib, oracle_mod, topology):
    rng = np.random.default_rng(2)
    st = particles(rng, 16)
    rows = pool(rng, 3000)
    kw = {} if topology is None else {"boundary_mode": N.BOUND_LOOP, "topology": topology}
    p = N.make_params(toggles=N.GRAVITY | N.COULOMB | N.BARNES_HUT, flags=N.FLAG_BOSONS, **kw)
    g, o = both(p, st, rows)
    for what in (1, 2, 3):
        kg, ko = g.boson_kicks(0.01, what), o.boson_kicks(0.01, what)
        e = vec_err(kg[:, 0], kg[:, 1], ko[:, 0], ko[:, 1])
        assert e["norm"] <= 1e-5, (what, e)
    assert np.all(g.boson_kicks(0.01, 2)[rows[:, 4] == 0] == 0)      # photons feel no Coulomb
    g.close()


def test_frames_with_boson_gravity(gpu_lib, oracle_mod):
    rng = np.random.default_rng(3)
    st = particles(rng, 2000)
    rows = pool(rng, 500)
    p = N.make_params(toggles=N.GRAVITY | N.COULOMB | N.BARNES_HUT, flags=N.FLAG_BOSONS, softening=2.0)
    g, o = both(p, st, rows)
    for _ in range(2):
        assert g.update(1 / 60) == o.update(1 / 60)
    sg, so = g.state(f64=True), o.state()
    for k in ("x", "y", "wx", "wy"):
        assert rel_err(sg[k], so[k])["norm"] <= 1e-5, k
    g.close()


def test_no_effect_without_flag_or_pool(gpu_lib):
    rng = np.random.default_rng(4)
    st = particles(rng, 500)
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, softening=2.0)
    g = GeonSystem(p, 500)
    g.upload(*[st[k] for k in STATE_KEYS])
    g.compute_forces()
    ref = g.forces()
    g.set_bosons(pool(rng, 200))                   # flag off: the pool is ignored
    g.compute_forces()
    f = g.forces()
    assert np.array_equal(f["fx"], ref["fx"]) and np.array_equal(f["fy"], ref["fy"])
    p.flags = N.FLAG_BOSONS
    g.set_params(p)
    g.set_bosons(np.zeros((0, 6)))                  # empty pool
    g.compute_forces()
    f = g.forces()
    assert np.array_equal(f["fx"], ref["fx"])
    g.close()


def test_gpu_physics_mirror_boson_pool(gpu_lib, oracle_mod):
    """The GPUPhysics mirror: bosonInterEnabled from setToggles, the pool from
    Simulation-style objects, kicks in pool order, the saved toggle."""
    from physsim_gb300.gpu_physics import GeonGPUPhysics

    class Phys:
        gravityEnabled = True
        coulombEnabled = True
        barnesHutEnabled = True
        bosonInterEnabled = True

    b = GeonGPUPhysics(domainW=100.0, domainH=100.0, maxParticles=16).init()
    b.setToggles(Phys())
    b.addParticle({"x": 40.0, "y": 50.0, "mass": 2.0})
    photons = [{"pos": {"x": 45.0, "y": 50.0}, "_srcMass": 1.0}]
    pions = [{"pos": {"x": 60.0, "y": 50.0}, "_srcMass": 0.5, "charge": 0.1, "vSq": 0.2},
             {"pos": {"x": 62.0, "y": 50.0}, "_srcMass": 0.5, "charge": 0.1, "vSq": 0.2},
             {"pos": {"x": 80.0, "y": 50.0}, "_srcMass": 0.5, "charge": 0.1, "vSq": 0.2, "alive": False}]
    b.setBosonPool(photons, pions)
    k = b.bosonKicks(0.01)
    assert k.shape == (3, 2)                      # the dead pion is left out
    assert k[0, 0] > 0 and k[1, 0] > 0 > k[2, 0]  # gravity pulls the three together
    assert np.array_equal(k, b._sys.boson_kicks(0.01, 3))
    b._sys.compute_forces()
    f = b._sys.forces()
    assert f["fx"][0] > 0                         # pulled towards the photon at x = 45
    assert b.serialize()["toggles"]["bosonInterEnabled"]
    b.destroy()
