"""Boson-tree walks in the FP64 oracle (CPU only): known answers for the
softened monopole walk over the boson pool (src/forces.js:713-901) and its
tree (src/integrator.js:263-277, src/quadtree.js:316-368)."""
import numpy as np

from physsim_gb300 import _native as N


def make(params, x, y, m):
    from oracle.oracle import OracleSim
    o = OracleSim(params)
    n = len(x)
    z = np.zeros(n)
    o.add(np.asarray(x, float), np.asarray(y, float), z, z, np.asarray(m, float), z, z)
    return o


def boson_rows(x, y, mass, charge=None, kind=None, vsq=None):
    n = len(x)
    z = np.zeros(n)
    return np.stack([x, y, mass, z if charge is None else charge, z if kind is None else kind,
                     z if vsq is None else vsq], 1).astype(np.float64)


def test_photon_gravity_on_a_particle(oracle_mod):
    eps = 2.0
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, flags=N.FLAG_BOSONS, softening=eps)
    o = make(p, [40.0], [50.0], [3.0])
    o.set_bosons(boson_rows(np.array([43.0]), np.array([54.0]), np.array([0.5])))
    o.compute_forces()
    f = o.forces()
    expect = 3.0 * 0.5 * np.array([3.0, 4.0]) / (25 + eps * eps) ** 1.5
    assert np.allclose([f["fx"][0], f["fy"][0]], expect, rtol=1e-14)
    assert np.allclose([f["grav_x"][0], f["grav_y"][0]], expect, rtol=1e-14)


def test_flag_off_means_no_boson_gravity(oracle_mod):
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, softening=2.0)
    o = make(p, [40.0], [50.0], [3.0])
    o.set_bosons(boson_rows(np.array([43.0]), np.array([54.0]), np.array([0.5])))
    o.compute_forces()
    assert o.forces()["fx"][0] == 0


def test_two_boson_kicks(oracle_mod):
    dt = 0.01
    p = N.make_params(toggles=N.GRAVITY | N.COULOMB | N.BARNES_HUT, flags=N.FLAG_BOSONS)
    o = make(p, [10.0], [10.0], [1.0])
    # a photon (energy 2) and a charged pion (gravitational mass 1.5, charge 0.1, v^2 0.25)
    o.set_bosons(boson_rows(np.array([50.0, 53.0]), np.array([50.0, 54.0]), np.array([2.0, 1.5]),
                            np.array([0.0, 0.1]), np.array([0, 1]), np.array([0.0, 0.25])))
    k = o.boson_kicks(dt, 3)
    d = np.array([3.0, 4.0])
    inv = 1 / (25 + 4.0) ** 1.5                 # BOSON_SOFTENING_SQ = 4
    assert np.allclose(k[0], 2 * dt * 1.5 * d * inv, rtol=1e-14)            # photon: 2 dt, pulled by the pion
    # pion: (1 + v^2) dt gravity from the photon; no Coulomb (the photon is neutral)
    assert np.allclose(k[1], (1 + 0.25) * dt * 2.0 * (-d) * inv, rtol=1e-14)
    assert np.allclose(o.boson_kicks(dt, 2), 0)


def test_like_charges_repel(oracle_mod):
    dt = 0.01
    p = N.make_params(toggles=N.COULOMB | N.BARNES_HUT, flags=N.FLAG_BOSONS)
    o = make(p, [10.0], [10.0], [1.0])
    o.set_bosons(boson_rows(np.array([50.0, 54.0]), np.array([50.0, 50.0]), np.array([1.0, 1.0]),
                            np.array([0.1, 0.1]), np.array([1, 1])))
    k = o.boson_kicks(dt, 2)
    inv = 1 / (16 + 4.0) ** 1.5
    assert np.allclose(k[0], [-0.1 * dt * 0.1 * 4 * inv, 0], rtol=1e-14)
    assert np.allclose(k[1], [0.1 * dt * 0.1 * 4 * inv, 0], rtol=1e-14)


def test_tree_walk_matches_direct_sum(oracle_mod):
    rng = np.random.default_rng(2)
    nb = 3000
    bx, by = rng.uniform(10, 90, nb), rng.uniform(10, 90, nb)
    e = rng.uniform(0.1, 1.0, nb)
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, flags=N.FLAG_BOSONS, theta=0.0)
    o = make(p, [50.0], [50.0], [1.0])
    o.set_params(p)                             # theta 0 (creation defaults a zero theta to 0.5)
    o.set_bosons(boson_rows(bx, by, e, kind=np.zeros(nb)))
    k = o.boson_kicks(1.0, 1)
    # theta 0 opens every cell: the walk is the exact softened sum
    dx, dy = bx[None, :] - bx[:, None], by[None, :] - by[:, None]
    inv = (dx * dx + dy * dy + 4.0) ** -1.5
    ref = np.stack([(2 * e[None, :] * dx * inv).sum(1), (2 * e[None, :] * dy * inv).sum(1)], 1)
    assert np.allclose(k, ref, rtol=1e-10, atol=1e-12)
    p.theta = 0.5
    o.set_params(p)
    k5 = o.boson_kicks(1.0, 1)
    err = np.linalg.norm(k5 - ref) / np.linalg.norm(ref)
    assert 0 < err < 5e-2               # monopole cells at theta 0.5
