"""Seeded synthetic inputs with the shapes of the five benchmark workloads.

There is no public dataset for this path; each generator draws particle
states with the stated distributions from a seeded PCG64 stream.  Positions
are expressed in the reference's frame [offX, offX + W] x [offY, offY + H]
(the box [-L/2, L/2]^2 shifted by +L/2), and every value is rounded to FP32
so the GPU state and the FP64 oracle start from identical numbers.

Initial spin follows main.js:517-521 (surface speed s -> angular celerity
angw = sign(s) |s| / (r sqrt(1 - s^2)), r = cbrt(m)); charge is k * 0.1 with
integer k uniform in [-5, 5] (main.js:511 quantises charge to 0.1).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _native as N


@dataclass
class Workload:
    name: str
    params: N.GeonParams
    state: dict                     # x, y, wx, wy, mass, charge, angw (float64 holding FP32 values)
    dt: float
    frames: int
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.state["x"].size)


def _f32(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def spin_to_angw(spin: np.ndarray, mass: np.ndarray) -> np.ndarray:
    """main.js:517-521 with MAX_SPEED_RATIO = 0.999."""
    sv = np.clip(spin, -0.999, 0.999)
    r = np.cbrt(mass)
    a = np.abs(sv)
    with np.errstate(divide="ignore", invalid="ignore"):
        angw = np.where(a > 0, np.sign(sv) * a / (r * np.sqrt(1 - a * a)), 0.0)
    return angw


def _charges(rng, n):
    return rng.integers(-5, 6, size=n) * 0.1


def _pack(x, y, wx, wy, m, q, angw):
    return {k: _f32(v) for k, v in zip(("x", "y", "wx", "wy", "mass", "charge", "angw"), (x, y, wx, wy, m, q, angw))}


def small_disk(n: int = 2048, seed: int = 1, relativity: bool = True, softening: float = 0.1,
               theta: float = 0.5, barnes_hut: bool = True) -> Workload:
    """Plain method, small: N particles uniform in a disk of radius 40 in a
    100 x 100 box, lognormal(0, 0.5) masses, spin U[-0.5, 0.5], proper
    velocity N(0, 0.05^2); gravity + Coulomb (+ relativity), softening 0.1,
    despawn boundary, BH theta 0.5, dt = 1/60."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = 100.0
    r = 40.0 * np.sqrt(rng.random(n))
    ph = rng.random(n) * 2 * np.pi
    x = L / 2 + r * np.cos(ph)
    y = L / 2 + r * np.sin(ph)
    m = rng.lognormal(0.0, 0.5, n)
    q = _charges(rng, n)
    spin = rng.uniform(-0.5, 0.5, n)
    wx = rng.normal(0, 0.05, n)
    wy = rng.normal(0, 0.05, n)
    st = _pack(x, y, wx, wy, m, q, spin_to_angw(spin, _f32(m)))
    tg = N.GRAVITY | N.COULOMB | (N.RELATIVITY if relativity else 0) | (N.BARNES_HUT if barnes_hut else 0)
    p = N.make_params(toggles=tg, boundary_mode=N.BOUND_DESPAWN, domain_w=L, domain_h=L,
                      theta=theta, softening=softening)
    return Workload("small_disk_n%d" % n, p, st, 1 / 60, 10, {"box": L})


def clusters_torus(n: int = 65536, seed: int = 2, barnes_hut: bool = True, relativity: bool = True,
                   softening: float = 8.0, theta: float = 0.5) -> Workload:
    """Full pairwise force set: 8 Gaussian clusters (sigma 4) at uniform
    centres in a 400 x 400 torus, lognormal(0, 0.7) masses, spin U[-1, 1]
    (clamped to 0.999); gravity, Coulomb, Yukawa (mu 0.15), magnetic and
    gravitomagnetic dipoles, 1PN, spin-orbit, relativity; loop boundary."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = 400.0
    centres = rng.random((8, 2)) * L
    which = rng.integers(0, 8, size=n)
    x = np.mod(centres[which, 0] + rng.normal(0, 4.0, n), L)
    y = np.mod(centres[which, 1] + rng.normal(0, 4.0, n), L)
    m = rng.lognormal(0.0, 0.7, n)
    q = _charges(rng, n)
    spin = rng.uniform(-1.0, 1.0, n)
    wx = rng.normal(0, 0.05, n)
    wy = rng.normal(0, 0.05, n)
    st = _pack(x, y, wx, wy, m, q, spin_to_angw(spin, _f32(m)))
    tg = (N.GRAVITY | N.COULOMB | N.YUKAWA | N.MAGNETIC | N.GRAVITOMAG | N.ONE_PN | N.SPIN_ORBIT
          | (N.RELATIVITY if relativity else 0) | (N.BARNES_HUT if barnes_hut else 0))
    p = N.make_params(toggles=tg, boundary_mode=N.BOUND_LOOP, topology=N.TORUS, domain_w=L, domain_h=L,
                      theta=theta, softening=softening, yukawa_mu=0.15)
    return Workload("clusters_torus_n%d" % n, p, st, 1 / 60, 100, {"box": L})


def ensemble(n_systems: int = 512, seed: int = 5, n_min: int = 256, n_max: int = 16384, box: float = 100.0,
             sigma: float = 10.0, theta: float = 0.6, softening: float = 8.0) -> Workload:
    """Batched ensemble: n_systems independent systems, N log-uniform in
    [n_min, n_max] (seeded), each one Gaussian cluster (sigma 10) at a uniform
    centre of a box x box torus; lognormal(0, 0.5) masses, quantised charges,
    spin U[-0.5, 0.5], proper velocity N(0, 0.05^2); gravity + Coulomb,
    Barnes-Hut theta 0.6.  The state is concatenated system by system;
    info["counts"] holds the particles of each system."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_systems)).astype(np.int64)
    counts = np.clip(counts, n_min, n_max)
    parts = {k: [] for k in ("x", "y", "wx", "wy", "m", "q", "spin")}
    for c in counts:
        c = int(c)
        cx, cy = rng.random(2) * box
        parts["x"].append(np.mod(cx + rng.normal(0, sigma, c), box))
        parts["y"].append(np.mod(cy + rng.normal(0, sigma, c), box))
        parts["wx"].append(rng.normal(0, 0.05, c))
        parts["wy"].append(rng.normal(0, 0.05, c))
        parts["m"].append(rng.lognormal(0.0, 0.5, c))
        parts["q"].append(_charges(rng, c))
        parts["spin"].append(rng.uniform(-0.5, 0.5, c))
    cat = {k: np.concatenate(v) for k, v in parts.items()}
    m32 = _f32(cat["m"])
    st = _pack(cat["x"], cat["y"], cat["wx"], cat["wy"], cat["m"], cat["q"], spin_to_angw(cat["spin"], m32))
    p = N.make_params(toggles=N.GRAVITY | N.COULOMB | N.BARNES_HUT, boundary_mode=N.BOUND_LOOP, topology=N.TORUS,
                      domain_w=box, domain_h=box, theta=theta, softening=softening)
    return Workload("ensemble_%dx[%d,%d]" % (n_systems, n_min, n_max), p, st, 1 / 60, 10,
                    {"counts": counts.astype(np.int32), "box": box})


def split_systems(wl: Workload) -> list:
    """The systems of an ensemble as separate state dicts."""
    off = np.concatenate([[0], np.cumsum(wl.info["counts"])])
    return [{k: v[off[s]:off[s + 1]] for k, v in wl.state.items()} for s in range(len(off) - 1)]


def sparse_field(n: int = 65536, seed: int = 9, box: float | None = None, anti_frac: float = 0.05,
                 theta: float = 0.5) -> Workload:
    """Merge-collision workload: n particles uniform over a square box whose
    side grows as sqrt(n) (2000 at n = 65536: mean spacing about 8, so about
    one particle in ten touches a neighbour at radius cbrt(m) ~ 1 in the
    first substep), lognormal(0, 0.5) masses, w ~ N(0, 0.05^2) per axis,
    charges as the other workloads, a fraction `anti_frac` of antimatter
    (info['antimatter']); gravity + Coulomb, Barnes-Hut, softening 8, merge
    collisions, despawn boundary."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = box if box is not None else 2000.0 * np.sqrt(n / 65536.0)
    x = rng.random(n) * L
    y = rng.random(n) * L
    m = rng.lognormal(0.0, 0.5, n)
    q = _charges(rng, n)
    wx = rng.normal(0, 0.05, n)
    wy = rng.normal(0, 0.05, n)
    anti = (rng.random(n) < anti_frac).astype(np.int32)
    st = _pack(x, y, wx, wy, m, q, np.zeros(n))
    p = N.make_params(toggles=N.GRAVITY | N.COULOMB | N.BARNES_HUT, boundary_mode=N.BOUND_DESPAWN, domain_w=L,
                      domain_h=L, theta=theta, softening=8.0, collision_mode=N.COL_MERGE)
    return Workload("sparse_field_n%d" % n, p, st, 1 / 60, 10, {"box": L, "antimatter": anti})


def plummer_disk(n: int = 1 << 20, seed: int = 3, theta: float = 0.5, softening: float = 8.0,
                 a: float = 50.0, background: float = 0.05) -> Workload:
    """Large plain BH: 2-D Plummer-like disk (surface density (1+r^2/a^2)^-2,
    a = 50, r = a sqrt(u/(1-u))) plus a uniform background (5 %) over a
    2000 x 2000 box; lognormal(0, 1) masses; gravity + Coulomb + Yukawa;
    spin U[-0.5, 0.5], proper velocity N(0, 0.05^2); despawn boundary."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = 2000.0
    nb = int(round(n * background))
    nd = n - nb
    xs, ys = [], []
    got = 0
    while got < nd:
        k = (nd - got) * 11 // 10 + 16
        u = rng.random(k)
        r = a * np.sqrt(u / (1 - u))
        ph = rng.random(k) * 2 * np.pi
        x = L / 2 + r * np.cos(ph)
        y = L / 2 + r * np.sin(ph)
        ok = (x >= 0) & (x <= L) & (y >= 0) & (y <= L)
        xs.append(x[ok]); ys.append(y[ok])
        got += int(ok.sum())
    x = np.concatenate(xs)[:nd]
    y = np.concatenate(ys)[:nd]
    x = np.concatenate([x, rng.random(nb) * L])
    y = np.concatenate([y, rng.random(nb) * L])
    m = rng.lognormal(0.0, 1.0, n)
    q = _charges(rng, n)
    spin = rng.uniform(-0.5, 0.5, n)
    wx = rng.normal(0, 0.05, n)
    wy = rng.normal(0, 0.05, n)
    st = _pack(x, y, wx, wy, m, q, spin_to_angw(spin, _f32(m)))
    tg = N.GRAVITY | N.COULOMB | N.YUKAWA | N.BARNES_HUT
    p = N.make_params(toggles=tg, boundary_mode=N.BOUND_DESPAWN, domain_w=L, domain_h=L,
                      theta=theta, softening=softening, yukawa_mu=0.15)
    return Workload("plummer_disk_n%d" % n, p, st, 1 / 60, 10, {"box": L, "a": a})


def straight_line_history(state: dict, count: int, t_end: float, spacing: float):
    """A history ring as if each particle had moved in a straight line at its
    current coordinate velocity, sampled every `spacing` time units up to
    t_end (the reference samples every 64 frames, integrator.js:1549-1565).
    Returns (times, x, y, vx, vy, angw) with planes of shape (n, count)."""
    w = np.stack([state["wx"], state["wy"]])
    g = np.sqrt(1 + (w ** 2).sum(0))
    vx, vy = state["wx"] / g, state["wy"] / g
    times = t_end - spacing * np.arange(count)[::-1]
    dt = (times - t_end)[None, :]
    X = state["x"][:, None] + vx[:, None] * dt
    Y = state["y"][:, None] + vy[:, None] * dt
    VX = np.repeat(vx[:, None], count, 1)
    VY = np.repeat(vy[:, None], count, 1)
    A = np.repeat(state["angw"][:, None], count, 1)
    f = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)
    return times, f(X), f(Y), f(VX), f(VY), f(A)
