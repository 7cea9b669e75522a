"""Batched systems (geon_create_batch) through the C ABI against the same
systems run one by one (each GeonSystem is itself parity-tested against the
FP64 oracle).

Bars: leaf membership of every tree point identical (the batched tree has
27 Morton levels below the system id; these inputs never need more); forces
and interaction counts identical (each system's targets start on a warp
boundary, so the walk groups the same 32 particles in the same order);
frames: the same substeps per system and identical positions; graph and
launch-by-launch execution identical; the autotuner restores the state.
"""
import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W
from physsim_gb300.system import BatchSystem, GeonSystem
from tests.parity import STATE_KEYS

pytestmark = pytest.mark.gpu


def small_ensemble(seed=41, n=6, lo=40, hi=900):
    return W.ensemble(n_systems=n, seed=seed, n_min=lo, n_max=hi, box=100.0, sigma=10.0)


def singles(wl):
    out = []
    for st in W.split_systems(wl):
        g = GeonSystem(wl.params, st["x"].size)
        g.upload(*[st[k] for k in STATE_KEYS])
        out.append(g)
    return out


def batch_of(wl):
    b = BatchSystem(wl.params, wl.info["counts"])
    b.upload(*[wl.state[k] for k in STATE_KEYS])
    return b


def leaf_rows(g, info):
    lop, bx, by, bw, lv = g.leaves(info)
    out = np.full((info["n_points"], 4), np.nan)
    ok = lop >= 0
    out[ok, 0], out[ok, 1], out[ok, 2], out[ok, 3] = bx[lop[ok]], by[lop[ok]], bw[lop[ok]], lv[lop[ok]]
    return out


def test_batched_tree_matches_single_systems(gpu_lib):
    wl = small_ensemble()
    b = batch_of(wl)
    ss = singles(wl)
    binfo = b.build_tree()
    brows = leaf_rows(b, binfo)
    counts = wl.info["counts"]
    ntot = int(counts.sum())
    off = np.concatenate([[0], np.cumsum(counts)])
    goff = ntot
    for s, g in enumerate(ss):
        info = g.build_tree()
        rows = leaf_rows(g, info)
        n, ng = int(counts[s]), info["n_ghosts"]
        np.testing.assert_array_equal(brows[off[s]:off[s + 1]], rows[:n], err_msg=f"system {s} particles")
        np.testing.assert_array_equal(brows[goff:goff + ng], rows[n:n + ng], err_msg=f"system {s} ghosts")
        goff += ng
        g.close()
    assert goff == binfo["n_points"]
    b.close()


def test_batched_forces_match_single_systems(gpu_lib):
    wl = small_ensemble(seed=42)
    b = batch_of(wl)
    ss = singles(wl)
    b.compute_forces()
    fb = b.forces()
    off = np.concatenate([[0], np.cumsum(wl.info["counts"])])
    inter = 0
    for s, g in enumerate(ss):
        g.compute_forces()
        f = g.forces()
        inter += g.interactions()
        for k in ("fx", "fy", "tidal", "pe"):
            np.testing.assert_array_equal(fb[k][off[s]:off[s + 1]], f[k], err_msg=f"system {s} {k}")
        g.close()
    assert b.interactions() == inter
    b.close()


@pytest.mark.parametrize("use_graph", [True, False])
def test_batched_frames_match_single_systems(gpu_lib, use_graph):
    wl = small_ensemble(seed=43)
    b = batch_of(wl)
    b.set_mode(use_graph=use_graph)
    ss = singles(wl)
    off = np.concatenate([[0], np.cumsum(wl.info["counts"])])
    for frame in range(3):
        mx = b.update(wl.dt)
        steps = b.substeps()
        assert mx == steps.max()
        for s, g in enumerate(ss):
            assert g.update(wl.dt) == steps[s], (frame, s)
    sb = b.state(f64=True)
    for s, g in enumerate(ss):
        st = g.state(f64=True)
        for k in ("x", "y", "wx", "wy"):
            np.testing.assert_array_equal(sb[k][off[s]:off[s + 1]], st[k], err_msg=f"system {s} {k}")
        g.close()
    b.close()


def test_autotune_restores_state_and_keeps_results(gpu_lib):
    wl = small_ensemble(seed=44, n=12, lo=64, hi=2000)
    ref = batch_of(wl)
    ref.set_mode(use_graph=False)
    ref.update(wl.dt)
    ref.update(wl.dt)
    want = ref.state(f64=True)
    ref.close()
    b = batch_of(wl)
    choice, ms = b.autotune(wl.dt, frames=1)
    assert 0 <= choice < N.BATCH_TUNE_MODES and np.all(ms > 0)
    st0 = b.state(f64=True)
    for k in ("x", "y", "wx", "wy"):
        np.testing.assert_array_equal(st0[k], wl.state[k].astype(np.float32).astype(np.float64))
    b.set_mode(use_graph=BatchSystem.tune_mode(choice)["use_graph"], simple_walk=False)
    b.set_shape(1, 6, 0, 0)
    b.update(wl.dt)
    b.update(wl.dt)
    got = b.state(f64=True)
    for k in ("x", "y", "wx", "wy"):
        np.testing.assert_array_equal(got[k], want[k])
    b.close()


def test_batched_rejects_unsupported(gpu_lib):
    wl = small_ensemble(seed=45, n=2, lo=40, hi=60)
    b = batch_of(wl)
    with pytest.raises(N.GeonError):
        b.direct_forces(np.arange(3))
    p = b.params()
    p.boundary_mode = N.BOUND_DESPAWN
    with pytest.raises(N.GeonError):
        b.set_params(p)
    b.close()


@pytest.mark.parametrize("warps,ctas,chunk", [(1, 3, 0), (4, 0, 0), (1, 0, 1), (1, 0, 4), (1, 7, 0)])
def test_walk_shapes(gpu_lib, warps, ctas, chunk):
    """The walk shapes the autotuner searches: a cap on resident walk CTAs and
    the work-queue form run the same code per group (bit-identical frames);
    four warps per group of targets, and the short stack (which pops fewer
    nodes at a time near its limit), change only the order of each target's
    sums (1e-6)."""
    wl = small_ensemble(seed=46, n=10, lo=64, hi=3000)
    ref = batch_of(wl)
    b = batch_of(wl)
    b.set_shape(warps, 6, ctas, chunk)
    try:
        for _ in range(2):
            assert np.array_equal(ref.update(wl.dt), b.update(wl.dt))
        sr, sb = ref.state(f64=True), b.state(f64=True)
    finally:
        ref.close()
        b.close()
    for k in ("x", "y", "wx", "wy"):
        if warps == 1 and ctas != 7:
            np.testing.assert_array_equal(sb[k], sr[k])
        else:
            d = np.linalg.norm(sb[k] - sr[k]) / max(np.linalg.norm(sr[k]), 1e-30)
            assert d <= 1e-6, (k, d)
