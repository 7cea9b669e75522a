"""The one-launch frame (frame.cu) against the launch-per-phase path and the
oracle, through the C ABI.

* small open systems run each frame as exactly one kernel launch;
* the frame kernel and the split path (GEON_FLAG_SPLIT_FRAME) run the same
  bodies on the same tree order: equal substep counts, ids and counts, and
  states equal to 1e-6 relative after ten frames (relativity on and off,
  despawn with compaction, bounce walls with external fields, the largest
  system the kernel takes);
* the split path itself stays within the trajectory bar of the oracle on the
  small config, as the frame kernel does (test_gpu_parity.py);
* a barrier that waits for a block that does not exist gives up after its
  time limit: geon_update returns GEON_ERR_TIMEOUT, and the GPU stays usable;
* the hand-traced cases of the oracle's known-answer tests: the substep
  count when dtRemain is an exact multiple of dtSafe, and the Yukawa cutoff
  at a separation of exactly 6 / mu.
"""
import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W
from physsim_gb300.system import GeonSystem
from tests.parity import STATE_KEYS, load_both, rel_err

pytestmark = pytest.mark.gpu

FRAME_TOL = 1e-6
TRAJ_TOL = 1e-5          # the trajectory bar of the frame parity tests


def make(wl, split=False):
    g = GeonSystem(wl.params, wl.n)
    g.upload(*[wl.state[k] for k in STATE_KEYS])
    if split:
        p = g.params()
        p.flags |= N.FLAG_SPLIT_FRAME
        g.set_params(p)
    return g


def run_pair(wl, frames):
    a, b = make(wl), make(wl, split=True)
    try:
        for f in range(frames):
            sa, sb = a.update(wl.dt), b.update(wl.dt)
            assert sa == sb, ("substeps", f, sa, sb)
        assert a.count() == b.count()
        assert np.array_equal(a.ids(), b.ids())
        return a.state(f64=True), b.state(f64=True), a.stats(), b.stats()
    finally:
        a.close()
        b.close()


def assert_close(sa, sb, keys=("x", "y", "wx", "wy", "angw")):
    errs = {k: rel_err(sa[k], sb[k]) for k in keys}
    print("frame kernel vs split path:", {k: e["norm"] for k, e in errs.items()})
    for k, e in errs.items():
        assert e["norm"] <= FRAME_TOL, (k, e)


def test_one_launch_per_frame(gpu_lib):
    wl = W.small_disk(2048)
    g = make(wl)
    try:
        g.update(wl.dt)                       # the first frame bootstraps forces on the split path
        c0 = g.launch_count()
        for _ in range(5):
            g.update(wl.dt)
        per_frame = (g.launch_count() - c0) / 5
    finally:
        g.close()
    assert per_frame == 1, per_frame


@pytest.mark.parametrize("relativity", [True, False])
def test_frame_kernel_matches_split_path(gpu_lib, relativity):
    wl = W.small_disk(2048, relativity=relativity, softening=0.1 if relativity else 8.0)
    sa, sb, ta, tb = run_pair(wl, 10)
    assert_close(sa, sb)
    assert ta["sim_time"] == tb["sim_time"]


def test_frame_kernel_despawn_compaction(gpu_lib):
    wl = W.small_disk(256, relativity=True, softening=8.0)
    wl.state["x"][[3, 100, 200]] = [170.0, -70.0, 180.0]
    sa, sb, ta, tb = run_pair(wl, 3)
    assert ta["alive_count"] == tb["alive_count"] == 253
    assert_close(sa, sb)


def test_frame_kernel_bounce_and_external_fields(gpu_lib):
    wl = W.small_disk(512, relativity=False, softening=8.0)
    p = wl.params
    p.boundary_mode = N.BOUND_BOUNCE
    p.ext_gravity, p.ext_electric, p.ext_bz = 0.3, 0.2, 0.05
    wl.state["x"][:8] = np.linspace(0.1, 0.8, 8)
    sa, sb, _, _ = run_pair(wl, 5)
    assert_close(sa, sb)


def test_frame_kernel_largest_system(gpu_lib):
    wl = W.small_disk(N.FRAME_MAX_POINTS, relativity=True, softening=0.1)
    sa, sb, _, _ = run_pair(wl, 4)
    assert_close(sa, sb)


def test_split_path_small_config_against_oracle(gpu_lib, oracle_mod):
    wl = W.small_disk(2048)
    g, o = load_both(wl)
    p = g.params()
    p.flags |= N.FLAG_SPLIT_FRAME
    g.set_params(p)
    try:
        for _ in range(10):
            assert g.update(wl.dt) == o.update(wl.dt)
        sg, so = g.state(f64=True), o.state()
    finally:
        g.close()
    for k in ("x", "y", "wx", "wy", "angw"):
        assert rel_err(sg[k], so[k])["norm"] <= TRAJ_TOL, k


def test_barrier_timeout_is_reported(gpu_lib):
    wl = W.small_disk(1024)
    g = make(wl)
    try:
        g.update(wl.dt)
        g.set_frame_wait(20_000_000, extra_arrivals=1)     # 20 ms, one block that never arrives
        with pytest.raises(N.GeonError) as ei:
            g.update(wl.dt)
        assert ei.value.code == N.GEON_ERR_TIMEOUT, str(ei.value)
    finally:
        g.close()
    # the context is still usable: a new system runs its frames
    h = make(wl)
    try:
        for _ in range(2):
            h.update(wl.dt)
        assert h.count() == wl.n
    finally:
        h.close()


# The hand-traced planner and cutoff cases of tests/test_oracle_kat.py on the
# device: the substep count at an exact multiple dtRemain = 4 dtSafe (and one
# part in 2^20 either side), through the one-launch frame, the split path and
# the pairwise path.
@pytest.mark.parametrize("g,expect", [(4096.0, 4), (4096.0 * (1 + 2.0 ** -20), 5), (4096.0 * (1 - 2.0 ** -20), 4)])
@pytest.mark.parametrize("path", ["frame", "split", "pairwise"])
def test_planner_ceil_at_exact_multiples(gpu_lib, g, expect, path):
    tg = N.GRAVITY | (0 if path == "pairwise" else N.BARNES_HUT)
    fl = N.FLAG_SPLIT_FRAME if path == "split" else 0
    p = N.make_params(toggles=tg, flags=fl, softening=1.0, domain_w=1000, domain_h=1000, ext_gravity=g)
    one = np.ones(1)
    g_ = GeonSystem(p, 1)
    try:
        g_.upload_f64(np.array([100.0]), np.array([500.0]), 0 * one, 0 * one, one, 0 * one, 0 * one)
        assert g_.update(1 / 16) == expect
        assert g_.update(1 / 16) == expect
    finally:
        g_.close()


@pytest.mark.parametrize("d,inside", [(8.0, False), (8.0 - 2.0 ** -40, True), (8.0 + 2.0 ** -40, False)])
@pytest.mark.parametrize("bh", [True, False])
def test_yukawa_cutoff_tie(gpu_lib, d, inside, bh):
    mu, eps = 0.75, 1.0
    p = N.make_params(toggles=N.YUKAWA | (N.BARNES_HUT if bh else 0), softening=eps, yukawa_mu=mu,
                      domain_w=1000, domain_h=1000)
    g_ = GeonSystem(p, 2)
    z = np.zeros(2)
    try:
        g_.upload_f64(np.array([100.0, 100.0 + d]), np.array([500.0, 500.0]), z, z, np.array([2.0, 1.5]), z, z)
        g_.compute_forces()
        fx = float(g_.forces()["fx"][0])
    finally:
        g_.close()
    if inside:
        r = np.sqrt(d * d + eps * eps)
        expect = 14 * 2.0 * 1.5 * np.exp(-mu * r) * (1 / r ** 2 + mu / r) / r * d
        assert abs(fx - expect) <= 1e-5 * abs(expect), (fx, expect)
    else:
        assert fx == 0.0


@pytest.mark.parametrize("dt,max_sub", [(0.0, 32), (2.0, 2), (2.0, 32)])
def test_frame_kernel_edge_frames(gpu_lib, dt, max_sub):
    """A zero-length frame (no substep: history and boundary only), a frame
    cut short by the substep cap, and a long frame of several substeps: the
    one-launch frame takes the same substeps as the split path and ends in
    the same state."""
    wl = W.small_disk(1024, relativity=True, softening=0.1)
    wl.params.max_substeps = max_sub
    a, b = make(wl), make(wl, split=True)
    try:
        a.update(1 / 60)
        b.update(1 / 60)                     # bootstrap forces and one ordinary frame first
        for _ in range(3 if dt == 0.0 else 1):
            sa, sb = a.update(dt), b.update(dt)
            assert sa == sb, (sa, sb)
            if dt == 0.0:
                assert sa == 0
            elif max_sub == 2:
                assert sa == 2
            else:
                assert sa > 2
        assert a.count() == b.count()
        assert_close(a.state(f64=True), b.state(f64=True))
        assert a.stats()["sim_time"] == b.stats()["sim_time"]
    finally:
        a.close()
        b.close()


def test_frame_kernel_history_and_signal_delay(gpu_lib):
    """Relativity samples the history every 64 frames, and the walk takes
    signal-delayed sources once a particle has two samples: 140 frames of a
    256-particle disk go through both inside the one-launch frame.  Same
    substeps, counts and states as the split path."""
    wl = W.small_disk(256, relativity=True, softening=8.0)
    a, b = make(wl), make(wl, split=True)
    try:
        for f in range(140):
            sa, sb = a.update(wl.dt), b.update(wl.dt)
            assert sa == sb, (f, sa, sb)
        assert a.count() == b.count()
        assert_close(a.state(f64=True), b.state(f64=True))
        assert a.stats()["sim_time"] == b.stats()["sim_time"]
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("path", ["frame", "split"])
def test_planner_cyclotron_limit(gpu_lib, path):
    """The cyclotron limit of the planner at an exact multiple (the case of
    tests/test_oracle_kat.py): dt = 4 dtCyc takes 4 substeps, a dt one part
    in 2^40 longer takes 5."""
    bz = 50.25
    dt4 = 4 * (0.7853981633974483 / bz)
    fl = N.FLAG_SPLIT_FRAME if path == "split" else 0
    p = N.make_params(toggles=N.GRAVITY | N.BARNES_HUT, flags=fl, softening=1.0, domain_w=1000, domain_h=1000,
                      ext_bz=bz)
    one = np.ones(1)
    g_ = GeonSystem(p, 1)
    try:
        g_.upload_f64(np.array([500.0]), np.array([500.0]), 0 * one, 0 * one, one, one, 0 * one)
        assert g_.update(dt4) == 4
        assert g_.update(dt4 * (1 + 2.0 ** -40)) == 5
    finally:
        g_.close()
