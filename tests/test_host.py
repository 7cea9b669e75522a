"""Host-side logic of the GPUPhysics mirror (no GPU)."""
import math

import numpy as np
import pytest

from physsim_gb300 import gpu_physics as G
from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W


def test_set_velocity_matches_relativity_js():
    (v, w) = G.set_velocity(0.3, 0.4)
    g = 1 / math.sqrt(1 - 0.25)
    assert np.allclose(v, (0.3, 0.4)) and np.allclose(w, (0.3 * g, 0.4 * g))
    (v, w) = G.set_velocity(3.0, 4.0)          # clamped to 0.999 c
    assert math.isclose(math.hypot(*v), 0.999, rel_tol=1e-12)


def test_charge_quantisation():
    assert G.quantise_charge(0.26) == pytest.approx(0.3)
    assert G.quantise_charge(-0.04) == pytest.approx(0.0)


def test_spin_to_angw_main_js():
    m = np.array([8.0])
    a = W.spin_to_angw(np.array([0.6]), m)
    assert np.isclose(a[0], 0.6 / (2.0 * math.sqrt(1 - 0.36)))
    assert W.spin_to_angw(np.array([2.0]), m)[0] > 0


def test_toggle_packing_reads_physics_like_objects():
    class P:
        gravityEnabled = True
        coulombEnabled = False
        barnesHutEnabled = True
        yukawaEnabled = True
        yukawaMu = 0.2
    gp = G.GeonGPUPhysics(None, 100, 100)
    gp.setToggles(P())
    assert gp._toggles == N.GRAVITY | N.BARNES_HUT | N.YUKAWA
    assert gp._params().yukawa_mu == pytest.approx(0.2)


def test_workloads_are_fp32_exact_and_seeded():
    a = W.small_disk(256)
    b = W.small_disk(256)
    for k in a.state:
        assert np.array_equal(a.state[k], b.state[k])
        assert np.array_equal(a.state[k], a.state[k].astype(np.float32).astype(np.float64))
    p = W.plummer_disk(4096)
    assert p.state["x"].min() >= 0 and p.state["x"].max() <= 2000
