"""Potential heat map through the C ABI against the FP64 oracle
(heatmap.js): tree walk and pairwise sum, open box and torus, with and
without signal delay, blurred and raw.  Bar: norm-wise relative error
<= 1e-5 per field (FP32 with compensated sums against FP64)."""
import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W
from tests.parity import load_both

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / nb) if nb > 0 else float(np.linalg.norm(a))


def check(wl, grid=48, blur=True, history=None, view=None):
    g, o = load_both(wl, history=history)
    L = wl.params.domain_w
    left, top, cw, ch = view if view else (-0.1 * L, -0.05 * L, 1.2 * L / grid, 1.1 * L / grid)
    hg = g.heatmap(left, top, cw, ch, grid, blur=blur)
    ho = o.heatmap(left, top, cw, ch, grid, blur=blur)
    g.close()
    o.close()
    for k in ("gravity", "electric", "yukawa"):
        if np.linalg.norm(ho[k]) == 0:
            assert np.linalg.norm(hg[k]) == 0, k
            continue
        e = rel(hg[k], ho[k])
        assert e <= TOL, (k, e)


def _with(wl, on=0, off=0):
    wl.params.toggles = (wl.params.toggles | on) & ~off
    return wl


@pytest.mark.parametrize("bh", [True, False])
@pytest.mark.parametrize("blur", [True, False])
def test_open_box(gpu_lib, bh, blur):
    wl = W.small_disk(2048, relativity=False, softening=8.0, barnes_hut=bh)
    check(_with(wl, on=N.YUKAWA), blur=blur)


@pytest.mark.parametrize("bh", [True, False])
def test_torus_with_yukawa(gpu_lib, bh):
    wl = W.clusters_torus(4096, relativity=False, barnes_hut=bh)
    check(_with(wl, off=N.MAGNETIC | N.GRAVITOMAG | N.ONE_PN | N.SPIN_ORBIT), grid=40)


@pytest.mark.parametrize("bh", [True, False])
def test_signal_delay(gpu_lib, bh):
    wl = W.small_disk(1024, relativity=True, softening=8.0, barnes_hut=bh)
    hist = W.straight_line_history(wl.state, 40, 0.0, 64 / 60)
    check(wl, grid=32, history=hist)


def test_fields_mask_and_grid_shape(gpu_lib):
    wl = W.small_disk(512, relativity=False, softening=8.0)
    g, o = load_both(wl)
    h = g.heatmap(0.0, 0.0, 2.0, 3.0, 50, fields=N.GEON_HEAT_ELECTRIC if hasattr(N, "GEON_HEAT_ELECTRIC") else 2)
    assert h["gravity"].shape == (50, 50)
    assert not h["gravity"].any() and h["electric"].any() and not h["yukawa"].any()
    g.close()
    o.close()
