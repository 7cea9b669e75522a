"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py
from the FP64 oracle): the oracle must reproduce them exactly, and the CUDA
path must match them at the parity tolerances — leaf membership exact,
forces <= 1e-5 norm-wise per quantity, BH interaction counts equal, one
frame of positions and velocities <= 1e-5 norm-wise with equal substeps."""
from pathlib import Path

import numpy as np
import pytest

from tests.golden.make_golden import FORCE_KEYS, STATE_KEYS, cases, run_case

GOLD = Path(__file__).resolve().parent / "golden"
CASES = sorted(cases())


def load(name):
    with np.load(GOLD / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name, oracle_mod):
    wl, hist = cases()[name]
    got = run_case(wl, hist)
    ref = load(name)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=f"{name}:{k}")


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(name, gpu_lib):
    from physsim_gb300.system import GeonSystem
    from physsim_gb300 import _native as N
    wl, hist = cases()[name]
    ref = load(name)
    wl.params.flags |= N.FLAG_PE            # the oracle always sums the potential energy
    g = GeonSystem(wl.params, wl.n)
    g.upload(*[wl.state[k] for k in STATE_KEYS])
    if hist is not None:
        g.upload_history(*hist)
        g.set_sim_time(float(hist[0][-1]))
    info = g.build_tree()
    lop, bx, by, bw, lv = g.leaves(info)
    assert info["n_points"] == len(ref["leaf"])
    leaf = np.full((info["n_points"], 4), np.nan)
    ok = lop >= 0
    leaf[ok, 0], leaf[ok, 1], leaf[ok, 2], leaf[ok, 3] = bx[lop[ok]], by[lop[ok]], bw[lop[ok]], lv[lop[ok]]
    np.testing.assert_array_equal(leaf, ref["leaf"])
    g.compute_forces()
    f = g.forces()
    for r, k in enumerate(FORCE_KEYS):
        e = rel(np.asarray(f[k], np.float64), ref["forces"][r])
        assert e <= 1e-5, (name, k, e)
    assert g.interactions() == int(ref["interactions"])
    sub = g.update(wl.dt)
    assert sub == int(ref["substeps"])
    st = g.state(f64=True)
    for r, k in enumerate(("x", "y", "wx", "wy")):
        e = rel(np.asarray(st[k], np.float64), ref["state1"][r])
        assert e <= 1e-5, (name, k, e)
    g.close()
