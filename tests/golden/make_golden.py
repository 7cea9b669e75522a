"""Generates the golden fixtures of tests/test_golden.py from the FP64 oracle.

The reference (browser JavaScript, no tests) has no golden vectors of its
own, so these fixtures pin the oracle restatement against regressions and
give the GPU tests fixed expected outputs.  Each case is a small seeded
workload of physsim_gb300.workloads; per case the file stores the tree's
leaf of every tree point (centre, half-size, level), the force pass
outputs and the state after one frame.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from physsim_gb300 import _native as N  # noqa: E402
from physsim_gb300 import workloads as W  # noqa: E402

STATE_KEYS = ("x", "y", "wx", "wy", "mass", "charge", "angw")
FORCE_KEYS = ("fx", "fy", "Bz", "Bgz", "dBzdx", "dBzdy", "dBgzdx", "dBgzdy", "tidal", "frameDrag", "f1pn_x",
              "f1pn_y", "pe")


def cases():
    """name -> (workload, history or None)."""
    out = {}
    out["disk256_gc"] = (W.small_disk(256, seed=21, relativity=False, softening=8.0), None)
    wl = W.clusters_torus(384, seed=22, relativity=False)
    wl.params.toggles &= ~N.ONE_PN          # 1PN needs relativity (Q7)
    out["torus384_full"] = (wl, None)
    wl = W.plummer_disk(512, seed=23, theta=0.5)
    out["plummer512_gcy"] = (wl, None)
    wl = W.small_disk(192, seed=24, relativity=True, softening=8.0)
    hist = W.straight_line_history(wl.state, 40, 0.0, 64 / 60)
    out["disk192_delay"] = (wl, hist)
    return out


def run_case(wl, hist):
    from oracle.oracle import OracleSim
    o = OracleSim(wl.params, threads=4)
    s = wl.state
    o.add(*[s[k] for k in STATE_KEYS])
    if hist is not None:
        o.upload_history(*hist)
        o.set_sim_time(float(hist[0][-1]))
    npts, _ = o.build_tree()
    lop, bx, by, bw, lv = o.leaves(npts)
    leaf = np.full((npts, 4), np.nan)
    ok = lop >= 0
    leaf[ok, 0] = bx[lop[ok]]
    leaf[ok, 1] = by[lop[ok]]
    leaf[ok, 2] = bw[lop[ok]]
    leaf[ok, 3] = lv[lop[ok]]
    o.compute_forces()
    f = o.forces()
    forces = np.stack([np.asarray(f[k], dtype=np.float64) for k in FORCE_KEYS])
    inter = o.interactions()
    o.update(wl.dt)
    st = o.state()
    state = np.stack([np.asarray(st[k], dtype=np.float64) for k in ("x", "y", "wx", "wy")])
    sub = o.last_substeps()
    o.close()
    return dict(leaf=leaf, forces=forces, interactions=np.int64(inter), state1=state, substeps=np.int64(sub))


def main():
    from oracle import oracle
    oracle.build()
    for name, (wl, hist) in cases().items():
        res = run_case(wl, hist)
        np.savez_compressed(HERE / f"{name}.npz", **res)
        print(name, {k: getattr(v, "shape", v) for k, v in res.items()})


if __name__ == "__main__":
    main()
