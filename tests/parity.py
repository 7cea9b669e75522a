"""Shared helpers of the parity tests: drive the CUDA library and the FP64
oracle from one workload and compare them quantity by quantity."""
from __future__ import annotations

import numpy as np

from physsim_gb300 import _native as N
from physsim_gb300.system import GeonSystem

STATE_KEYS = ("x", "y", "wx", "wy", "mass", "charge", "angw")


def load_both(wl, capacity=None, oracle_threads=8, history=None):
    from oracle.oracle import OracleSim
    s = wl.state
    g = GeonSystem(wl.params, capacity or wl.n)
    g.upload(*[s[k] for k in STATE_KEYS])
    o = OracleSim(wl.params, threads=oracle_threads)
    o.add(*[s[k] for k in STATE_KEYS])
    if history is not None:
        times, X, Y, VX, VY, A = history
        g.upload_history(times, X, Y, VX, VY, A)
        o.upload_history(times, X, Y, VX, VY, A)
        g.set_sim_time(float(times[-1]))
        o.set_sim_time(float(times[-1]))
    return g, o


def rel_err(gpu: np.ndarray, ref: np.ndarray) -> dict:
    """Norm-wise and per-particle relative errors of one quantity.

    norm: ||gpu - ref||_2 / ||ref||_2 over all particles.
    max:  max_i |gpu_i - ref_i| / max(|ref_i|, 1e-3 * rms(ref)).
    """
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    d = gpu - ref
    nr = np.linalg.norm(ref)
    rms = nr / np.sqrt(max(ref.size, 1))
    if nr == 0:
        return {"norm": float(np.linalg.norm(d)), "max": float(np.abs(d).max(initial=0.0)), "scale": 0.0}
    floor = max(1e-3 * rms, 1e-300)
    return {"norm": float(np.linalg.norm(d) / nr),
            "max": float(np.max(np.abs(d) / np.maximum(np.abs(ref), floor))),
            "scale": float(rms)}


def vec_err(gx, gy, rx, ry) -> dict:
    """Relative error of a 2-vector quantity: per-particle |dF| / max(|F|, 1e-3 rms|F|)."""
    g = np.stack([gx, gy]).astype(np.float64)
    r = np.stack([rx, ry]).astype(np.float64)
    d = np.linalg.norm(g - r, axis=0)
    mag = np.linalg.norm(r, axis=0)
    nr = np.linalg.norm(r)
    if nr == 0:
        return {"norm": float(np.linalg.norm(d)), "max": float(d.max(initial=0.0)), "p999": 0.0}
    rms = nr / np.sqrt(mag.size)
    rel = d / np.maximum(mag, 1e-3 * rms)
    return {"norm": float(np.linalg.norm(d) / nr), "max": float(rel.max()),
            "p999": float(np.quantile(rel, 0.999))}


def leaf_signature(bx, by, bw, lv, lop):
    """Per tree point: the exact (centre, half-size, level) of its leaf, or None."""
    out = []
    for l in lop:
        out.append(None if l < 0 else (float(bx[l]), float(by[l]), float(bw[l]), int(lv[l])))
    return out


def compare_trees(g: GeonSystem, o) -> dict:
    info = g.build_tree()
    lop, bx, by, bw, lv = g.leaves(info)
    npts, _ = o.build_tree()
    olop, obx, oby, obw, olv = o.leaves(npts)
    res = {"gpu_points": info["n_points"], "oracle_points": npts, "gpu_leaves": info["n_leaves"],
           "oracle_leaves": len(obx), "n_bucket": info["n_bucket"], "max_level": info["max_level"]}
    if npts != info["n_points"]:
        res["mismatch"] = npts
        return res
    sg = leaf_signature(bx, by, bw, lv, lop)
    so = leaf_signature(obx, oby, obw, olv, olop)
    bad = sum(1 for a, b in zip(sg, so) if a != b)
    # grouping: points sharing a leaf on one side share it on the other
    gmap, omap = {}, {}
    for i, (a, b) in enumerate(zip(sg, so)):
        gmap.setdefault(a, set()).add(i)
        omap.setdefault(b, set()).add(i)
    groups_equal = sorted(map(sorted, gmap.values())) == sorted(map(sorted, omap.values()))
    res["mismatch"] = bad
    res["groups_equal"] = groups_equal
    return res
