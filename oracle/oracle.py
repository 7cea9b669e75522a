"""ctypes wrapper of the FP64 oracle (oracle/geon_oracle.cpp).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  Its API mirrors
physsim_gb300.system.GeonSystem so a test can drive both with one script.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from physsim_gb300 import _native as N

HERE = Path(__file__).resolve().parent
SRC = HERE / "geon_oracle.cpp"
LIB = HERE / "libgeon_oracle.so"


def build(force: bool = False) -> Path:
    """Compiles the oracle with g++ (OpenMP for the threaded CPU baseline)."""
    hdr = HERE.parent / "include" / "geon.h"
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-o", str(tmp), str(SRC)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    P = C.POINTER
    d, i, v = C.c_double, C.c_int, C.c_void_p
    sig = {
        "oracle_create": ([P(N.GeonParams)], v),
        "oracle_destroy": ([v], None),
        "oracle_set_params": ([v, P(N.GeonParams)], None),
        "oracle_set_threads": ([v, i], None),
        "oracle_max_threads": ([], i),
        "oracle_add_particles": ([v, i] + [P(d)] * 7 + [d], i),
        "oracle_count": ([v], i),
        "oracle_set_sim_time": ([v, d], None),
        "oracle_sim_time": ([v], d),
        "oracle_last_substeps": ([v], i),
        "oracle_interactions": ([v], C.c_longlong),
        "oracle_pe": ([v], d),
        "oracle_set_forces_init": ([v, i], None),
        "oracle_update": ([v, d], i),
        "oracle_compute_forces": ([v], None),
        "oracle_compute_forces_no_build": ([v], None),
        "oracle_compute_1pn": ([v], None),
        "oracle_get_state": ([v, P(d), i], i),
        "oracle_get_ids": ([v, P(C.c_int), i], None),
        "oracle_get_forces": ([v, P(d), i], i),
        "oracle_build_tree": ([v, P(C.c_int)], i),
        "oracle_tree_overflow": ([v], i),
        "oracle_tree_leaves": ([v, P(C.c_int), i, P(d), P(d), P(d), P(C.c_int), i], i),
        "oracle_ghost_origins": ([v, P(C.c_int), i], i),
        "oracle_tree_nodes": ([v, P(d), P(C.c_int), i], i),
        "oracle_upload_history": ([v, i, i, P(d), P(d)], i),
        "oracle_set_hist_stride": ([v, i], None),
        "oracle_stats": ([v, P(N.GeonStats)], None),
        "oracle_min_image": ([d, d, d, d, i, d, d, P(d)], None),
        "oracle_delayed_state": ([v, i, d, d, P(d)], i),
        "oracle_compute_forces_subset": ([v, P(C.c_int), i], C.c_longlong),
        "oracle_heatmap": ([v, d, d, d, d, i, C.c_uint, i, P(d), P(d), P(d)], None),
        "oracle_set_matter": ([v, i, P(C.c_int), P(d)], None),
        "oracle_tree_leaf_slots": ([v, P(C.c_int), i], None),
        "oracle_set_bosons": ([v, i, P(d)], None),
        "oracle_boson_kicks": ([v, d, C.c_uint, P(d)], None),
        "oracle_get_matter": ([v, P(C.c_int), P(d), i], i),
        "oracle_collision_events": ([v, P(d), i], i),
        "oracle_collision_counts": ([v, P(C.c_int)], None),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def max_threads() -> int:
    return load().oracle_max_threads()


def min_image(ox, oy, sx, sy, topology, W, H):
    out = np.zeros(2)
    load().oracle_min_image(ox, oy, sx, sy, topology, W, H, _dp(out))
    return out


class OracleSim:
    """FP64 restatement of the reference's Physics + QuadTreePool."""

    def __init__(self, params: N.GeonParams, threads: int = 1):
        self.lib = load()
        self.params = params
        self._h = self.lib.oracle_create(C.byref(params))
        self.lib.oracle_set_threads(self._h, threads)

    def close(self):
        if self._h:
            self.lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self.params = params
        self.lib.oracle_set_params(self._h, C.byref(params))

    def set_threads(self, n: int):
        self.lib.oracle_set_threads(self._h, n)

    def add(self, x, y, wx, wy, mass, charge, angw, creation_time=float("-inf")) -> int:
        cols = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (x, y, wx, wy, mass, charge, angw)]
        n = cols[0].size
        return self.lib.oracle_add_particles(self._h, n, *[_dp(c) for c in cols], creation_time)

    def count(self) -> int:
        return self.lib.oracle_count(self._h)

    def update(self, dt: float) -> int:
        return self.lib.oracle_update(self._h, dt)

    def compute_forces(self):
        self.lib.oracle_compute_forces(self._h)

    def compute_forces_subset(self, idx) -> int:
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        return self.lib.oracle_compute_forces_subset(self._h, _ip(idx), idx.size)

    def compute_1pn(self):
        self.lib.oracle_compute_1pn(self._h)

    def state(self) -> dict:
        n = self.count()
        out = np.zeros((10, max(n, 1)))
        self.lib.oracle_get_state(self._h, _dp(out), max(n, 1))
        return {k: out[r, :n].copy() for r, k in enumerate(N.ST_NAMES)}

    def ids(self) -> np.ndarray:
        n = self.count()
        out = np.zeros(max(n, 1), dtype=np.int32)
        self.lib.oracle_get_ids(self._h, _ip(out), max(n, 1))
        return out[:n]

    def forces(self) -> dict:
        n = self.count()
        out = np.zeros((N.OUT_ROWS, max(n, 1)))
        self.lib.oracle_get_forces(self._h, _dp(out), max(n, 1))
        return {k: out[r, :n].copy() for r, k in enumerate(N.OUT_NAMES)}

    def build_tree(self):
        nn = C.c_int()
        npts = self.lib.oracle_build_tree(self._h, C.byref(nn))
        return npts, nn.value

    def leaves(self, n_points: int):
        cap = max(4 * n_points + 8, 8)
        lop = np.zeros(max(n_points, 1), dtype=np.int32)
        bx = np.zeros(cap); by = np.zeros(cap); bw = np.zeros(cap)
        lv = np.zeros(cap, dtype=np.int32)
        nl = self.lib.oracle_tree_leaves(self._h, _ip(lop), n_points, _dp(bx), _dp(by), _dp(bw), _ip(lv), cap)
        return lop[:n_points], bx[:nl], by[:nl], bw[:nl], lv[:nl]

    def leaf_slots(self, n_points: int) -> np.ndarray:
        """Storage slot of each tree point in its leaf (insertion history order)."""
        out = np.zeros(max(n_points, 1), dtype=np.int32)
        self.lib.oracle_tree_leaf_slots(self._h, _ip(out), n_points)
        return out[:n_points]

    def ghost_origins(self) -> np.ndarray:
        n = self.lib.oracle_ghost_origins(self._h, None, 0)
        out = np.zeros(max(n, 1), dtype=np.int32)
        self.lib.oracle_ghost_origins(self._h, _ip(out), n)
        return out[:n]

    def tree_nodes(self):
        total = self.lib.oracle_tree_nodes(self._h, None, None, 0)
        cap = max(total, 1)
        out = np.zeros((12, cap))
        meta = np.zeros((3, cap), dtype=np.int32)
        self.lib.oracle_tree_nodes(self._h, _dp(out), _ip(meta), cap)
        names = ["bx", "by", "bw", "mass", "charge", "mag", "angmom", "momx", "momy", "comx", "comy", "bh"]
        d = {k: out[r, :total] for r, k in enumerate(names)}
        d["divided"], d["count"], d["level"] = meta[0, :total], meta[1, :total], meta[2, :total]
        return d

    def upload_history(self, times, x, y, vx, vy, angw):
        times = np.ascontiguousarray(times, dtype=np.float64)
        planes = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, vx, vy, angw)]
        n, count = planes[0].shape
        samples = np.ascontiguousarray(np.stack(planes))
        rc = self.lib.oracle_upload_history(self._h, n, count, _dp(times), _dp(samples))
        if rc != 0:
            raise ValueError("history upload rejected")

    def set_sim_time(self, t):
        self.lib.oracle_set_sim_time(self._h, t)

    def sim_time(self):
        return self.lib.oracle_sim_time(self._h)

    def last_substeps(self):
        return self.lib.oracle_last_substeps(self._h)

    def interactions(self):
        return self.lib.oracle_interactions(self._h)

    def pe(self):
        return self.lib.oracle_pe(self._h)

    def stats(self) -> dict:
        s = N.GeonStats()
        self.lib.oracle_stats(self._h, C.byref(s))
        return s.as_dict()

    def delayed_state(self, src: int, ox: float, oy: float):
        out = np.zeros(5)
        ok = self.lib.oracle_delayed_state(self._h, src, ox, oy, _dp(out))
        return out if ok else None

    def heatmap(self, left, top, cell_w, cell_h, grid, fields=7, blur=True) -> dict:
        """Potential grids (heatmap.js:152-206, 278-302), grid x grid each."""
        out = [np.zeros(grid * grid) for _ in range(3)]
        self.lib.oracle_heatmap(self._h, left, top, cell_w, cell_h, grid, fields, 1 if blur else 0,
                                *[_dp(a) for a in out])
        return {k: a.reshape(grid, grid) for k, a in zip(("gravity", "electric", "yukawa"), out)}

    def set_matter(self, antimatter=None, base_mass=None):
        """Antimatter flags / base masses of the particles (None: unchanged)."""
        n = self.count()
        am = None if antimatter is None else np.ascontiguousarray(antimatter, dtype=np.int32)
        bm = None if base_mass is None else np.ascontiguousarray(base_mass, dtype=np.float64)
        self.lib.oracle_set_matter(self._h, n, None if am is None else _ip(am), None if bm is None else _dp(bm))

    def matter(self) -> dict:
        n = self.count()
        am = np.zeros(max(n, 1), dtype=np.int32)
        bm = np.zeros(max(n, 1))
        self.lib.oracle_get_matter(self._h, _ip(am), _dp(bm), max(n, 1))
        return {"antimatter": am[:n].astype(bool), "base_mass": bm[:n]}

    def collision_events(self) -> np.ndarray:
        """Events of the last update: rows (type, x, y, energy, px, py);
        type 1 annihilation, 2 merge."""
        k = self.lib.oracle_collision_events(self._h, None, 0)
        out = np.zeros((max(k, 1), 6))
        self.lib.oracle_collision_events(self._h, _dp(out), k)
        return out[:k]

    def collision_counts(self) -> dict:
        out = np.zeros(4, dtype=np.int32)
        self.lib.oracle_collision_counts(self._h, _ip(out))
        return dict(zip(("merges", "annihilations", "spawned", "removed"), out.tolist()))

    def set_bosons(self, rows):
        """Boson pool: rows (x, y, src_mass, src_charge, kind, vSq); kind 0 photon, 1 massive."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 6)
        self._bosons = len(rows)
        self.lib.oracle_set_bosons(self._h, len(rows), _dp(rows))

    def boson_kicks(self, dt: float, what: int = 3) -> np.ndarray:
        n = getattr(self, "_bosons", 0)
        out = np.zeros((max(n, 1), 2))
        self.lib.oracle_boson_kicks(self._h, dt, what, _dp(out))
        return out[:n]

    def set_forces_init(self, v: bool):
        self.lib.oracle_set_forces_init(self._h, 1 if v else 0)

    def set_hist_stride(self, v: int):
        self.lib.oracle_set_hist_stride(self._h, v)
