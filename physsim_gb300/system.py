"""Pythonic handle over the C ABI: one GPU-resident particle system."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


class GeonSystem:
    """Owns one ``GeonHandle``.  Arrays in and out are host NumPy arrays."""

    def __init__(self, params: N.GeonParams, capacity: int):
        self.lib = N.load()
        self._h = C.c_void_p()
        rc = self.lib.geon_create(C.byref(params), int(capacity), C.byref(self._h))
        if rc < 0:
            raise N.GeonError(rc, self.lib.geon_last_error(None).decode())
        self.capacity = int(capacity)

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if self._h:
            self.lib.geon_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        return N.check(self.lib, self._h, rc)

    # -- parameters -----------------------------------------------------------
    def set_params(self, params: N.GeonParams):
        self._ck(self.lib.geon_set_params(self._h, C.byref(params)))

    def params(self) -> N.GeonParams:
        p = N.GeonParams()
        self._ck(self.lib.geon_get_params(self._h, C.byref(p)))
        return p

    # -- state ------------------------------------------------------------------
    @staticmethod
    def _rows(x, y, wx, wy, mass, charge, angw) -> np.ndarray:
        cols = [np.asarray(a, dtype=np.float32).ravel() for a in (x, y, wx, wy, mass, charge, angw)]
        n = cols[0].size
        if any(c.size != n for c in cols):
            raise ValueError("state arrays must have equal length")
        return np.ascontiguousarray(np.stack(cols)), n

    def add(self, x, y, wx, wy, mass, charge, angw, creation_time: float = float("-inf")) -> int:
        rows, n = self._rows(x, y, wx, wy, mass, charge, angw)
        first = C.c_int32()
        self._ck(self.lib.geon_add_particles(self._h, n, N.fptr(rows), creation_time, C.byref(first)))
        return first.value

    def upload(self, x, y, wx, wy, mass, charge, angw, sim_time: float = 0.0):
        rows, n = self._rows(x, y, wx, wy, mass, charge, angw)
        self._ck(self.lib.geon_upload_state(self._h, n, N.fptr(rows), sim_time))

    def upload_f64(self, x, y, wx, wy, mass, charge, angw, sim_time: float = 0.0):
        """upload() from doubles: positions keep their compensated low parts."""
        cols = [np.asarray(a, dtype=np.float64).ravel() for a in (x, y, wx, wy, mass, charge, angw)]
        n = cols[0].size
        rows = np.ascontiguousarray(np.stack(cols)) if n else np.zeros((7, 1))
        self._ck(self.lib.geon_upload_state_f64(self._h, n, N.dptr(rows), sim_time))

    def count(self) -> int:
        n = C.c_int32()
        self._ck(self.lib.geon_particle_count(self._h, C.byref(n)))
        return n.value

    def state(self, f64: bool = False) -> dict:
        n = self.count()
        cap = max(n, 1)
        if f64:
            out = np.zeros((N.ST_ROWS, cap), dtype=np.float64)
            self._ck(self.lib.geon_download_state_f64(self._h, N.dptr(out), N.ST_ROWS, cap, None))
        else:
            out = np.zeros((N.ST_ROWS, cap), dtype=np.float32)
            self._ck(self.lib.geon_download_state(self._h, N.fptr(out), N.ST_ROWS, cap, None))
        return {k: out[r, :n].copy() for r, k in enumerate(N.ST_NAMES)}

    def ids(self) -> np.ndarray:
        n = self.count()
        out = np.zeros(max(n, 1), dtype=np.int32)
        self._ck(self.lib.geon_download_ids(self._h, N.iptr(out), out.size, None))
        return out[:n]

    def remove(self, index: int):
        self._ck(self.lib.geon_remove_particle(self._h, int(index)))

    def reset(self):
        self._ck(self.lib.geon_reset(self._h))

    # -- stepping ------------------------------------------------------------
    def update(self, dt: float) -> int:
        s = C.c_int32()
        self._ck(self.lib.geon_update(self._h, float(dt), C.byref(s)))
        return s.value

    FRAME_PHASES = ("scan", "push+keys", "sort", "gather", "scans", "emit", "link", "aggregate", "walk", "rest")

    def frame_phases(self) -> dict:
        """Phase durations (us) of the last one-launch frame."""
        out = (C.c_double * 16)()
        k = self._ck(self.lib.geon_frame_phases(self._h, out, 16))
        return {name: float(out[i]) for i, name in enumerate(self.FRAME_PHASES[:k])}

    def set_frame_wait(self, wait_ns: int = 1_000_000_000, extra_arrivals: int = 0):
        """Time limit of the one-launch frame's barriers; extra_arrivals > 0
        makes them wait for blocks that do not exist (time-out test)."""
        self._ck(self.lib.geon_set_frame_wait(self._h, int(wait_ns), int(extra_arrivals)))

    def synchronize(self):
        self._ck(self.lib.geon_synchronize(self._h))

    def compute_forces(self):
        self._ck(self.lib.geon_compute_forces(self._h))

    def compute_1pn(self):
        self._ck(self.lib.geon_compute_1pn(self._h))

    def direct_forces(self, idx) -> tuple:
        """Pairwise (fx, fy) on the listed particles from all particles; state unchanged."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        fx = np.zeros(max(idx.size, 1), dtype=np.float32)
        fy = np.zeros(max(idx.size, 1), dtype=np.float32)
        self._ck(self.lib.geon_direct_forces(self._h, N.iptr(idx), idx.size, N.fptr(fx), N.fptr(fy)))
        return fx[:idx.size], fy[:idx.size]

    def learn_dataset(self, group_stride: int = 1, cap: int | None = None, gfloor: float = 0.0) -> dict:
        """Training records of the learned correction at the current theta for
        the groups 0, stride, 2 stride, ... (geon_learn_dataset): features
        [m, 14], targets [m, 18] (y*[6], A[12]) and the group of each record.
        With cap None the records are counted first and all returned."""
        if cap is None:
            cnt = C.c_int64()
            self._ck(self.lib.geon_learn_dataset(self._h, int(group_stride), 0, float(gfloor), None, None, None,
                                                 C.byref(cnt)))
            cap = cnt.value
        cap = int(cap)
        feat = np.zeros((max(cap, 1), N.LEARN_FEATURES), dtype=np.float32)
        tg = np.zeros((max(cap, 1), N.LEARN_TARGETS), dtype=np.float32)
        grp = np.zeros(max(cap, 1), dtype=np.int32)
        cnt = C.c_int64()
        self._ck(self.lib.geon_learn_dataset(self._h, int(group_stride), cap, float(gfloor), N.fptr(feat), N.fptr(tg),
                                             N.iptr(grp), C.byref(cnt)))
        m = min(cnt.value, cap)
        return {"count": cnt.value, "feat": feat[:m], "target": tg[:m], "group": grp[:m]}

    def learn_apply(self, y):
        """Barnes-Hut force pass plus the correction with the given network
        outputs y[m, 6] for the records of all groups (geon_learn_apply)."""
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1, N.LEARN_OUTPUTS)
        self._ck(self.lib.geon_learn_apply(self._h, N.fptr(y), len(y)))

    def learn_set_weights(self, weights):
        """Weights of the learned correction (None clears them)."""
        if weights is None:
            self._ck(self.lib.geon_learn_set_weights(self._h, None, 0))
            return
        w = np.ascontiguousarray(weights, dtype=np.float32)
        self._ck(self.lib.geon_learn_set_weights(self._h, N.fptr(w), w.size))

    def mlp_forward(self, weights, x) -> np.ndarray:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N.LEARN_FEATURES)
        y = np.zeros((max(len(x), 1), N.LEARN_OUTPUTS), dtype=np.float32)
        self._ck(self.lib.geon_mlp_forward(self._h, N.fptr(w), N.fptr(x), len(x), N.fptr(y)))
        return y[:len(x)]

    def mlp_grad(self, weights, x, t, wt=None) -> tuple:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N.LEARN_FEATURES)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, N.LEARN_TARGETS)
        wp = None
        if wt is not None:
            wt = np.ascontiguousarray(wt, dtype=np.float32)
            wp = N.fptr(wt)
        g = np.zeros(N.MLP_NPARAM, dtype=np.float32)
        loss = C.c_double()
        self._ck(self.lib.geon_mlp_grad(self._h, N.fptr(w), N.fptr(x), N.fptr(t), wp, len(x), N.fptr(g),
                                        C.byref(loss)))
        return g, loss.value

    def mlp_train(self, weights, x, t, steps: int, batch: int, lr: float, seed: int = 1, wt=None) -> tuple:
        """Adam training on the device; returns (trained weights, per-step loss)."""
        w = np.array(weights, dtype=np.float32, copy=True)
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N.LEARN_FEATURES)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, N.LEARN_TARGETS)
        wp = None
        if wt is not None:
            wt = np.ascontiguousarray(wt, dtype=np.float32)
            wp = N.fptr(wt)
        hist = np.zeros(max(int(steps), 1), dtype=np.float64)
        self._ck(self.lib.geon_mlp_train(self._h, N.fptr(w), N.fptr(x), N.fptr(t), wp, len(x), int(steps), int(batch),
                                         float(lr), int(seed), hist.ctypes.data_as(C.POINTER(C.c_double))))
        return w, hist[:int(steps)]

    def heatmap(self, left: float, top: float, cell_w: float, cell_h: float, grid: int, fields: int = 7,
                blur: bool = True) -> dict:
        """Gravitational, electric and Yukawa potential grids (grid x grid)."""
        out = [np.zeros(grid * grid, dtype=np.float32) for _ in range(3)]
        self._ck(self.lib.geon_heatmap(self._h, float(left), float(top), float(cell_w), float(cell_h), int(grid),
                                       int(fields), 1 if blur else 0, *[N.fptr(a) for a in out]))
        return {k: a.reshape(grid, grid) for k, a in zip(("gravity", "electric", "yukawa"), out)}

    def set_matter(self, antimatter=None, base_mass=None, first: int = 0):
        """Antimatter flags / base masses of particles first, first+1, ... (None: unchanged)."""
        arrs = [a for a in (antimatter, base_mass) if a is not None]
        if not arrs:
            return
        k = len(arrs[0])
        am = None if antimatter is None else np.ascontiguousarray(antimatter, dtype=np.int32)
        bm = None if base_mass is None else np.ascontiguousarray(base_mass, dtype=np.float32)
        self._ck(self.lib.geon_set_matter(self._h, int(first), int(k), None if am is None else N.iptr(am),
                                          None if bm is None else N.fptr(bm)))

    def matter(self) -> dict:
        n = self.count()
        am = np.zeros(max(n, 1), dtype=np.int32)
        bm = np.zeros(max(n, 1), dtype=np.float32)
        cnt = C.c_int32()
        self._ck(self.lib.geon_get_matter(self._h, N.iptr(am), N.fptr(bm), max(n, 1), C.byref(cnt)))
        return {"antimatter": am[:n].astype(bool), "base_mass": bm[:n]}

    def set_bosons(self, rows):
        """Boson pool: rows (x, y, src_mass, src_charge, kind, v^2); kind 0 photon, 1 pion or lepton."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 6)
        self._nb = len(rows)
        self._ck(self.lib.geon_set_bosons(self._h, len(rows), N.dptr(rows) if len(rows) else None))

    def boson_kicks(self, dt: float, what: int = 3) -> np.ndarray:
        n = getattr(self, "_nb", 0)
        out = np.zeros((max(n, 1), 2), dtype=np.float32)
        self._ck(self.lib.geon_boson_kicks(self._h, float(dt), int(what), N.fptr(out)))
        return out[:n]

    def collision_info(self) -> dict:
        info = N.GeonCollisionInfo()
        self._ck(self.lib.geon_collision_info(self._h, C.byref(info)))
        return info.as_dict()

    def collision_events(self) -> np.ndarray:
        """Events of the last update: rows (type, x, y, energy, px, py);
        type 1 annihilation, 2 merge."""
        cnt = C.c_int32()
        self._ck(self.lib.geon_collision_events(self._h, None, 0, C.byref(cnt)))
        out = np.zeros((max(cnt.value, 1), 6))
        self._ck(self.lib.geon_collision_events(self._h, N.dptr(out), cnt.value, C.byref(cnt)))
        return out[:cnt.value]

    def forces(self) -> dict:
        n = self.count()
        cap = max(n, 1)
        out = np.zeros((N.OUT_ROWS, cap), dtype=np.float32)
        self._ck(self.lib.geon_download_forces(self._h, 0, N.OUT_ROWS, N.fptr(out), cap))
        return {k: out[r, :n].copy() for r, k in enumerate(N.OUT_NAMES)}

    # -- tree --------------------------------------------------------------
    def build_tree(self) -> dict:
        info = N.GeonTreeInfo()
        self._ck(self.lib.geon_build_tree(self._h, C.byref(info)))
        return info.as_dict()

    def leaves(self, info: dict | None = None):
        info = info or self.build_tree()
        npts, nl = max(info["n_points"], 1), max(info["n_leaves"], 1)
        lop = np.zeros(npts, dtype=np.int32)
        bx = np.zeros(nl); by = np.zeros(nl); bw = np.zeros(nl)
        lv = np.zeros(nl, dtype=np.int32)
        self._ck(self.lib.geon_tree_leaves(self._h, N.iptr(lop), npts, N.dptr(bx), N.dptr(by), N.dptr(bw),
                                           N.iptr(lv), nl))
        n = info["n_leaves"]
        return lop[:info["n_points"]], bx[:n], by[:n], bw[:n], lv[:n]

    def interactions(self) -> int:
        c = C.c_int64()
        self._ck(self.lib.geon_interaction_count(self._h, C.byref(c)))
        return c.value

    # -- diagnostics ---------------------------------------------------------------
    def stats(self) -> dict:
        s = N.GeonStats()
        self._ck(self.lib.geon_stats(self._h, C.byref(s)))
        return s.as_dict()

    def upload_history(self, times, x, y, vx, vy, angw):
        times = np.ascontiguousarray(times, dtype=np.float64)
        planes = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, vx, vy, angw)]
        n, count = planes[0].shape
        samples = np.ascontiguousarray(np.stack(planes))
        self._ck(self.lib.geon_upload_history(self._h, n, count, N.dptr(times), N.fptr(samples)))

    def set_sim_time(self, t: float):
        self._ck(self.lib.geon_set_sim_time(self._h, float(t)))

    def sim_time(self) -> float:
        t = C.c_double()
        self._ck(self.lib.geon_get_sim_time(self._h, C.byref(t)))
        return t.value

    def profile(self, enable: bool) -> dict:
        """Starts (True) or stops (False) per-phase CUDA-event timing; returns totals so far."""
        out = N.GeonProfile()
        self._ck(self.lib.geon_profile(self._h, 1 if enable else 0, C.byref(out)))
        return out.as_dict()

    def stream_ptr(self) -> int:
        p = C.c_void_p()
        self._ck(self.lib.geon_get_stream(self._h, C.byref(p)))
        return p.value or 0

    def launch_count(self) -> int:
        c = C.c_int64()
        self._ck(self.lib.geon_launch_count(self._h, C.byref(c)))
        return c.value


class BatchSystem(GeonSystem):
    """Many independent systems with one parameter set in one handle
    (``geon_create_batch``).  State arrays are concatenated system by system;
    ``update`` advances every system by one frame."""

    def __init__(self, params: N.GeonParams, counts):
        self.lib = N.load()
        self._h = C.c_void_p()
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        rc = self.lib.geon_create_batch(C.byref(params), int(self.counts.size), N.iptr(self.counts), C.byref(self._h))
        if rc < 0:
            raise N.GeonError(rc, self.lib.geon_last_error(None).decode())
        self.capacity = int(self.counts.sum())
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)

    def substeps(self) -> np.ndarray:
        out = np.zeros(self.counts.size, dtype=np.int32)
        self._ck(self.lib.geon_batch_substeps(self._h, N.iptr(out), out.size))
        return out

    def set_mode(self, use_graph: bool = True, simple_walk: bool = False):
        self._ck(self.lib.geon_batch_set_mode(self._h, int(use_graph), int(simple_walk)))

    def set_shape(self, warps_per_group: int = 1, split_level: int = 6, ctas_per_sm: int = 0, queue_chunk: int = 0):
        self._ck(self.lib.geon_batch_set_shape(self._h, int(warps_per_group), int(split_level), int(ctas_per_sm),
                                               int(queue_chunk)))

    @staticmethod
    def tune_mode(mode: int) -> dict:
        """Candidate `mode` of autotune: graph, simple walk, warps per group, split level, CTAs per SM,
        work-queue chunk."""
        d = (C.c_int32 * 6)()
        lib = N.load()
        N.check(lib, None, lib.geon_batch_tune_mode(int(mode), d))
        return {"use_graph": bool(d[0]), "simple_walk": bool(d[1]), "warps_per_group": int(d[2]),
                "split_level": int(d[3]), "ctas_per_sm": int(d[4]), "queue_chunk": int(d[5])}

    def autotune(self, dt: float, frames: int = 2) -> tuple:
        """Times every candidate mode (tune_mode), keeps the fastest; returns
        (choice, ms per frame of each)."""
        ch = C.c_int32()
        ms = np.zeros(N.BATCH_TUNE_MODES, dtype=np.float64)
        self._ck(self.lib.geon_batch_autotune(self._h, float(dt), int(frames), C.byref(ch),
                                              ms.ctypes.data_as(C.POINTER(C.c_double))))
        return ch.value, ms
