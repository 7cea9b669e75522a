"""ctypes binding of libgeon_cuda.so (declarations in include/geon.h).

Every call is checked: a negative status raises :class:`GeonError` with the
library's message.  The library must exist (``physsim_gb300.build.build()``);
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB

# ---- constants (include/geon.h) ---------------------------------------------
GEON_OK = 0
GEON_ERR_ARG = -1
GEON_ERR_FULL = -2
GEON_ERR_CUDA = -3
GEON_ERR_OVERFLOW = -4
GEON_ERR_TIMEOUT = -5
GEON_ERR_NOMEM = -6
GEON_ERR_UNSUPPORTED = -7

GRAVITY = 1 << 0
COULOMB = 1 << 1
MAGNETIC = 1 << 2
GRAVITOMAG = 1 << 3
ONE_PN = 1 << 4
RELATIVITY = 1 << 5
SPIN_ORBIT = 1 << 6
RADIATION = 1 << 7
BLACK_HOLE = 1 << 8
YUKAWA = 1 << 11
HIGGS = 1 << 12
AXION = 1 << 13
BARNES_HUT = 1 << 14

BOUND_DESPAWN, BOUND_BOUNCE, BOUND_LOOP = 0, 1, 2
TORUS, KLEIN, RP2 = 0, 1, 2
COL_PASS, COL_MERGE, COL_BOUNCE = 0, 1, 2

FLAG_PE = 1 << 0
FLAG_BREAKDOWN = 1 << 1
FLAG_NO_GHOSTS = 1 << 2
FLAG_SIMPLE_WALK = 1 << 3
FLAG_LEARN = 1 << 4
FLAG_BOSONS = 1 << 5
FLAG_SPLIT_FRAME = 1 << 6
FRAME_MAX_POINTS = 4096
MLP_NPARAM = 5538
LEARN_FEATURES = 14
LEARN_OUTPUTS = 6
LEARN_TARGETS = 18
DIRECT_NOALLOC_MAX_K = 16384
BATCH_MAX_SYSTEMS = 512
BATCH_TUNE_MODES = 13

OUT_ROWS = 25
OUT_NAMES = ["fx", "fy", "Bz", "Bgz", "dBzdx", "dBzdy", "dBgzdx", "dBgzdy", "tidal", "frameDrag",
             "f1pn_x", "f1pn_y", "pe", "grav_x", "grav_y", "coul_x", "coul_y", "mag_x", "mag_y",
             "gm_x", "gm_y", "yuk_x", "yuk_y", "ext_x", "ext_y"]
ST_ROWS_IN = 7
ST_ROWS = 10
ST_NAMES = ["x", "y", "wx", "wy", "mass", "charge", "angw", "vx", "vy", "angVel"]


class GeonParams(C.Structure):
    _fields_ = [
        ("toggles", C.c_uint32),
        ("flags", C.c_uint32),
        ("boundary_mode", C.c_int32),
        ("topology", C.c_int32),
        ("domain_w", C.c_double),
        ("domain_h", C.c_double),
        ("off_x", C.c_double),
        ("off_y", C.c_double),
        ("theta", C.c_double),
        ("softening", C.c_double),
        ("yukawa_mu", C.c_double),
        ("bounce_friction", C.c_double),
        ("ext_gravity", C.c_double),
        ("ext_gravity_angle", C.c_double),
        ("ext_electric", C.c_double),
        ("ext_electric_angle", C.c_double),
        ("ext_bz", C.c_double),
        ("max_substeps", C.c_int32),
        ("collision_mode", C.c_int32),
    ]


class GeonStats(C.Structure):
    _fields_ = [
        ("linear_ke", C.c_double), ("spin_ke", C.c_double), ("pe", C.c_double),
        ("px", C.c_double), ("py", C.c_double),
        ("orbital_ang_mom", C.c_double), ("spin_ang_mom", C.c_double),
        ("com_x", C.c_double), ("com_y", C.c_double), ("total_mass", C.c_double),
        ("sim_time", C.c_double),
        ("alive_count", C.c_int32), ("last_substeps", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GeonTreeInfo(C.Structure):
    _fields_ = [(k, C.c_int32) for k in
                ("n_points", "n_ghosts", "n_dropped", "n_internal", "n_leaves", "max_level", "n_bucket", "reserved")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GeonCollisionInfo(C.Structure):
    _fields_ = [(k, C.c_int32) for k in
                ("merges", "annihilations", "spawned", "removed", "candidates", "events", "events_dropped",
                 "order_approx")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GeonProfile(C.Structure):
    _fields_ = [("tree_ms", C.c_double), ("force_ms", C.c_double), ("onepn_ms", C.c_double), ("push_ms", C.c_double),
                ("tree_count", C.c_int64), ("force_count", C.c_int64), ("onepn_count", C.c_int64),
                ("push_count", C.c_int64), ("interactions", C.c_int64), ("particle_substeps", C.c_int64),
                ("learn_ms", C.c_double), ("learn_count", C.c_int64), ("learn_pairs", C.c_int64),
                ("collide_ms", C.c_double), ("collide_count", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def make_params(toggles=GRAVITY | COULOMB, flags=0, boundary_mode=BOUND_DESPAWN, topology=TORUS,
                domain_w=100.0, domain_h=100.0, off_x=0.0, off_y=0.0, theta=0.5, softening=8.0,
                yukawa_mu=0.15, bounce_friction=0.4, ext_gravity=0.0, ext_gravity_angle=np.pi * 0.5,
                ext_electric=0.0, ext_electric_angle=0.0, ext_bz=0.0, max_substeps=32,
                collision_mode=COL_PASS) -> GeonParams:
    """GeonParams with the reference's defaults (src/config.js, src/integrator.js:65-99)."""
    return GeonParams(toggles, flags, boundary_mode, topology, domain_w, domain_h, off_x, off_y, theta,
                      softening, yukawa_mu, bounce_friction, ext_gravity, ext_gravity_angle, ext_electric,
                      ext_electric_angle, ext_bz, max_substeps, collision_mode)


class GeonError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"geon error {code}: {msg}")
        self.code = code


_P = C.POINTER
_handle_t = C.c_void_p

# (name, argtypes) in declaration order of include/geon.h
SIGNATURES = {
    "geon_create": [_P(GeonParams), C.c_int32, _P(_handle_t)],
    "geon_destroy": [_handle_t],
    "geon_set_params": [_handle_t, _P(GeonParams)],
    "geon_get_params": [_handle_t, _P(GeonParams)],
    "geon_add_particles": [_handle_t, C.c_int32, _P(C.c_float), C.c_double, _P(C.c_int32)],
    "geon_remove_particle": [_handle_t, C.c_int32],
    "geon_upload_state": [_handle_t, C.c_int32, _P(C.c_float), C.c_double],
    "geon_download_state": [_handle_t, _P(C.c_float), C.c_int32, C.c_int32, _P(C.c_int32)],
    "geon_download_ids": [_handle_t, _P(C.c_int32), C.c_int32, _P(C.c_int32)],
    "geon_download_state_f64": [_handle_t, _P(C.c_double), C.c_int32, C.c_int32, _P(C.c_int32)],
    "geon_reset": [_handle_t],
    "geon_upload_state_f64": [_handle_t, C.c_int32, _P(C.c_double), C.c_double],
    "geon_particle_count": [_handle_t, _P(C.c_int32)],
    "geon_update": [_handle_t, C.c_double, _P(C.c_int32)],
    "geon_set_frame_wait": [_handle_t, C.c_int64, C.c_int32],
    "geon_frame_phases": [_handle_t, _P(C.c_double), C.c_int32],
    "geon_synchronize": [_handle_t],
    "geon_compute_forces": [_handle_t],
    "geon_compute_1pn": [_handle_t],
    "geon_direct_forces": [_handle_t, _P(C.c_int32), C.c_int32, _P(C.c_float), _P(C.c_float)],
    "geon_direct_forces_noalloc": [_handle_t, _P(C.c_int32), C.c_int32, _P(C.c_float), _P(C.c_float)],
    "geon_learn_dataset": [_handle_t, C.c_int32, C.c_int64, C.c_float, _P(C.c_float), _P(C.c_float),
                           _P(C.c_int32), _P(C.c_int64)],
    "geon_learn_apply": [_handle_t, _P(C.c_float), C.c_int64],
    "geon_learn_set_weights": [_handle_t, _P(C.c_float), C.c_int32],
    "geon_mlp_forward": [_handle_t, _P(C.c_float), _P(C.c_float), C.c_int32, _P(C.c_float)],
    "geon_mlp_grad": [_handle_t, _P(C.c_float), _P(C.c_float), _P(C.c_float), _P(C.c_float), C.c_int32,
                      _P(C.c_float), _P(C.c_double)],
    "geon_mlp_train": [_handle_t, _P(C.c_float), _P(C.c_float), _P(C.c_float), _P(C.c_float), C.c_int32, C.c_int32,
                       C.c_int32, C.c_float, C.c_uint64, _P(C.c_double)],
    "geon_create_batch": [_P(GeonParams), C.c_int32, _P(C.c_int32), _P(_handle_t)],
    "geon_batch_substeps": [_handle_t, _P(C.c_int32), C.c_int32],
    "geon_batch_set_mode": [_handle_t, C.c_int32, C.c_int32],
    "geon_batch_autotune": [_handle_t, C.c_double, C.c_int32, _P(C.c_int32), _P(C.c_double)],
    "geon_batch_set_shape": [_handle_t, C.c_int32, C.c_int32, C.c_int32, C.c_int32],
    "geon_batch_tune_mode": [C.c_int32, _P(C.c_int32)],
    "geon_heatmap": [_handle_t, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_uint32, C.c_int32,
                     _P(C.c_float), _P(C.c_float), _P(C.c_float)],
    "geon_set_matter": [_handle_t, C.c_int32, C.c_int32, _P(C.c_int32), _P(C.c_float)],
    "geon_get_matter": [_handle_t, _P(C.c_int32), _P(C.c_float), C.c_int32, _P(C.c_int32)],
    "geon_set_bosons": [_handle_t, C.c_int32, _P(C.c_double)],
    "geon_boson_kicks": [_handle_t, C.c_double, C.c_uint32, _P(C.c_float)],
    "geon_collision_info": [_handle_t, _P(GeonCollisionInfo)],
    "geon_collision_events": [_handle_t, _P(C.c_double), C.c_int32, _P(C.c_int32)],
    "geon_download_forces": [_handle_t, C.c_int32, C.c_int32, _P(C.c_float), C.c_int32],
    "geon_build_tree": [_handle_t, _P(GeonTreeInfo)],
    "geon_tree_leaves": [_handle_t, _P(C.c_int32), C.c_int32, _P(C.c_double), _P(C.c_double), _P(C.c_double),
                         _P(C.c_int32), C.c_int32],
    "geon_interaction_count": [_handle_t, _P(C.c_int64)],
    "geon_stats": [_handle_t, _P(GeonStats)],
    "geon_upload_history": [_handle_t, C.c_int32, C.c_int32, _P(C.c_double), _P(C.c_float)],
    "geon_set_sim_time": [_handle_t, C.c_double],
    "geon_get_sim_time": [_handle_t, _P(C.c_double)],
    "geon_profile": [_handle_t, C.c_int32, _P(GeonProfile)],
    "geon_fp32_peak": [_handle_t, _P(C.c_double)],
    "geon_get_stream": [_handle_t, _P(C.c_void_p)],
    "geon_launch_count": [_handle_t, _P(C.c_int64)],
    "geon_last_error": [_handle_t],
    "geon_version": [],
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Loads the library (once) and declares every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run physsim_gb300.build.build() (nvcc for sm_103a)")
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_char_p if name in ("geon_last_error", "geon_version") else C.c_int
    _lib = lib
    return lib


def check(lib, h, rc: int):
    if rc < 0:
        msg = lib.geon_last_error(h)
        raise GeonError(rc, msg.decode() if msg else "")
    return rc


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_float))


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_P(C.c_int32))
