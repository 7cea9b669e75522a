"""The C-ABI library loads and exports every entry point include/geon.h declares
(no compute call: these run without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "geon.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(geon_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "geon_create" in syms and "geon_update" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol(gpu_lib):
    missing = [s for s in declared_symbols() if not hasattr(gpu_lib, s)]
    assert not missing, f"missing exports: {missing}"


def test_bindings_cover_header(gpu_lib):
    from physsim_gb300 import _native as N
    assert sorted(N.SIGNATURES) == declared_symbols()


def test_integration_notes_name_every_entry_point():
    notes = (ROOT / "INTEGRATION.md").read_text()
    missing = [s for s in declared_symbols() if s not in notes]
    assert not missing, f"entry points INTEGRATION.md does not name: {missing}"


def test_version_and_error_strings(gpu_lib):
    assert gpu_lib.geon_version().startswith(b"geon-gb300")
    assert isinstance(gpu_lib.geon_last_error(None), bytes)


def test_params_struct_layout():
    from physsim_gb300 import _native as N
    # 4 x 4-byte ints, 13 doubles, 2 ints
    assert ctypes.sizeof(N.GeonParams) == 16 + 13 * 8 + 8
    assert ctypes.sizeof(N.GeonTreeInfo) == 32


def test_create_rejects_bad_arguments(gpu_lib):
    """Argument checks run on the host before any device work."""
    from physsim_gb300 import _native as N
    h = ctypes.c_void_p()
    p = N.make_params(domain_w=-1.0)
    assert gpu_lib.geon_create(ctypes.byref(p), 16, ctypes.byref(h)) == N.GEON_ERR_ARG
    p = N.make_params()
    assert gpu_lib.geon_create(ctypes.byref(p), 0, ctypes.byref(h)) == N.GEON_ERR_ARG
    p = N.make_params(toggles=N.GRAVITY | N.HIGGS)
    assert gpu_lib.geon_create(ctypes.byref(p), 16, ctypes.byref(h)) == N.GEON_ERR_UNSUPPORTED
    assert b"Higgs" in gpu_lib.geon_last_error(None)


def test_batch_tune_modes_table(gpu_lib):
    """The autotuner's candidates (a host table, no device work): the header's
    count, every shape geon_batch_set_shape accepts, the short-stack walk at
    seven CTAs per SM among them, and GEON_ERR_ARG past the end."""
    from physsim_gb300 import _native as N
    from physsim_gb300.system import BatchSystem
    text = HEADER.read_text()
    assert int(re.search(r"#define GEON_BATCH_TUNE_MODES (\d+)", text).group(1)) == N.BATCH_TUNE_MODES == 13
    modes = [BatchSystem.tune_mode(m) for m in range(N.BATCH_TUNE_MODES)]
    for d in modes:
        assert d["use_graph"] in (0, 1) and d["simple_walk"] in (0, 1)
        assert d["warps_per_group"] in (1, 4) and d["ctas_per_sm"] in (0, 3, 4, 5, 7)
        assert d["queue_chunk"] in (0, 1, 4)
        # one shape at a time: split walk, CTA cap, or work queue
        assert sum([d["warps_per_group"] > 1, d["ctas_per_sm"] > 0, d["queue_chunk"] > 0]) <= 1
    assert any(d["ctas_per_sm"] == 7 for d in modes)
    assert len({tuple(sorted(d.items())) for d in modes}) == len(modes)
    desc = (ctypes.c_int32 * 6)()
    assert gpu_lib.geon_batch_tune_mode(N.BATCH_TUNE_MODES, desc) == N.GEON_ERR_ARG
    assert gpu_lib.geon_batch_tune_mode(-1, desc) == N.GEON_ERR_ARG
