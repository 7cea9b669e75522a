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
