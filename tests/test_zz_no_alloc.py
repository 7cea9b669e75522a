"""geon_direct_forces_noalloc through the C ABI: the same results as
geon_direct_forces on two calls in a row, without device allocation, and a
clear rejection of subsets beyond its fixed scratch.

The file name sorts last so that the test also runs after every other test
file in one process; it needs nothing from them and passes alone."""
import ctypes as C

import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300 import workloads as W
from physsim_gb300.system import GeonSystem
from tests.parity import STATE_KEYS

pytestmark = pytest.mark.gpu


def call(lib, fn, h, idx):
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    fx = np.full(max(idx.size, 1), np.nan, dtype=np.float32)
    fy = np.full(max(idx.size, 1), np.nan, dtype=np.float32)
    rc = getattr(lib, fn)(h, N.iptr(idx), idx.size, N.fptr(fx), N.fptr(fy))
    return rc, fx[:idx.size], fy[:idx.size]


def test_noalloc_matches_direct_forces_twice(gpu_lib):
    import torch
    wl = W.plummer_disk(40000, theta=0.5)
    g = GeonSystem(wl.params, wl.n)
    g.upload(*[wl.state[k] for k in STATE_KEYS])
    lib, h = g.lib, g._h
    rng = np.random.default_rng(4)
    first = rng.choice(wl.n, N.DIRECT_NOALLOC_MAX_K, replace=False).astype(np.int32)   # the maximum size
    second = rng.choice(wl.n, 777, replace=False).astype(np.int32)                      # then a smaller one
    # reference outputs from the allocating entry point
    rc, ax1, ay1 = call(lib, "geon_direct_forces", h, first)
    assert rc == N.GEON_OK
    rc, ax2, ay2 = call(lib, "geon_direct_forces", h, second)
    assert rc == N.GEON_OK
    # the first call on the device does the setup (address lookup; the
    # driver may load the module holding the scratch array)
    rc, sx, sy = call(lib, "geon_direct_forces_noalloc", h, second[:3])
    assert rc == N.GEON_OK, lib.geon_last_error(h)
    assert np.array_equal(sx, ax2[:3]) and np.array_equal(sy, ay2[:3])
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc, bx1, by1 = call(lib, "geon_direct_forces_noalloc", h, first)
    assert rc == N.GEON_OK, lib.geon_last_error(h)
    rc, bx2, by2 = call(lib, "geon_direct_forces_noalloc", h, second)
    assert rc == N.GEON_OK, lib.geon_last_error(h)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    # same kernel on the same inputs: identical bits
    assert np.array_equal(bx1, ax1) and np.array_equal(by1, ay1)
    assert np.array_equal(bx2, ax2) and np.array_equal(by2, ay2)
    assert np.isfinite(bx1).all() and np.isfinite(bx2).all()
    assert free1 == free0, (free0, free1)
    g.close()


def test_noalloc_rejects_oversize_and_bad_arguments(gpu_lib):
    wl = W.small_disk(512, relativity=False, softening=8.0)
    g = GeonSystem(wl.params, wl.n)
    g.upload(*[wl.state[k] for k in STATE_KEYS])
    lib, h = g.lib, g._h
    big = np.zeros(N.DIRECT_NOALLOC_MAX_K + 1, dtype=np.int32)
    rc, _, _ = call(lib, "geon_direct_forces_noalloc", h, big)
    assert rc == N.GEON_ERR_ARG
    msg = lib.geon_last_error(h).decode()
    assert "exceeds GEON_DIRECT_NOALLOC_MAX_K" in msg and str(N.DIRECT_NOALLOC_MAX_K) in msg
    rc, _, _ = call(lib, "geon_direct_forces_noalloc", h, np.array([wl.n], dtype=np.int32))
    assert rc == N.GEON_ERR_ARG
    assert lib.geon_direct_forces_noalloc(h, None, 3, None, None) == N.GEON_ERR_ARG
    rc, fx, fy = call(lib, "geon_direct_forces_noalloc", h, np.zeros(0, dtype=np.int32))
    assert rc == N.GEON_OK
    # still usable after the rejections
    rc, bx, by = call(lib, "geon_direct_forces_noalloc", h, np.arange(5, dtype=np.int32))
    assert rc == N.GEON_OK
    rc, ax, ay = call(lib, "geon_direct_forces", h, np.arange(5, dtype=np.int32))
    assert rc == N.GEON_OK and np.array_equal(ax, bx) and np.array_equal(ay, by)
    g.close()
