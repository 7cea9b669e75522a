"""physsim_gb300 — GB300-native force-and-push path of Geon (a9lim/physsim).

The compute path is libgeon_cuda.so (hand-written sm_103a CUDA behind the C
ABI in include/geon.h).  This package builds it, binds it with ctypes and
mirrors the reference's GPUPhysics backend surface on top of it.
"""
from . import _native
from .build import build
from .system import GeonSystem

__all__ = ["build", "GeonSystem", "_native"]
__version__ = "1.0.0"
