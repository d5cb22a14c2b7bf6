"""GB300-native (sm_103a) implementation of VectorTA's GPU indicator hot path.

The compute lives in libvta_gb300.so (hand-written CUDA for sm_103a behind the
C ABI in include/vta_gb300.h); this package is the Python mirror of the
crate's per-indicator CUDA wrappers.  Build with ``vectorta_gb300.build.build()``.
"""
from . import datagen  # noqa: F401
from ._native import INDICATORS, VtaError  # noqa: F401

try:
    from .cuda import *  # noqa: F401,F403
    from .cuda import CLASSES, Context, DeviceArrayF32, device_count  # noqa: F401
except ImportError as e:  # library not built yet: import works, calls fail loudly
    _import_error = e

    def __getattr__(name):
        raise ImportError(f"vectorta_gb300 native library unavailable: {_import_error}")

__version__ = "0.1.0"
