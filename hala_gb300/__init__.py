"""hala_gb300: GB300-native (sm_103a) sparse Krylov path with HALA's GPU-engine interface.

The compute lives in libhgb.so (hala_gb300/csrc, C ABI in include/hgb.h); this package is the
host-side mirror of the reference's gpu_engine overloads for Python callers and tests.
"""
from .hgb import HgbError, lib, lib_path  # noqa: F401

__version__ = "1.1.0"


def __getattr__(name):
    # the engine module imports torch; load it on first use
    if name in ("engine",):
        import importlib
        return importlib.import_module(".engine", __name__)
    raise AttributeError(name)
