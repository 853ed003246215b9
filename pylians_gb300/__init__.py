"""pylians_gb300: GB300-native (sm_103a) density-field and clustering path of Pylians.

    import pylians_gb300.MAS_library as MASL
    import pylians_gb300.Pk_library as PKL

MASL.MA, PKL.Pk / XPk / Bk keep the reference's signatures and result
attributes; the arithmetic runs in libpylgpu.so (include/pylians_gb300.h)
through ctypes.  There is no CPU fallback.
"""
from . import _lib  # noqa: F401

__version__ = '0.1.0'

