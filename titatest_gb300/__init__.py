"""GB300-native (sm_103a) forward + sensitivity hot path of CRMod/CRTomo.

    from titatest_gb300 import formats, CRMod
    m = CRMod(grid, survey)               # precal on the device
    out = m.forward(sigma)                # kompab/scalab/chol/vre/rtrafo/bvolt
    J = m.bsens()                         # bsens

See include/crtomo_gb300.h for the C ABI that a Fortran host binds.  The
ctypes binding (and with it libcrtomo_gb300.so) is imported on first use of
one of the names below, so that the file-format classes (formats) can be used
without loading the library.
"""
from . import formats

__all__ = ["formats", "CRMod", "PLAIN", "MIXED", "cutmck", "rwaven", "run_tomodir"]

_FROM_CRMOD = ("CRMod", "PLAIN", "MIXED", "cutmck", "rwaven", "run_tomodir")


def __getattr__(name):
    if name in _FROM_CRMOD:
        from . import crmod
        return getattr(crmod, name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
