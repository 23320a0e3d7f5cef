"""GB300-native (sm_103a) forward + sensitivity hot path of CRMod/CRTomo.

    from titatest_gb300 import formats, CRMod
    m = CRMod(grid, survey)               # precal on the device
    out = m.forward(sigma)                # kompab/scalab/chol/vre/rtrafo/bvolt
    J = m.bsens()                         # bsens

See include/crtomo_gb300.h for the C ABI that a Fortran host binds.
"""
from . import formats
from .crmod import MIXED, PLAIN, CRMod, cutmck, run_tomodir, rwaven

__all__ = ["formats", "CRMod", "PLAIN", "MIXED", "cutmck", "rwaven", "run_tomodir"]
