"""ctypes binding of libcrtomo_gb300 (include/crtomo_gb300.h).

The library is built in-tree by titatest_gb300.build (or
__graft_entry__.build()).  Loading fails loudly when it is missing: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcrtomo_gb300.so")

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)
vp = C.c_void_p

_lock = threading.Lock()
_lib = None

# every exported entry point of include/crtomo_gb300.h
EXPORTS = (
    "crgpu_create", "crgpu_destroy", "crgpu_last_error", "crgpu_set_refinement", "crgpu_set_stream",
    "crgpu_set_memory_budget", "crgpu_forward", "crgpu_forward_device", "crgpu_sens",
    "crgpu_sens_device", "crgpu_device_buffers", "crgpu_factor_system", "crgpu_update",
    "crgpu_rwaven", "crgpu_cutmck", "crgpu_bkfak", "crgpu_get_stats", "crgpu_factor_system_noalloc",
    "crgpu_adjoint", "crgpu_adjoint_device", "crgpu_autotune", "crgpu_get_tune", "crgpu_set_tune", "crgpu_forward_sens_graph",
    "crgpu_set_boundary_values", "crgpu_update_fpi", "crgpu_blam0_jtj", "crgpu_set_dc", "crgpu_update_dc",
    "crgpu_mcm", "crgpu_column_sums", "crgpu_device_memory", "crgpu_create2", "crgpu_node_order",
    "crgpu_forward_sens_batch", "crgpu_memory_need",
)


class CGrid(C.Structure):
    _fields_ = [("sanz", C.c_int32), ("typanz", C.c_int32), ("mb", C.c_int32),
                ("typ", i32p), ("nelanz", i32p), ("selanz", i32p), ("snr", i32p),
                ("sx", f64p), ("sy", f64p), ("nrel", i32p), ("ld_nrel", C.c_int32),
                ("rnr", i32p)]


class CSurvey(C.Structure):
    _fields_ = [("eanz", C.c_int32), ("enr", i32p), ("nanz", C.c_int32), ("strnr", i32p),
                ("vnr", i32p), ("strom", f64p), ("kwnanz", C.c_int32), ("kwn", f64p),
                ("kwnwi", f64p), ("swrtr", C.c_int32), ("lsr", C.c_int32), ("lsink", C.c_int32),
                ("nsink", C.c_int32), ("lsytop", C.c_int32)]


class CStats(C.Structure):
    _fields_ = [("kernel_launches", C.c_int64), ("ms_forward", C.c_double),
                ("ms_factor", C.c_double), ("ms_solve", C.c_double), ("ms_sens", C.c_double),
                ("ms_update", C.c_double), ("refine_iterations", C.c_int32),
                ("nsystems", C.c_int32), ("nbatches", C.c_int32),
                ("refine_last_correction", C.c_double), ("ms_adjoint", C.c_double)]


def lib() -> C.CDLL:
    """Load libcrtomo_gb300.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -m titatest_gb300.build` "
                    "(there is no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            L.crgpu_last_error.restype = C.c_char_p
            L.crgpu_last_error.argtypes = [vp]
            for name in EXPORTS:
                if name != "crgpu_last_error":
                    getattr(L, name).restype = C.c_int
            _lib = L
    return _lib


def device_memory():
    """(free, total) bytes of the current device (crgpu_device_memory)."""
    fr, tot = C.c_int64(0), C.c_int64(0)
    code = lib().crgpu_device_memory(C.byref(fr), C.byref(tot))
    if code:
        raise CRGPUError(code, "crgpu_device_memory")
    return fr.value, tot.value


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class CRGPUError(RuntimeError):
    def __init__(self, errnr: int, text: str):
        super().__init__(f"errnr {errnr}: {text}")
        self.errnr = errnr
        self.text = text


def make_cgrid(grid):
    """crgpu_grid view of a formats.Grid (keeps the arrays alive)."""
    keep = dict(
        typ=np.ascontiguousarray(grid.typ, np.int32),
        nelanz=np.ascontiguousarray(grid.nelanz, np.int32),
        selanz=np.ascontiguousarray(grid.selanz, np.int32),
        snr=np.ascontiguousarray(grid.snr, np.int32),
        sx=np.ascontiguousarray(grid.sx, np.float64),
        sy=np.ascontiguousarray(grid.sy, np.float64),
        nrel=grid.nrel_colmajor(),
        rnr=np.ascontiguousarray(grid.rnr if len(grid.rnr) else np.zeros(1, np.int32), np.int32),
    )
    cg = CGrid(grid.sanz, grid.typanz, grid.mb, ptr(keep["typ"], i32p), ptr(keep["nelanz"], i32p),
               ptr(keep["selanz"], i32p), ptr(keep["snr"], i32p), ptr(keep["sx"], f64p),
               ptr(keep["sy"], f64p), ptr(keep["nrel"], i32p), grid.nrel.shape[0],
               ptr(keep["rnr"], i32p))
    return cg, keep
