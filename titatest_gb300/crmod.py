"""Host-side mirror of the reference's forward-modelling interface.

``CRMod`` follows the control flow of the CRMod driver (src/fem.f90): read the
inputs, pick the wavenumbers (src/rwaven.f90), then the forward block,
back-transform, voltages (src/bvolt.f90) and optionally the sensitivities
(src/bsens.f90) -- every numerical step running in libcrtomo_gb300 on the GPU.
The routine names of the reference are kept as method names where a method
stands for one routine (rwaven, bkfak, bsens, bsensi, cutmck).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import formats
from ._lib import (CGrid, CRGPUError, CStats, CSurvey, f32p, f64p, i32p, lib, make_cgrid, ptr)

PLAIN = 0
MIXED = 1


def _check(ctx, code):
    if code != 0:
        text = lib().crgpu_last_error(ctx).decode() if ctx else ""
        raise CRGPUError(code, text)


def rwaven(grid: formats.Grid, survey: formats.Survey):
    """Wavenumbers and weights of src/rwaven.f90 (computed by the library)."""
    cg, keep = make_cgrid(grid)
    enr = np.ascontiguousarray(survey.enr, np.int32)
    s = np.ascontiguousarray(survey.strnr, np.int32)
    v = np.ascontiguousarray(survey.vnr, np.int32)
    kwn = np.zeros(32)
    kwnwi = np.zeros(32)
    n = C.c_int32(0)
    code = lib().crgpu_rwaven(C.byref(cg), survey.eanz, ptr(enr, i32p), survey.nanz, ptr(s, i32p),
                              ptr(v, i32p), ptr(kwn, f64p), ptr(kwnwi, f64p), C.byref(n))
    if code:
        raise CRGPUError(code, "rwaven")
    return kwn[: n.value].copy(), kwnwi[: n.value].copy()


def cutmck(grid: formats.Grid, enr: np.ndarray):
    """Cuthill-McKee renumbering of cutmckee/cutmck.f: (new grid, new enr)."""
    g = grid.copy()
    nrel = g.nrel_colmajor()
    snr = np.ascontiguousarray(g.snr, np.int32).copy()
    en = np.ascontiguousarray(enr, np.int32).copy()
    mb = C.c_int32(0)
    code = lib().crgpu_cutmck(g.sanz, g.typanz, ptr(np.ascontiguousarray(g.typ, np.int32), i32p),
                              ptr(np.ascontiguousarray(g.nelanz, np.int32), i32p),
                              ptr(np.ascontiguousarray(g.selanz, np.int32), i32p), ptr(nrel, i32p),
                              g.nrel.shape[0], ptr(snr, i32p), len(en), ptr(en, i32p), C.byref(mb))
    if code:
        raise CRGPUError(code, "cutmck")
    g.nrel = np.ascontiguousarray(nrel.T)
    g.snr = snr
    g.mb = mb.value
    return g, en


class CRMod:
    """One grid + survey on the GPU; forward and sensitivities for any sigma.

    precision: PLAIN (complex128, the reference arithmetic) or MIXED (complex64
    factorisation with FP64 iterative refinement).
    band_order: 1 (default) lets a MIXED context factor in the geometric node
    order when that band is narrower (crgpu_create2); 2 lets any context
    factor in that order whenever its band is narrower; 0 keeps the grid's
    band.
    """

    def __init__(self, grid: formats.Grid, survey: formats.Survey, kwn=None, kwnwi=None,
                 swrtr: int = 1, lsink: bool = False, nsink: int = 0, lsytop: bool = False,
                 precision: int = PLAIN, lsr: bool = False, band_order: int = 1):
        self.grid = grid
        self.survey = survey
        if kwn is None:
            if swrtr:
                kwn, kwnwi = rwaven(grid, survey)
            else:
                kwn, kwnwi = np.zeros(1), np.zeros(1)
        self.kwn = np.ascontiguousarray(kwn, np.float64)
        self.kwnwi = np.ascontiguousarray(kwnwi, np.float64)
        self.swrtr = swrtr
        self.precision = precision
        self._cg, self._keep = make_cgrid(grid)
        self._keep.update(
            enr=np.ascontiguousarray(survey.enr, np.int32),
            strnr=np.ascontiguousarray(survey.strnr, np.int32),
            vnr=np.ascontiguousarray(survey.vnr, np.int32),
            strom=np.ascontiguousarray(survey.strom, np.float64))
        k = self._keep
        self._cs = CSurvey(survey.eanz, ptr(k["enr"], i32p), survey.nanz, ptr(k["strnr"], i32p),
                           ptr(k["vnr"], i32p), ptr(k["strom"], f64p), len(self.kwn),
                           ptr(self.kwn, f64p), ptr(self.kwnwi, f64p), int(swrtr), int(lsr),
                           int(lsink), int(nsink), int(lsytop))
        h = C.c_void_p()
        code = lib().crgpu_create2(C.byref(self._cg), C.byref(self._cs), int(precision), int(band_order),
                                   C.byref(h))
        self._h = h
        if code:
            msg = lib().crgpu_last_error(h).decode() if h.value else ""
            if h.value:
                lib().crgpu_destroy(h)
            self._h = C.c_void_p()
            raise CRGPUError(code, msg)

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if self._h and self._h.value:
            lib().crgpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- options ----------------------------------------------------------
    def set_refinement(self, maxit: int, tol: float):
        _check(self._h, lib().crgpu_set_refinement(self._h, int(maxit), C.c_double(tol)))

    def set_boundary_values(self, nodes, values):
        """Dirichlet boundary values (src/randb2.f90): nodes 1-based in the band
        numbering, complex values, in the order of the boundary-value file
        (formats.read_boundary_values).  None or an empty list removes them."""
        if nodes is None or len(nodes) == 0:
            _check(self._h, lib().crgpu_set_boundary_values(self._h, 0, None, None))
            return
        nr = np.ascontiguousarray(nodes, np.int32)
        vv = np.ascontiguousarray(values, np.complex128)
        if nr.shape != vv.shape:
            raise ValueError("nodes and values differ in length")
        _check(self._h, lib().crgpu_set_boundary_values(self._h, len(nr), ptr(nr, i32p), ptr(vv, f64p)))

    def set_dc(self, ldc: bool = True):
        """DC mode (crgpu_set_dc): the real routines of CRTomo's ldc."""
        _check(self._h, lib().crgpu_set_dc(self._h, int(bool(ldc))))

    def set_stream(self, stream_handle: int):
        """Issue the work on a caller-owned cudaStream_t (e.g.
        torch.cuda.current_stream().cuda_stream); 0 restores the own stream."""
        _check(self._h, lib().crgpu_set_stream(self._h, C.c_void_p(stream_handle or None)))

    def set_memory_budget(self, nbytes: int):
        _check(self._h, lib().crgpu_set_memory_budget(self._h, C.c_int64(int(nbytes))))

    @property
    def kwnanz(self) -> int:
        return len(self.kwn)

    # -- forward ----------------------------------------------------------
    def forward(self, sigma, kpot: bool = False, hpot: bool = False, volt_mode: int = 0,
                kfak: Optional[np.ndarray] = None):
        """Forward block + rtrafo + bvolt/bvolti.  Returns a dict with
        'volt', 'sigmaa' (nanz complex) and optionally 'kpot'
        (kwnanz, eanz, sanz) and 'hpot' (eanz, sanz)."""
        g, sv = self.grid, self.survey
        sig = np.ascontiguousarray(sigma, np.complex128)
        out = {"volt": np.zeros(sv.nanz, np.complex128), "sigmaa": np.zeros(sv.nanz, np.complex128)}
        kp = np.zeros((self.kwnanz, sv.eanz, g.sanz), np.complex128) if kpot else None
        hp = np.zeros((sv.eanz, g.sanz), np.complex128) if hpot else None
        kf = None if kfak is None else np.ascontiguousarray(kfak, np.float64)
        code = lib().crgpu_forward(self._h, ptr(sig, f64p), None if kp is None else ptr(kp, f64p),
                                   None if hp is None else ptr(hp, f64p), int(volt_mode),
                                   None if kf is None else ptr(kf, f64p), ptr(out["volt"], f64p),
                                   ptr(out["sigmaa"], f64p))
        _check(self._h, code)
        if kp is not None:
            out["kpot"] = kp
        if hp is not None:
            out["hpot"] = hp
        return out

    def forward_device(self, sigma_ptr: int, volt_ptr: int, sigmaa_ptr: int = 0, volt_mode: int = 0,
                       kfak_ptr: int = 0):
        """Forward with device pointers (e.g. torch tensor data_ptr())."""
        code = lib().crgpu_forward_device(self._h, C.c_void_p(sigma_ptr), int(volt_mode),
                                          C.c_void_p(kfak_ptr or None), C.c_void_p(volt_ptr or None),
                                          C.c_void_p(sigmaa_ptr or None))
        _check(self._h, code)

    # -- sensitivities ----------------------------------------------------
    def sens(self, mode: int = 0) -> np.ndarray:
        """src/bsens.f90 (mode 0) / src/bsensi.f90 (mode 1) of the last
        forward: array (nanz, elanz) complex128."""
        sv, g = self.survey, self.grid
        buf = np.zeros((g.elanz, sv.nanz), np.complex128)  # column-major (nanz, manz)
        _check(self._h, lib().crgpu_sens(self._h, int(mode), ptr(buf, f64p)))
        return buf.T

    def blam0_jtj(self, wmatd, wdfak, phase_only: bool = False) -> np.ndarray:
        """|(J^H W J 1)_j| of src/blam0.f90 on the device sensitivities."""
        out = np.zeros(self.grid.elanz)
        _check(self._h, lib().crgpu_blam0_jtj(self._h, ptr(np.ascontiguousarray(wmatd, np.float64), f64p),
                                              ptr(np.ascontiguousarray(wdfak, np.int32), i32p),
                                              int(bool(phase_only)), ptr(out, f64p)))
        return out

    def mcm(self, wmatd, wdfak, ltri, smatm, nx=0, nachbar=None, lam=1.0, res=True, cov2=True) -> dict:
        """crgpu_mcm: the diagonals of src/bmcm_mod.f90 (ata, ata_reg, cov and,
        if asked, cov ata and cov ata cov) on the device sensitivities."""
        manz = self.grid.elanz
        out = {k: np.zeros(manz) for k in ("ata", "reg", "cov1", "res", "cov2")}
        nb = np.ascontiguousarray(nachbar if nachbar is not None else np.zeros(1), np.int32)
        flags = (1 if res else 0) | (2 if (res and cov2) else 0)
        _check(self._h, lib().crgpu_mcm(
            self._h, ptr(np.ascontiguousarray(wmatd, np.float64), f64p),
            ptr(np.ascontiguousarray(wdfak, np.int32), i32p), int(ltri),
            ptr(np.ascontiguousarray(smatm, np.float64), f64p), int(nx), ptr(nb, i32p), C.c_double(lam),
            int(flags), ptr(out["ata"], f64p), ptr(out["reg"], f64p), ptr(out["cov1"], f64p),
            ptr(out["res"], f64p), ptr(out["cov2"], f64p)))
        if not res:
            del out["res"]
        if not (res and cov2):
            del out["cov2"]
        return out

    def column_sums(self, wa, wb, wc):
        """crgpu_column_sums: sum_i |J_ij| wa_i, sum_i |Re J_ij| wb_i,
        sum_i Re(J_ij)^2 wc_i on the device sensitivities."""
        manz = self.grid.elanz
        c = [np.zeros(manz) for _ in range(3)]
        ws = [np.ascontiguousarray(w, np.float64) for w in (wa, wb, wc)]
        _check(self._h, lib().crgpu_column_sums(self._h, *(ptr(w, f64p) for w in ws), *(ptr(x, f64p) for x in c)))
        return tuple(c)

    def sens_on_device(self, mode: int = 1):
        """The sensitivities of the last forward into the context's device
        array only (for update), with no host copy."""
        _check(self._h, lib().crgpu_sens(self._h, int(mode), None))

    def bsens(self) -> np.ndarray:
        return self.sens(0)

    def bsensi(self) -> np.ndarray:
        return self.sens(1)

    def adjoint(self, g) -> np.ndarray:
        """Exact dL/dsigma (elanz complex128) of L = sum_i g_i V_i, V the
        voltages of the last forward, by adjoint solves that reuse the
        forward's band factors (crgpu_adjoint)."""
        gg = np.ascontiguousarray(g, np.complex128)
        if gg.shape != (self.survey.nanz,):
            raise ValueError(f"g must have shape ({self.survey.nanz},)")
        out = np.zeros(self.grid.elanz, np.complex128)
        _check(self._h, lib().crgpu_adjoint(self._h, ptr(gg, f64p), ptr(out, f64p)))
        return out

    def adjoint_device(self, g_ptr: int, grad_ptr: int):
        """crgpu_adjoint_device on device pointers (nanz and elanz complex128)."""
        _check(self._h, lib().crgpu_adjoint_device(self._h, C.c_void_p(g_ptr), C.c_void_p(grad_ptr)))

    def sens_device(self, mode: int, sens_ptr: int):
        _check(self._h, lib().crgpu_sens_device(self._h, int(mode), C.c_void_p(sens_ptr)))

    def memory_need(self) -> int:
        """crgpu_memory_need: device bytes a forward + Jacobian still allocates."""
        b = C.c_int64(0)
        _check(self._h, lib().crgpu_memory_need(self._h, C.byref(b)))
        return b.value

    def node_order(self) -> np.ndarray:
        """crgpu_node_order: the grid node (1-based) in each position of the
        context's device arrays."""
        out = np.zeros(self.grid.sanz, np.int32)
        _check(self._h, lib().crgpu_node_order(self._h, ptr(out, i32p)))
        return out

    def device_buffers(self):
        kp = C.c_void_p()
        hp = C.c_void_p()
        _check(self._h, lib().crgpu_device_buffers(self._h, C.byref(kp), C.byref(hp)))
        return kp.value, hp.value

    def factor_system(self, sigma, k: int, l: int):
        """Band factor a((mb+1)*sanz) and fak of system (k, l), 1-based."""
        g = self.grid
        sig = np.ascontiguousarray(sigma, np.complex128)
        a = np.zeros((g.sanz, g.mb + 1), np.complex128)
        fak = np.zeros(g.sanz)
        _check(self._h, lib().crgpu_factor_system(self._h, ptr(sig, f64p), int(k), int(l),
                                                  ptr(a, f64p), ptr(fak, f64p)))
        return a, fak

    def bkfak(self) -> np.ndarray:
        kf = np.zeros(self.survey.nanz)
        code = lib().crgpu_bkfak(C.byref(self._cg), C.byref(self._cs), ptr(kf, f64p))
        if code:
            raise CRGPUError(code, "bkfak")
        return kf

    def forward_sens_graph(self, sigma_ptr: int, volt_ptr: int, mode: int, sens_ptr: int):
        """crgpu_forward_sens_graph: forward + Jacobian of device buffers,
        replayed as one CUDA graph after the first call."""
        _check(self._h, lib().crgpu_forward_sens_graph(self._h, C.c_void_p(sigma_ptr), C.c_void_p(volt_ptr),
                                                        int(mode), C.c_void_p(sens_ptr)))

    def autotune(self, sigma, force: bool = False) -> dict:
        """crgpu_autotune: the fastest factor and Jacobian kernels for this
        problem (mixed precision), timed on its own systems; returns the
        choices of tune()."""
        sig = np.ascontiguousarray(sigma, np.complex128)
        _check(self._h, lib().crgpu_autotune(self._h, sig.ctypes.data_as(f64p), int(bool(force))))
        return self.tune()

    def tune(self) -> dict:
        out = np.zeros(3, np.int32)
        _check(self._h, lib().crgpu_get_tune(self._h, out.ctypes.data_as(i32p)))
        names = {0: "default", 1: "tensor cores", 2: "SIMT register tiles", 3: "SIMT shared-memory tiles",
                 4: "SIMT warp per system"}
        return {"factor": names[int(out[0])], "factor_blocks_per_sm": int(out[1]),
                "jacobian": {0: "default", 1: "tensor cores", 2: "SIMT"}[int(out[2])]}

    def set_tune(self, factor: int = 0, blocks_per_sm: int = 0, jacobian: int = 0):
        """crgpu_set_tune: factor 0 default, 1 tensor cores, 2 SIMT register
        tiles, 3 SIMT shared-memory tiles, 4 one warp per system (mb <= 63);
        jacobian 0 default, 1 tensor cores, 2 SIMT."""
        a = np.array([factor, blocks_per_sm, jacobian], np.int32)
        _check(self._h, lib().crgpu_set_tune(self._h, a.ctypes.data_as(i32p)))

    def stats(self) -> dict:
        s = CStats()
        _check(self._h, lib().crgpu_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in CStats._fields_}

    # -- inversion update ---------------------------------------------------
    def update(self, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx=0, nachbar=None, lam=1.0, eps=1e-4,
               ncgmax=100, step=1.0, par=None, phase_only: bool = False, dc: bool = False):
        """src/update.f90 + cjggra on the sensitivities of the last sens(1);
        phase_only: the final phase improvement (crgpu_update_fpi, cjggdc);
        dc: DC inversion (crgpu_update_dc, cjggdc)."""
        sv, g = self.survey, self.grid
        manz = g.elanz
        par = np.zeros(manz, np.complex128) if par is None else np.array(par, np.complex128)
        dpar = np.zeros(manz, np.complex128)
        cgfac = np.zeros(manz)
        cgres = np.zeros(ncgmax + 2, np.float32)
        ncg = C.c_int32(0)
        nb = np.ascontiguousarray(nachbar if nachbar is not None else np.zeros(1), np.int32)
        fn = lib().crgpu_update_fpi if phase_only else lib().crgpu_update_dc if dc else lib().crgpu_update
        code = fn(
            self._h, ptr(np.ascontiguousarray(wmatd, np.float64), f64p),
            ptr(np.ascontiguousarray(wdfak, np.int32), i32p),
            ptr(np.ascontiguousarray(dat, np.complex128), f64p),
            ptr(np.ascontiguousarray(sigmaa, np.complex128), f64p), int(ltri),
            ptr(np.ascontiguousarray(smatm, np.float64), f64p), int(nx), ptr(nb, i32p),
            C.c_double(lam), C.c_double(eps), int(ncgmax), C.c_double(step), ptr(par, f64p),
            ptr(dpar, f64p), ptr(cgfac, f64p), ptr(cgres, f32p), C.byref(ncg))
        _check(self._h, code)
        return par, dpar, cgfac, cgres, ncg.value


def run_tomodir(exe_dir: str, precision: int = PLAIN, write: bool = True):
    """CRMod on a tomodir: reads exe_dir/crmod.cfg and its inputs, runs the
    forward (and the sensitivities if requested) and writes volt.dat."""
    import os
    td = formats.load_crmod(exe_dir)
    cfg = td.cfg
    m = CRMod(td.grid, td.survey, swrtr=cfg.swrtr, lsink=cfg.lsink, nsink=cfg.nsink,
              precision=precision, lsr=cfg.lsr)
    try:
        if td.boundary_values is not None:
            m.set_boundary_values(*td.boundary_values)
        kfak = m.bkfak() if (cfg.wkfak and td.grid.relanz and 11 in set(td.grid.typ.tolist())) else None
        out = m.forward(td.sigma, kfak=kfak, hpot=bool(write and cfg.lpot))
        if write and cfg.lpot:  # src/fem.f90:409-412
            formats.write_potentials(os.path.normpath(os.path.join(exe_dir, cfg.dpot)), out["hpot"],
                                     td.survey.strnr, np.asarray(td.survey.strom), td.grid)
        if write and cfg.lvolt:
            formats.write_volt(os.path.normpath(os.path.join(exe_dir, cfg.dvolt)), td.survey.strnr,
                               td.survey.vnr, out["sigmaa"])
        if cfg.lsens:
            out["sens"] = m.bsens()
            if write:  # src/fem.f90:436-467
                from .regularization import _centroids
                cx, cy = _centroids(td.grid)
                formats.write_sensitivities(os.path.normpath(os.path.join(exe_dir, cfg.dsens)), out["sens"], cx, cy)
        return out
    finally:
        m.close()


def forward_sens_batch(models, sigmas, sens_mode: int = 0, volt_mode: int = 0):
    """crgpu_forward_sens_batch: the forward of every model (MIXED contexts
    whose bands fit the tensor-core window), their band factors in one
    persistent launch; the Jacobians (sens_mode 0 or 1; -1 none) stay on the
    devices of the contexts.  Returns the voltages, one array per model."""
    n = len(models)
    sig = [np.ascontiguousarray(s, np.complex128) for s in sigmas]
    volts = [np.zeros(m.survey.nanz, np.complex128) for m in models]
    ctxs = (C.c_void_p * n)(*[m._h.value for m in models])
    sp = (C.c_void_p * n)(*[s.ctypes.data for s in sig])
    vp = (C.c_void_p * n)(*[v.ctypes.data for v in volts])
    code = lib().crgpu_forward_sens_batch(ctxs, n, sp, int(volt_mode), vp, int(sens_mode))
    if code:
        bad = next((m for m in models if lib().crgpu_last_error(m._h)), models[0])
        raise CRGPUError(code, lib().crgpu_last_error(bad._h).decode())
    return volts

