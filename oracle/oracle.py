"""ctypes front end of the CPU oracle (oracle/crt_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the titatest_gb300 package.  It builds
the oracle with oracle/Makefile on first use.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcrt_oracle.so")
# the same source built with the reference's optimisation flags
# (configure.ac:19-26: -O3 -ffast-math ..., less -march=native), for timing
# only: the parity checks use the strict build above
_LIB_TIMING_PATH = os.path.join(_HERE, "_build", "libcrt_oracle_timing.so")
_lock = threading.Lock()
_lib = None
_lib_timing = None

i32p = C.POINTER(C.c_int)
f64p = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "crt_oracle.c")
    stale = [p for p in (_LIB_PATH, _LIB_TIMING_PATH)
             if not os.path.exists(p) or os.path.getmtime(p) < os.path.getmtime(src)]
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class OrMesh(C.Structure):
    _fields_ = [
        ("sanz", C.c_int), ("typanz", C.c_int), ("mb", C.c_int),
        ("typ", i32p), ("nelanz", i32p), ("selanz", i32p),
        ("snr", i32p), ("sx", f64p), ("sy", f64p),
        ("nrel", i32p), ("ld_nrel", C.c_int), ("rnr", i32p),
        ("eanz", C.c_int), ("enr", i32p),
        ("nanz", C.c_int), ("strnr", i32p), ("vnr", i32p), ("strom", f64p),
    ]


class OrOpts(C.Structure):
    _fields_ = [("swrtr", C.c_int), ("lsr", C.c_int), ("lana", C.c_int), ("lsink", C.c_int),
                ("nsink", C.c_int), ("lsytop", C.c_int), ("nthreads", C.c_int),
                ("rwdanz", C.c_int), ("rwdnr", i32p), ("rwd", f64p), ("ldc", C.c_int)]


def _declare(L):
    L.or_rwaven.restype = C.c_int
    L.or_forward.restype = C.c_int
    L.or_forward_pairs.restype = C.c_int
    L.or_bvolt.restype = C.c_int
    L.or_bkfak.restype = C.c_int
    L.or_cutmck.restype = C.c_int
    L.or_elbg.restype = C.c_int
    L.or_precal_all.restype = C.c_int
    L.or_update.restype = C.c_int
    L.or_factor.restype = C.c_int
    L.or_bsytop.restype = C.c_double
    L.or_bessk0.restype = C.c_double
    L.or_bessk0.argtypes = [C.c_double]
    L.or_bessk1.restype = C.c_double
    L.or_bessk1.argtypes = [C.c_double]
    return L


def lib_timing():
    """The timing build (reference optimisation flags); not for parity."""
    global _lib_timing
    with _lock:
        if _lib_timing is None:
            build()
            _lib_timing = _declare(C.CDLL(_LIB_TIMING_PATH))
    return _lib_timing


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = _declare(C.CDLL(_LIB_PATH))
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


class Problem:
    """Holds the arrays of one grid + survey and the or_mesh view of them.
    timing=True runs the timing build (reference optimisation flags)."""

    def __init__(self, grid, survey, timing: bool = False):
        self._L = lib_timing() if timing else lib()
        self.grid = grid
        self.survey = survey
        self._keep = dict(
            typ=np.ascontiguousarray(grid.typ, np.int32),
            nelanz=np.ascontiguousarray(grid.nelanz, np.int32),
            selanz=np.ascontiguousarray(grid.selanz, np.int32),
            snr=np.ascontiguousarray(grid.snr, np.int32),
            sx=np.ascontiguousarray(grid.sx, np.float64),
            sy=np.ascontiguousarray(grid.sy, np.float64),
            nrel=grid.nrel_colmajor(),
            rnr=np.ascontiguousarray(grid.rnr if len(grid.rnr) else np.zeros(1, np.int32), np.int32),
            enr=np.ascontiguousarray(survey.enr, np.int32),
            strnr=np.ascontiguousarray(survey.strnr, np.int32),
            vnr=np.ascontiguousarray(survey.vnr, np.int32),
            strom=np.ascontiguousarray(survey.strom, np.float64),
        )
        self._rwd = None
        self._ldc = 0
        k = self._keep
        self.m = OrMesh(
            grid.sanz, grid.typanz, grid.mb, _p(k["typ"], i32p), _p(k["nelanz"], i32p),
            _p(k["selanz"], i32p), _p(k["snr"], i32p), _p(k["sx"], f64p), _p(k["sy"], f64p),
            _p(k["nrel"], i32p), grid.elanz + grid.relanz, _p(k["rnr"], i32p),
            survey.eanz, _p(k["enr"], i32p), survey.nanz, _p(k["strnr"], i32p),
            _p(k["vnr"], i32p), _p(k["strom"], f64p))

    # --- wavenumbers -------------------------------------------------------
    def rwaven(self):
        kwn = np.zeros(32)
        kwnwi = np.zeros(32)
        n = self._L.or_rwaven(C.byref(self.m), _p(kwn, f64p), _p(kwnwi, f64p))
        if n < 0:
            raise RuntimeError(f"rwaven errnr {-n}")
        return kwn[:n].copy(), kwnwi[:n].copy()

    def refsig(self, sigma):
        sigma = np.ascontiguousarray(sigma, np.complex128)
        out = np.zeros(2)
        self._L.or_refsig(C.byref(self.m), _p(sigma, f64p), _p(out, f64p))
        return complex(out[0], out[1])

    def precal(self, kwn, sytop=0.0):
        g = self.grid
        kwn = np.ascontiguousarray(kwn, np.float64)
        K = len(kwn)
        elbg = np.zeros(g.elanz * 10 * K)
        relbg = np.zeros(max(g.relanz, 1) * 10)
        kg = np.zeros(max(g.relanz, 1) * self.survey.eanz * K)
        flags = np.zeros(2, np.int32)
        e = self._L.or_precal_all(C.byref(self.m), K, _p(kwn, f64p), C.c_double(sytop),
                                _p(elbg, f64p), _p(relbg, f64p), _p(kg, f64p), _p(flags, i32p))
        if e:
            raise RuntimeError(f"precal errnr {e}")
        # Fortran layouts: elbg(elanz,10,K), relbg(relanz,10), kg(relanz,eanz,K)
        return (elbg.reshape(K, 10, g.elanz), relbg.reshape(10, max(g.relanz, 1)),
                kg.reshape(K, self.survey.eanz, max(g.relanz, 1)), bool(flags[0]), bool(flags[1]))

    def set_boundary_values(self, nodes, values):
        """Dirichlet boundary values of src/randb2.f90 (lrandb2): node numbers
        (1-based, band numbering) and complex values, in file order; None or an
        empty list switches them off."""
        if nodes is None or len(nodes) == 0:
            self._rwd = None
            return
        nr = np.ascontiguousarray(nodes, np.int32)
        vv = np.ascontiguousarray(values, np.complex128)
        assert nr.shape == vv.shape
        self._rwd = (nr, vv)

    def set_dc(self, ldc=True):
        """DC twins (CRTomo ldc): Re(sigma) in the assembly, the pivot test of
        src/choldc.f90; bvolt(..., mode=2) and update(..., dc=True) go with it."""
        self._ldc = int(bool(ldc))

    def _opts(self, *args):
        o = OrOpts(*args)
        o.ldc = self._ldc
        if self._rwd is not None:
            nr, vv = self._rwd
            o.rwdanz = len(nr)
            o.rwdnr = _p(nr, i32p)
            o.rwd = _p(vv, f64p)
        return o

    # --- forward -----------------------------------------------------------
    def forward(self, sigma, kwn, kwnwi, swrtr=1, lsr=False, lana=False, lsink=False, nsink=0,
                lsytop=False, nthreads=0):
        """kpot as array (kwnanz, eanz, sanz) complex128 (Fortran kpot(j,l,k))."""
        g = self.grid
        sigma = np.ascontiguousarray(sigma, np.complex128)
        kwn = np.ascontiguousarray(kwn, np.float64)
        kwnwi = np.ascontiguousarray(kwnwi, np.float64)
        K = len(kwn)
        kpot = np.zeros((K, self.survey.eanz, g.sanz), np.complex128)
        o = self._opts(swrtr, int(lsr), int(lana), int(lsink), int(nsink), int(lsytop), int(nthreads))
        e = self._L.or_forward(C.byref(self.m), C.byref(o), K, _p(kwn, f64p), _p(kwnwi, f64p),
                             _p(sigma, f64p), _p(kpot, f64p))
        if e:
            raise RuntimeError(f"forward errnr {e}")
        return kpot

    def forward_pairs(self, sigma, kwn, kwnwi, pairs, nthreads=0, **kw):
        """Solve only the (k, l) pairs (0-based) given; returns kpot array."""
        g = self.grid
        sigma = np.ascontiguousarray(sigma, np.complex128)
        kwn = np.ascontiguousarray(kwn, np.float64)
        kwnwi = np.ascontiguousarray(kwnwi, np.float64)
        K = len(kwn)
        kpot = np.zeros((K, self.survey.eanz, g.sanz), np.complex128)
        pr = np.ascontiguousarray(np.asarray(pairs, np.int32) + 1)
        o = self._opts(kw.get("swrtr", 1), int(kw.get("lsr", 0)), int(kw.get("lana", 0)),
                   int(kw.get("lsink", 0)), int(kw.get("nsink", 0)), int(kw.get("lsytop", 0)),
                   int(nthreads))
        e = self._L.or_forward_pairs(C.byref(self.m), C.byref(o), K, _p(kwn, f64p), _p(kwnwi, f64p),
                                   _p(sigma, f64p), len(pr), _p(pr, i32p), _p(kpot, f64p))
        if e:
            raise RuntimeError(f"forward errnr {e}")
        return kpot

    def factor(self, sigma, kwn, k, l, **kw):
        """Band factor a (sanz, mb+1) and fak of system (k, l), 1-based."""
        g = self.grid
        sigma = np.ascontiguousarray(sigma, np.complex128)
        kwn = np.ascontiguousarray(kwn, np.float64)
        a = np.zeros((g.sanz, g.mb + 1), np.complex128)
        fak = np.zeros(g.sanz)
        o = self._opts(kw.get("swrtr", 1), 0, 0, int(kw.get("lsink", 0)), int(kw.get("nsink", 0)),
                   int(kw.get("lsytop", 0)), 0)
        e = self._L.or_factor(C.byref(self.m), C.byref(o), len(kwn), _p(kwn, f64p), _p(sigma, f64p),
                            int(k), int(l), _p(a, f64p), _p(fak, f64p))
        if e:
            raise RuntimeError(f"factor errnr {e}")
        return a, fak

    def rtrafo(self, kpot, kwnwi, swrtr=1):
        g = self.grid
        kpot = np.ascontiguousarray(kpot, np.complex128)
        kwnwi = np.ascontiguousarray(kwnwi, np.float64)
        hpot = np.zeros((self.survey.eanz, g.sanz), np.complex128)
        self._L.or_rtrafo(C.byref(self.m), swrtr, len(kwnwi), _p(kwnwi, f64p), _p(kpot, f64p),
                        _p(hpot, f64p))
        return hpot

    def bkfak(self):
        kfak = np.zeros(self.survey.nanz)
        e = self._L.or_bkfak(C.byref(self.m), _p(kfak, f64p))
        if e:
            raise RuntimeError(f"bkfak errnr {e}")
        return kfak

    def bvolt(self, hpot, mode=0, kfak=None):
        hpot = np.ascontiguousarray(hpot, np.complex128)
        volt = np.zeros(self.survey.nanz, np.complex128)
        sigmaa = np.zeros(self.survey.nanz, np.complex128)
        kf = None if kfak is None else np.ascontiguousarray(kfak, np.float64)
        e = self._L.or_bvolt(C.byref(self.m), mode, _p(hpot, f64p),
                           None if kf is None else _p(kf, f64p), _p(volt, f64p), _p(sigmaa, f64p))
        if e:
            raise RuntimeError(f"bvolt errnr {e}")
        return volt, sigmaa

    def bsens(self, kpot, kwn, kwnwi, sigma, volt=None, mode=0, swrtr=1, nthreads=0, sytop=0.0,
              contiguous=True):
        """sens as array (nanz, elanz) complex128 (C order; Fortran sens(i, m));
        contiguous=False returns the transposed view of the column-major
        result instead of a C-ordered copy."""
        g = self.grid
        kwn = np.ascontiguousarray(kwn, np.float64)
        kwnwi = np.ascontiguousarray(kwnwi, np.float64)
        K = len(kwn)
        elbg = np.zeros(g.elanz * 10 * K)
        e = self._L.or_elbg(C.byref(self.m), K, _p(kwn, f64p), C.c_double(sytop), _p(elbg, f64p))
        if e:
            raise RuntimeError(f"precal errnr {e}")
        kpot = np.ascontiguousarray(kpot, np.complex128)
        sigma = np.ascontiguousarray(sigma, np.complex128)
        volt = np.ascontiguousarray(volt if volt is not None else np.ones(self.survey.nanz),
                                    np.complex128)
        sens = np.zeros((g.elanz, self.survey.nanz), np.complex128)  # column-major (nanz, manz)
        o = self._opts(swrtr, 0, 0, 0, 0, 0, int(nthreads))
        self._L.or_bsens_elbg(C.byref(self.m), C.byref(o), mode, swrtr, K, _p(kwnwi, f64p),
                            _p(elbg, f64p), _p(kpot, f64p), _p(sigma, f64p), _p(volt, f64p),
                            _p(sens, f64p))
        return np.ascontiguousarray(sens.T) if contiguous else sens.T

    def potana(self, l, kw, sigma0):
        pota = np.zeros(self.grid.sanz, np.complex128)
        s0 = np.array([sigma0.real, sigma0.imag])
        self._L.or_potana(C.byref(self.m), int(l), C.c_double(kw), _p(s0, f64p), _p(pota, f64p))
        return pota

    def bnachbar(self):
        g = self.grid
        nb = np.zeros((g.maxnk + 1, g.elanz), np.int32)
        self._L.or_bnachbar(C.byref(self.m), _p(nb, i32p))
        return nb  # [col][elem] == Fortran nachbar(elem, col)

    def bsmatmreg(self, nx, nz, alfx=1.0, alfz=1.0):
        sm = np.zeros((3, nx * nz))
        self._L.or_bsmatmreg(C.byref(self.m), nx, nz, C.c_double(alfx), C.c_double(alfz),
                           _p(sm, f64p))
        return sm

    def bsmatmtri(self, nachbar, alfx=1.0, alfz=1.0):
        g = self.grid
        sm = np.zeros((g.maxnk + 1, g.elanz))
        nb = np.ascontiguousarray(nachbar, np.int32)
        self._L.or_bsmatmtri(C.byref(self.m), _p(nb, i32p), C.c_double(alfx), C.c_double(alfz),
                           _p(sm, f64p))
        return sm


def cutmck(grid, enr):
    """cutmckee/cutmck.f: returns (new_grid, new_enr)."""
    g = grid.copy()
    nrel = g.nrel_colmajor()
    snr = np.ascontiguousarray(g.snr, np.int32)
    en = np.ascontiguousarray(enr, np.int32).copy()
    typ = np.ascontiguousarray(g.typ, np.int32)
    nel = np.ascontiguousarray(g.nelanz, np.int32)
    sel = np.ascontiguousarray(g.selanz, np.int32)
    mb = lib().or_cutmck(g.sanz, g.typanz, _p(typ, i32p), _p(nel, i32p), _p(sel, i32p),
                         _p(nrel, i32p), g.nrel.shape[0], _p(snr, i32p), len(en), _p(en, i32p))
    if mb < 0:
        raise RuntimeError(f"cutmck errnr {-mb}")
    g.nrel = np.ascontiguousarray(nrel.T)
    g.snr = snr
    g.mb = mb
    return g, en


def update(sens, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx=0, nachbar=None, maxnk=4, lam=1.0,
           eps=1e-4, ncgmax=100, step=1.0, par=None, phase_only=False, dc=False):
    """src/update.f90 + cjggra (phase_only: the final phase improvement with
    cjggdc); sens (nanz, manz) complex.  Returns (par_new, dpar, cgfac,
    cgres, ncg)."""
    nanz, manz = sens.shape
    s = np.ascontiguousarray(np.asarray(sens, np.complex128).T)  # column-major
    par = np.zeros(manz, np.complex128) if par is None else np.array(par, np.complex128)
    dpar = np.zeros(manz, np.complex128)
    cgfac = np.zeros(manz)
    cgres = np.zeros(ncgmax + 2, np.float32)
    wm = np.ascontiguousarray(wmatd, np.float64)
    wd = np.ascontiguousarray(wdfak, np.int32)
    d = np.ascontiguousarray(dat, np.complex128)
    sa = np.ascontiguousarray(sigmaa, np.complex128)
    sm = np.ascontiguousarray(smatm, np.float64)
    nb = np.ascontiguousarray(nachbar if nachbar is not None else np.zeros(1), np.int32)
    fn = lib().or_update_fpi if phase_only else lib().or_update_dc if dc else lib().or_update
    ncg = fn(nanz, manz, _p(s, f64p), _p(wm, f64p), _p(wd, i32p), _p(d, f64p),
                          _p(sa, f64p), ltri, _p(sm, f64p), nx, _p(nb, i32p), maxnk,
                          C.c_double(lam), C.c_double(eps), ncgmax, C.c_double(step),
                          _p(par, f64p), _p(dpar, f64p), _p(cgfac, f64p),
                          cgres.ctypes.data_as(C.POINTER(C.c_float)))
    return par, dpar, cgfac, cgres, ncg


def mcm(sens, wmatd, wdfak, ltri, smatm, nx=0, nachbar=None, maxnk=4, lam=1.0, res=True, cov2=True):
    """src/bmcm_mod.f90 buncert on the host Jacobian sens (nanz, manz):
    dict of the diagonals 'ata', 'reg', 'cov1' and (if asked) 'res', 'cov2'."""
    nanz, manz = sens.shape
    s = np.ascontiguousarray(np.asarray(sens, np.complex128).T)  # column-major
    out = {k: np.zeros(manz) for k in ("ata", "reg", "cov1", "res", "cov2")}
    nb = np.ascontiguousarray(nachbar if nachbar is not None else np.zeros(1), np.int32)
    e = lib().or_mcm(nanz, manz, _p(s, f64p), _p(np.ascontiguousarray(wmatd, np.float64), f64p),
                     _p(np.ascontiguousarray(wdfak, np.int32), i32p), int(ltri),
                     _p(np.ascontiguousarray(smatm, np.float64), f64p), int(nx), _p(nb, i32p), int(maxnk),
                     C.c_double(lam), _p(out["ata"], f64p), _p(out["reg"], f64p), _p(out["cov1"], f64p),
                     _p(out["res"], f64p) if res else None, _p(out["cov2"], f64p) if (res and cov2) else None)
    if e:
        raise RuntimeError(f"mcm errnr {e}")
    if not res:
        del out["res"]
    if not (res and cov2):
        del out["cov2"]
    return out


def column_sums(sens, wa, wb, wc):
    """src/bbsens.f90 / bata column sums: sum_i |J_ij| wa_i, sum_i |Re J_ij|
    wb_i, sum_i Re(J_ij)^2 wc_i."""
    J = np.asarray(sens)
    return (np.abs(J).T @ wa, np.abs(J.real).T @ wb, (J.real ** 2).T @ wc)
