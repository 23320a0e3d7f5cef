"""CRTomo's complex-resistivity inversion loop over the GPU hot path.

The outer loop of src/inv.f90:330-990 restated on the host: the data misfit
(src/dmisft.f90), the first regularisation parameter (src/blam0.f90), the
lambda search and the step-length search (src/inv.f90:760-905 with
src/parfit.f90), src/bpar.f90, src/bsigma.f90 and the roughness
(src/brough_mod.f90).  Each step calls a backend for the three heavy parts:
the forward with src/bvolti.f90 voltages, the Jacobian of src/bsensi.f90, and
the Gauss-Newton update of src/update.f90 + src/cg_mod.f90.  DeviceBackend
runs them through the C ABI (crgpu_forward, crgpu_sens, crgpu_update); the
controller holds only O(nanz + manz) vectors.

Covered: the complex inversion stage (CRI) and the final phase improvement
(lfphai: phase weights, a new lambda_0 from Re(J), the phase-only update of
crgpu_update_fpi, the optional restart from the homogeneous phase, lffhom)
with the error model of src/rdati.f90 (or individual errors), homogeneous or
file start models (src/bsigm0.f90), structured (ltri 0) and triangular
(ltri 1, 2) smoothness, a fixed lambda (llamf), the polarity checks
(src/chkpol.f90, chkpo2 of src/dmisft.f90), the stopping rules of
src/inv.f90:560-640, DC inversion (ldc: the backends in DC mode,
crgpu_set_dc, and the real update crgpu_update_dc) and robust inversion
(lrobust: the reweighting of src/dmisft.f90:128-176), and difference
inversion (ldiff: read_difference, the misfit and update against d0 - fm0).
Data noise (lnse, noise.py) is added to the data as they are read.  Prior
models without reference-state data raise NotImplementedError.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import List, Optional

import numpy as np

from . import formats
from . import fortran_io as FIO
from . import noise as N
from . import regularization as R

_PI = math.acos(-1.0)


def _q(a: float, b: float) -> float:
    """a / b with IEEE semantics (0/0 is NaN and compares false, as in the
    reference's tests on bdpar/bdalt when an update is zero)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


# ---------------------------------------------------------------------------
# crtomo.cfg (src/rall.f90:230-470)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class CRTomoConfig:
    mswitch: int
    delem: str
    delectr: str
    dstrom: str
    ramd: str
    ldiff: bool
    dd0: str
    dm0: str
    dfm0: str
    nx: int
    nz: int
    alfx: float
    alfz: float
    itmax: int
    ldc: bool
    lrobust: bool
    lfphai: bool
    stabw0: float
    stabm0: float
    stabpA1: float
    stabpB: float
    stabpA2: float
    stabp0: float
    lrho0: bool
    bet0: float
    pha0: float
    lagain: bool
    swrtr: int
    lsink: bool
    nsink: int
    lrandb2: bool
    drandb: str
    ltri: int = 0
    llamf: int = 0
    lamfix: float = 0.0
    lffhom: bool = False
    noise: Optional[tuple] = None  # (iseed, A, B, A1, B1, A2, p0) when data noise is added


def _cfg_lines(path: str):
    with open(path) as fh:
        lines = fh.read().splitlines()
    pos = 0

    def next_line() -> str:
        """src/get_unit.f90 read_comments, then one record."""
        nonlocal pos
        while pos < len(lines) and lines[pos].lstrip().startswith("#"):
            pos += 1
        if pos >= len(lines):
            raise formats.CRError(2, f"end of file in {path}")
        pos += 1
        return lines[pos - 1]

    def at_end() -> bool:
        q = pos
        while q < len(lines) and lines[q].lstrip().startswith("#"):
            q += 1
        return q >= len(lines)

    return next_line, at_end


def _tok(line: str, n: int = 1):
    toks = formats._Records._tokens(line)
    if len(toks) < n:
        raise ValueError(line)
    return toks[:n]


def read_crtomo_cfg(path: str) -> CRTomoConfig:
    """crtomo.cfg in the order src/rall.f90:230-470 reads it."""
    nxt, at_end = _cfg_lines(path)
    v = {}
    line = nxt()
    try:
        v["mswitch"] = int(_tok(line)[0])
    except ValueError:  # src/rall.f90:234 (err=98: mswitch stays 0)
        v["mswitch"] = 0
    for key in ("delem", "delectr", "dstrom", "ramd"):
        v[key] = nxt().strip()
    v["ldiff"] = formats._logical(_tok(nxt())[0])
    for key in ("dd0", "dm0", "dfm0"):
        v[key] = nxt().strip()
    line = nxt()  # iseedpri, modl_stdn (a failing read consumes the record)
    v["nx"] = int(_tok(nxt())[0])
    v["nz"] = int(_tok(nxt())[0])
    v["alfx"] = formats._f(_tok(nxt())[0])
    v["alfz"] = formats._f(_tok(nxt())[0])
    v["itmax"] = int(_tok(nxt())[0])
    for key in ("ldc", "lrobust", "lfphai"):
        v[key] = formats._logical(_tok(nxt())[0])
    for key in ("stabw0", "stabm0", "stabpA1", "stabpB", "stabpA2", "stabp0"):
        v[key] = formats._f(_tok(nxt())[0])
    v["lrho0"] = formats._logical(_tok(nxt())[0])
    v["bet0"] = formats._f(_tok(nxt())[0])
    v["pha0"] = formats._f(_tok(nxt())[0])
    v["lagain"] = formats._logical(_tok(nxt())[0])
    v["swrtr"] = int(_tok(nxt())[0])
    v["lsink"] = formats._logical(_tok(nxt())[0])
    v["nsink"] = int(_tok(nxt())[0])
    v["lrandb2"] = formats._logical(_tok(nxt())[0])
    v["drandb"] = nxt().strip()
    cfg = CRTomoConfig(**v)
    if not at_end():  # src/rall.f90:420-445, read '(I2)'
        line = nxt()
        try:
            cfg.ltri = int(line[:2])
        except ValueError:
            cfg.ltri = 0
        if cfg.ltri & 32:
            cfg.llamf = 1
            try:
                cfg.lamfix = formats._f(_tok(nxt())[0])
            except (ValueError, formats.CRError):
                cfg.lamfix = 1.0
            cfg.ltri -= 32
            if cfg.ltri & 64:
                cfg.llamf += 2
                cfg.ltri -= 64
    if cfg.ltri > 15:
        raise formats.CRError(1, "ltri switch above 15")
    cfg.lffhom = cfg.stabp0 < 0  # src/rall.f90:470-471
    if cfg.lffhom:
        cfg.stabp0 = -cfg.stabp0
    noisemod = os.path.join(os.path.dirname(os.path.abspath(path)), "crt.noisemod")
    if cfg.stabw0 < 0:  # src/rall.f90:484-505: noise coupled to the error model, seed on the next line
        cfg.stabw0 = -cfg.stabw0
        iseed = 1
        if not at_end():
            try:
                iseed = int(_tok(nxt())[0])
            except (ValueError, IndexError):
                iseed = 1
        cfg.noise = (iseed, cfg.stabw0, cfg.stabm0, cfg.stabpA1, cfg.stabpB, cfg.stabpA2, cfg.stabp0)
    elif os.path.exists(noisemod):  # src/rall.f90:480-516 (lnse2)
        cfg.noise = N.read_noisemodel(noisemod)
    if (cfg.nx <= 0 or cfg.nz <= 0) and cfg.ltri == 0:
        cfg.ltri = 1
    if cfg.ltri == 0 and (cfg.nx < 2 or cfg.nz < 2):
        raise formats.CRError(89, "structured smoothness needs nx, nz >= 2")
    if cfg.itmax < 0 or cfg.itmax >= 100:
        raise formats.CRError(61, "itmax outside 0..99")
    if cfg.stabw0 <= 0.0 or cfg.stabm0 < 0.0:
        raise formats.CRError(104, "resistance error model")
    if (not cfg.ldc and cfg.lfphai and (cfg.stabp0 < 0 or cfg.stabpA2 < 0 or
                                        (cfg.stabp0 == 0 and cfg.stabpA2 == 0 and cfg.stabpA1 == 0))):
        raise formats.CRError(105, "phase error model")
    if cfg.lrho0 and (cfg.bet0 <= 0.0 or (not cfg.ldc and abs(cfg.pha0) > 1e3 * _PI)):
        raise formats.CRError(91, "homogeneous start model")
    if cfg.ldiff:  # src/rall.f90:624-629 (with reference-state data and response given)
        cfg.lrho0 = False
        cfg.ldc = True
    if cfg.ldc:
        cfg.lfphai = False
    return cfg


# ---------------------------------------------------------------------------
# data and error model (src/rdati.f90:100-375)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Data:
    strnr: np.ndarray
    vnr: np.ndarray
    dat: np.ndarray        # -ln|R| - i phase/1000 (complex)
    wmatdr: np.ndarray     # 1/eps_r^2
    wmatdp: np.ndarray     # 1/eps_p^2
    wmatd_cri: np.ndarray  # 1/(eps_r^2 + eps_p^2)
    wmatd: Optional[np.ndarray] = None  # the working weights when set apart (difference inversion)
    d0: Optional[np.ndarray] = None   # difference inversion: -ln|R| of the reference-state data
    fm0: Optional[np.ndarray] = None  # and of the reference-state model's response


def make_data(strnr, vnr, bet, pha, cfg: CRTomoConfig) -> Data:
    """Data from arrays with the error model of src/rdati.f90:234-255 (bet:
    |R| in ohm, pha: phase in mrad)."""
    bet = np.asarray(bet, np.float64)
    pha = np.zeros_like(bet) if cfg.ldc else np.asarray(pha, np.float64)
    if np.any(bet <= 0.0):
        raise formats.CRError(94, "resistance not positive")
    stabw = 1e-2 * cfg.stabw0 + cfg.stabm0 / bet
    stabwp = (cfg.stabpA1 * bet ** cfg.stabpB + 1e-2 * cfg.stabpA2 * np.abs(pha) + cfg.stabp0) * 1e-3
    dat = -np.log(bet) - 1j * pha / 1e3
    with np.errstate(divide="ignore"):
        wr = 1.0 / stabw ** 2
        wp = np.zeros_like(bet) if cfg.ldc else 1.0 / stabwp ** 2
        wc = np.zeros_like(bet) if cfg.ldc else 1.0 / (stabw ** 2 + stabwp ** 2)
    return Data(strnr=np.asarray(strnr, np.int32), vnr=np.asarray(vnr, np.int32), dat=dat, wmatdr=wr,
                wmatdp=wp, wmatd_cri=wc)


def read_difference(data: Data, d0_path: str, fm0_path: str, m0_path: str, elanz: int,
                    cfg: Optional[CRTomoConfig] = None):
    """The reference state of a difference inversion (src/rall.f90:853-943):
    d0 from the reference-state data file, fm0 from the reference-state
    model's response (a voltNN.dat: strnr vnr |R| wdfak), both matched to
    the data by (strnr, vnr) where wdfak is 1; data without a match are
    discarded.  m0 = ln sigma of the reference-state model (a rhoNN.mag:
    x y log10 rho).  Returns (data kept, with d0 / fm0 set; m0).

    As the reference's loop drops a datum it moves strnr, vnr, dat and the
    working weights wmatd (set before, src/rall.f90:805-817) down by one, but
    not wmatdr, wmatd_cri or (without lfphai) wmatdp: those keep the entries
    of the original positions.  The magnitude RMS of src/dmisft.f90 reads
    wmatdr, so it is reproduced with those weights."""
    rec = formats._Records(d0_path)
    nanz0 = int(rec._tokens(rec.read_line())[0])
    ic, ip, dum = [], [], []
    for _ in range(nanz0):
        t = rec._tokens(rec.read_line())
        if int(t[0]) - 10000 > 0:
            ic.append(int(t[0]))
            ip.append(int(t[1]))
            dum.append(formats._f(t[2]))
        else:
            e = [int(x) for x in t[:4]]
            ic.append(e[0] * 10000 + e[1])
            ip.append(e[2] * 10000 + e[3])
            dum.append(formats._f(t[4]))
    rec = formats._Records(fm0_path)
    rec.read_line()
    dum2, idum = [], []
    for _ in range(nanz0):
        t = rec._tokens(rec.read_line())
        dum2.append(formats._f(t[2]))
        idum.append(int(t[3]))
    keep, d0, fm0 = [], [], []
    for i in range(len(data.strnr)):
        for j in range(nanz0):  # the first match, as the reference's search finds it
            if data.strnr[i] == ic[j] and data.vnr[i] == ip[j] and idum[j] == 1:
                keep.append(i)
                d0.append(complex(-math.log(dum[j]), 0.0))
                fm0.append(complex(-math.log(dum2[j]), 0.0))
                break
    k = np.asarray(keep, np.int64)
    nk = len(k)
    lelerr = cfg is not None and ((not cfg.lfphai and not cfg.ldc) or bool(cfg.mswitch & 32))
    wmatd = (data.wmatd_cri if lelerr else data.wmatdr)[k]
    lfphai = cfg is not None and cfg.lfphai
    kept = Data(strnr=data.strnr[k], vnr=data.vnr[k], dat=data.dat[k], wmatdr=data.wmatdr[:nk].copy(),
                wmatdp=(data.wmatdp[k] if lfphai else data.wmatdp[:nk].copy()),
                wmatd_cri=data.wmatd_cri[:nk].copy(), wmatd=wmatd, d0=np.asarray(d0, np.complex128),
                fm0=np.asarray(fm0, np.complex128))
    rec = formats._Records(m0_path)
    rec.read_line()
    m0 = np.zeros(elanz, np.complex128)
    for j in range(elanz):
        m0[j] = complex(-math.log(10.0) * formats._f(rec._tokens(rec.read_line())[2]), 0.0)
    return kept, m0


def read_data(path: str, cfg: CRTomoConfig, eanz: int, noise_records: Optional[list] = None) -> Data:
    """Measurements and their weights.  Without individual errors the error
    model err(R) = A1 |R| + A2 (as an error of ln R: 1e-2 A1 + A2/|R|) and
    err(phase) = (A1p |R|^B + 1e-2 A2p |phase| + A3p) mrad, and with
    cfg.noise the synthetic noise of the noise model on R and the phase
    (noise.py; the weights keep the clean values' errors).  noise_records
    receives per datum (g_r, g_p, eps_r, eps_p, R, phase, R_new, phase_new)."""
    rec = formats._Records(path)
    first = rec._tokens(rec.read_line())
    nanz = int(first[0])
    lindiv = False
    if len(first) > 1:
        try:
            lindiv = formats._logical(first[1])
        except ValueError:
            lindiv = False
    strnr = np.zeros(nanz, np.int32)
    vnr = np.zeros(nanz, np.int32)
    dat = np.zeros(nanz, np.complex128)
    wr = np.zeros(nanz)
    wp = np.zeros(nanz)
    wc = np.zeros(nanz)
    crtf = None
    g_r = g_p = None
    if cfg.noise is not None:  # src/rdati.f90:127-138, drawn before any datum
        g_r, g_p = N.draw(cfg.noise, nanz, cfg.ldc)
    for i in range(nanz):
        t = rec._tokens(rec.read_line())
        if crtf is None:
            crtf = int(t[0]) - 10000 >= 0
        if crtf:
            s, v, rest = int(t[0]), int(t[1]), t[2:]
        else:
            e = [int(x) for x in t[:4]]
            s, v, rest = e[0] * 10000 + e[1], e[2] * 10000 + e[3], t[4:]
        bet = formats._f(rest[0])
        pha = 0.0 if cfg.ldc else formats._f(rest[1])
        if lindiv:
            k = 1 if cfg.ldc else 2
            stabw = formats._f(rest[k]) / bet
            stabwp = 0.0 if cfg.ldc else 1e-3 * formats._f(rest[k + 1])
            if stabw <= 0 or (not cfg.ldc and stabwp <= 0):
                raise formats.CRError(88, f"datum {i + 1}: error not positive")
        else:
            stabwp = (cfg.stabpA1 * bet ** cfg.stabpB + 1e-2 * cfg.stabpA2 * abs(pha) + cfg.stabp0) * 1e-3
            if bet <= 0.0:
                raise formats.CRError(94, f"datum {i + 1}: resistance not positive")
            stabw = 1e-2 * cfg.stabw0 + cfg.stabm0 / bet
            if g_r is not None:  # src/rdati.f90:257-290
                gp = None if g_p is None else float(g_p[i])
                nb, npha, er, ep = N.apply(bet, pha, float(g_r[i]), gp, cfg.noise, cfg.ldc)
                if noise_records is not None:
                    noise_records.append((float(g_r[i]), gp, er, ep, bet, pha, nb, npha))
                bet, pha = nb, npha
        if bet <= 0.0:
            raise formats.CRError(94, f"datum {i + 1}: resistance not positive")
        if not cfg.ldc and abs(pha) > 1e3 * _PI:
            raise formats.CRError(95, f"datum {i + 1}: phase beyond pi")
        e1, e2, e3, e4 = s % 10000, s // 10000, v % 10000, v // 10000
        if min(e1, e2, e3, e4) < 0 or max(e1, e2, e3, e4) > eanz:
            raise formats.CRError(46, f"datum {i + 1}: electrode number")
        strnr[i], vnr[i] = s, v
        dat[i] = complex(-math.log(bet), -pha / 1e3)
        wr[i] = _q(1.0, stabw ** 2)
        if not cfg.ldc:  # a phase error of 0 gives an infinite weight, as in the reference
            wc[i] = _q(1.0, stabw ** 2 + stabwp ** 2)
            wp[i] = _q(1.0, stabwp ** 2)
    if lindiv:
        t = rec._tokens(rec.read_line())
        sw = formats._f(t[0])
        if cfg.ldc:
            wr *= sw * sw
        else:
            swp = formats._f(t[1])
            if sw <= 0 or swp <= 0:
                raise formats.CRError(88, "error scale not positive")
            wr *= sw * sw
            wp *= swp * swp
    return Data(strnr=strnr, vnr=vnr, dat=dat, wmatdr=wr, wmatdp=wp, wmatd_cri=wc)


# ---------------------------------------------------------------------------
# misfit, polarity, first lambda, step length, roughness
# ---------------------------------------------------------------------------
def _phase_class(im: float) -> int:
    """+1 / -1 when a phase lies outside (-pi/2, pi/2] (src/chkpol.f90)."""
    if im > _PI / 2.0:
        return -1
    if im <= -_PI / 2.0:
        return 1
    return 0


def chkpo2(dati: complex, sigi: complex, lpol: bool = False):
    """Local polarity correction of one datum for the misfit (chkpo2 of
    src/dmisft.f90:230-300): (cdat, csig, wdlok)."""
    redat, imdat, resig, imsig = dati.real, dati.imag, sigi.real, sigi.imag
    idat, isig = _phase_class(imdat), _phase_class(imsig)
    wdlok = 1
    if idat == 0 and isig != 0:
        imsig = imsig + isig * _PI
        if not lpol:
            imdat = imdat - math.copysign(_PI, imdat)
        wdlok = 0
    elif idat != 0 and isig == 0:
        if lpol:
            imdat = imdat + idat * _PI
        wdlok = 0
    elif idat != 0 and isig != 0:
        imsig = imsig + isig * _PI
        imdat = imdat + idat * _PI
    return complex(redat, imdat), complex(resig, imsig), wdlok


@dataclasses.dataclass
class Misfit:
    nrmsd: float
    betrms: float
    pharms: float
    npol: int


def _phase_classes(im: np.ndarray) -> np.ndarray:
    """_phase_class of every element."""
    return np.where(im > _PI / 2.0, -1, np.where(im <= -_PI / 2.0, 1, 0))


def _seqsum(v: np.ndarray) -> float:
    """A sum in index order, as the reference's loops add (cumsum is sequential)."""
    return float(np.cumsum(v)[-1]) if len(v) else 0.0


def dmisft(dat, sigmaa, wmatd, wmatdr, wmatdp, lfpi: bool = False, lpol: bool = False, off=None) -> Misfit:
    """src/dmisft.f90:60-125 (robust reweighting: robust_weights), the
    polarity cases of chkpo2 applied element-wise and the sums taken in index
    order.  off: d0 - fm0 of a difference inversion (src/dmisft.f90:97-101)."""
    dat = np.asarray(dat, np.complex128)
    sigmaa = np.asarray(sigmaa, np.complex128)
    redat, imdat = dat.real.copy(), dat.imag.copy()
    resig, imsig = sigmaa.real.copy(), sigmaa.imag.copy()
    idat, isig = _phase_classes(imdat), _phase_classes(imsig)
    wdlok = np.ones(len(dat), np.int64)
    c1 = (idat == 0) & (isig != 0)
    c2 = (idat != 0) & (isig == 0)
    c3 = (idat != 0) & (isig != 0)
    imsig[c1] = imsig[c1] + isig[c1] * _PI
    if not lpol:
        imdat[c1] = imdat[c1] - np.copysign(_PI, imdat[c1])
    wdlok[c1] = 0
    if lpol:
        imdat[c2] = imdat[c2] + idat[c2] * _PI
    wdlok[c2] = 0
    imsig[c3] = imsig[c3] + isig[c3] * _PI
    imdat[c3] = imdat[c3] + idat[c3] * _PI
    dre, dim = redat - resig, imdat - imsig
    if off is not None:
        dre, dim = dre - off.real, dim - off.imag
    psi = np.sqrt(np.asarray(wmatd, np.float64)) * (np.abs(dim) if lfpi else np.hypot(dre, dim))
    idum = int(wdlok.sum())
    with np.errstate(invalid="ignore"):  # an infinite weight times 0 is NaN, as in the reference
        nrmsd = _seqsum(psi * psi * wdlok)
        betrms = _seqsum(np.asarray(wmatdr, np.float64) * wdlok * dre * dre)
        pharms = _seqsum(np.asarray(wmatdp, np.float64) * wdlok * dim * dim)
    if idum == 0:
        raise formats.CRError(99, "no datum left for the misfit")
    m = Misfit(math.sqrt(nrmsd / idum), math.sqrt(betrms / idum), math.sqrt(pharms / idum), len(dat) - idum)
    m.psi, m.wdlok = psi, wdlok
    return m


def robust_weights(wmatd, psi, wdlok, l1min: float = 1.0):
    """The robust reweighting of src/dmisft.f90:128-176 (after LaBrecque):
    estimated errors eps2_i = sqrt(psi_i) / sqrt(wmatd_i), scaled to the
    1-norm and kept at least the prior errors; (l1rat, new wmatd or None when
    l1rat <= l1min).  Sums in index order."""
    wmatd = np.asarray(wmatd, np.float64)
    dum = 1.0 / np.sqrt(wmatd)
    eps2 = dum * np.sqrt(psi)
    with np.errstate(divide="ignore", invalid="ignore"):
        norm = _seqsum(psi * wdlok)
        norm2 = _seqsum(psi * wdlok * dum / eps2)
        eps2 = eps2 * norm2 / norm
        eps2 = np.maximum(dum, eps2)
        norm2 = _seqsum(psi * wdlok * dum / eps2)
    l1rat = norm / norm2
    if l1rat > l1min:
        return l1rat, 1.0 / (eps2 * eps2)
    return l1rat, None


def parfit(fa: float, fb: float, fc: float, fmin: float, smin: float, step: float) -> float:
    """src/parfit.f90: step length from the misfits at steps 0, 0.5 and 1
    (parabola through the three, or a linear interpolation to fmin), clipped
    to [smin, 1].  `step` is kept where no case applies."""
    a, b, c = 0.0, 0.5, 1.0

    def parabola():
        bma, fbmfc, bmc, fbmfa = b - a, fb - fc, b - c, fb - fa
        return b - (bma * bma * fbmfc - bmc * bmc * fbmfa) / (2.0 * (bma * fbmfc - bmc * fbmfa))

    if fa > fb:
        if fb <= fc:
            if fb <= fmin:
                if fa < fmin and fc > fa:
                    step = b + (c - b) * (fmin - fb) / (fc - fb)
                else:
                    step = a + (b - a) * (fmin - fa) / (fb - fa)
            else:
                step = parabola()
        elif fb > fc:
            if fb <= fmin:
                step = a + (b - a) * (fmin - fa) / (fb - fa)
            elif fc <= fmin:
                step = b + (c - b) * (fmin - fb) / (fc - fb)
            else:
                step = c
    elif fa < fb:
        if fb >= fc:
            if fb >= fmin:
                if fa > fmin and fc < fa:
                    step = b + (c - b) * (fmin - fb) / (fc - fb)
                else:
                    step = a + (b - a) * (fmin - fa) / (fb - fa)
            else:
                step = parabola()
        elif fb < fc:
            if fb >= fmin:
                step = a + (b - a) * (fmin - fa) / (fb - fa)
            elif fc >= fmin:
                step = b + (c - b) * (fmin - fb) / (fc - fb)
            else:
                step = c
    elif fa == fb:
        if fb > fc:
            if fb < fmin:
                step = parabola()
            elif fc <= fmin:
                step = b + (c - b) * (fmin - fb) / (fc - fb)
            else:
                step = c
        elif fb < fc:
            if fb > fmin:
                step = parabola()
            elif fc >= fmin:
                step = b + (c - b) * (fmin - fb) / (fc - fb)
            else:
                step = c
        elif fb == fc:
            step = smin
    step = max(smin, step)
    return min(c, step)


def roughness(par: np.ndarray, ltri: int, smatm: np.ndarray, nachbar: Optional[np.ndarray], nx: int,
              lfpi: bool = False) -> float:
    """Re(m^H R^T R m) of src/brough_mod.f90 (broughreg, broughtri)."""
    manz = len(par)
    if ltri == 0:
        cd = smatm[0] * par
        cd[1:] += smatm[1][:-1] * par[:-1]
        cd[:-1] += smatm[1][:-1] * par[1:]
        cd[nx:] += smatm[2][:-nx] * par[:-nx]
        cd[:manz - nx] += smatm[2][:manz - nx] * par[nx:]
    elif ltri in (1, 2):
        nk = smatm.shape[0] - 1
        cd = smatm[nk] * par
        for j in range(nk):
            nbj = nachbar[j]
            ok = nbj != 0
            cd[ok] += smatm[j][ok] * par[nbj[ok] - 1]
    else:
        raise NotImplementedError(f"roughness for ltri = {ltri}")
    # the reference sums element by element; the order changes only rounding
    if lfpi:
        return float(np.sum(cd.imag * par.imag))
    return float(np.sum((cd * np.conj(par)).real))


# ---------------------------------------------------------------------------
# backends: forward + bvolti, bsensi, update
# ---------------------------------------------------------------------------
class DeviceBackend:
    """The heavy steps on the GPU through the C ABI (one context)."""

    def __init__(self, grid, survey, kwn, kwnwi, swrtr: int, lsink: bool, nsink: int, precision: int,
                 refinement: Optional[tuple] = None, ldc: bool = False):
        from .crmod import CRMod
        self.m = CRMod(grid, survey, kwn, kwnwi, swrtr=swrtr, lsink=lsink, nsink=nsink, precision=precision)
        if refinement is not None:
            self.m.set_refinement(*refinement)
        if ldc:
            self.m.set_dc(True)

    def forward(self, sigma: np.ndarray) -> np.ndarray:
        return self.m.forward(sigma, volt_mode=1)["sigmaa"]

    def sensitivities(self):
        self.m.sens_on_device(1)

    def update(self, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx, nachbar, lam, eps, ncgmax, step, par,
               phase_only=False, dc=False):
        p, dp, cgfac, cgres, ncg = self.m.update(wmatd, wdfak, dat, sigmaa, ltri, smatm, nx=nx, nachbar=nachbar,
                                                 lam=lam, eps=eps, ncgmax=ncgmax, step=step, par=par,
                                                 phase_only=phase_only, dc=dc)
        return dp, ncg

    def jtj(self, wmatd, wdfak, phase_only: bool) -> np.ndarray:
        return self.m.blam0_jtj(wmatd, wdfak, phase_only)

    def kfak(self) -> np.ndarray:
        return self.m.bkfak()

    def mcm(self, wmatd, wdfak, ltri, smatm, nx, nachbar, lam, res, cov2) -> dict:
        return self.m.mcm(wmatd, wdfak, ltri, smatm, nx=nx, nachbar=nachbar, lam=lam, res=res, cov2=cov2)

    def column_sums(self, wa, wb, wc):
        return self.m.column_sums(wa, wb, wc)

    def close(self):
        self.m.close()


def blam0(cfg: CRTomoConfig, lamnull_cri: float, lamnull_fpi: float, manz: int, nanz: int, lfpi: bool,
          jtj_fn, wmatd, wdfak) -> float:
    """src/blam0.f90: a preset lambda_0 (nz = -1: max(manz, nanz); nz < -1:
    |nz|; crt.lamnull), else 5 mean_j |(J^H W J 1)_j| 2/(alfx + alfz) --
    jtj_fn(wmatd, wdfak, lfpi) gives |(J^H W J 1)_j| (Re(J) when lfpi)."""
    eps = np.finfo(np.float64).eps
    if ((cfg.llamf & 1) or lamnull_cri > eps) and not lfpi:
        return float(max(manz, nanz)) if cfg.nz == -1 else float(lamnull_cri)
    if (cfg.llamf & 1) or lamnull_fpi > eps:
        return float(lamnull_fpi)
    jtj = np.asarray(jtj_fn(wmatd, wdfak, lfpi))
    lam = float(np.sum(jtj)) / manz
    return lam * 2.0 / (cfg.alfx + cfg.alfz) * 5.0


# ---------------------------------------------------------------------------
# the loop (src/inv.f90:330-990)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Row:
    """One line of inv.ctr (src/kont2.f90): kind 'IT' (an accepted model) or
    'UP' (a trial of the lambda or step-length search); 'PIT' and 'PUP' in
    the final phase improvement."""
    kind: str
    index: int
    nrmsd: float
    bdpar: float = 0.0
    lam: float = 0.0
    rough: float = 0.0
    ncg: int = 0
    betrms: float = 0.0
    pharms: float = 0.0
    npol: int = 0
    step: float = 0.0
    first: bool = False
    l1rat: Optional[float] = None  # robust inversion: the L1 ratio of src/dmisft.f90


class Inversion:
    """CRTomo's inversion of one data set (complex stage).

    grid, enr: the mesh and electrodes; data: read_data(); cfg:
    read_crtomo_cfg().  backend: an object with forward(sigma) -> sigmaa,
    sensitivities(), update(...) -> (dpar, ncg) and jtj(wmatd, wdfak,
    phase_only) -> |(J^H W J 1)_j|, as DeviceBackend.  sigma_start: the start
    model when cfg.lrho0 is off; ncgmax: a cap on the CG steps other than
    the reference's manz/10."""

    # src/rall.f90:196-222 defaults
    nrmsdm = 1.0
    mqrms = 2e-2
    eps = 1e-4
    stpmin = 1e-3
    bdmin = 1e-3
    nlam = 30
    fstart = 0.5
    fstop = 0.9
    lpol = False

    def __init__(self, grid, data: Data, cfg: CRTomoConfig, backend, sigma_start=None,
                 lamnull: Optional[tuple] = None, phase_stage: bool = True, ncgmax: Optional[int] = None,
                 m0=None):
        if cfg.ldiff and (data.d0 is None or m0 is None):
            raise NotImplementedError("difference inversion needs the reference state (read_difference)")
        self.doff = (data.d0 - data.fm0) if cfg.ldiff else None
        if cfg.ltri not in (0, 1, 2):
            raise NotImplementedError(f"regularisation ltri = {cfg.ltri} is not built")
        self.grid, self.data, self.cfg, self.b = grid, data, cfg, backend
        self.manz = grid.elanz if cfg.ltri != 0 else cfg.nx * cfg.nz
        if self.manz != grid.elanz:
            raise formats.CRError(50, "manz /= elanz is not implemented")
        self.nanz = len(data.dat)
        self.ncgmax = self.manz // 10 if cfg.ltri < 5 else self.manz  # src/rall.f90:745-746
        if ncgmax is not None:
            self.ncgmax = int(ncgmax)
        # first lambda (src/rall.f90:768-796; lamnull = the crt.lamnull file)
        if lamnull is not None:
            self.lamnull_cri, self.lamnull_fpi = lamnull
        elif cfg.llamf & 1:
            self.lamnull_cri = self.lamnull_fpi = cfg.lamfix
        elif cfg.nz == -1:
            self.lamnull_cri, self.lamnull_fpi = float(max(self.manz, self.nanz)), 0.0
        elif cfg.nz < 0:
            self.lamnull_cri, self.lamnull_fpi = float(abs(cfg.nz)), 0.0
        else:
            self.lamnull_cri = self.lamnull_fpi = 0.0
        # weights (src/rall.f90:805-817): the complex stage with a final phase
        # improvement fits the magnitude error only
        lelerr = (not cfg.lfphai and not cfg.ldc) or bool(cfg.mswitch & 32)
        self.wmatd = (data.wmatd_cri if lelerr else data.wmatdr).copy() if data.wmatd is None else data.wmatd.copy()
        # smoothness (src/bsmatm_mod.f90)
        if cfg.ltri == 0:
            self.nachbar = None
            self.smatm = R.bsmatmreg(grid, cfg.nx, cfg.nz, cfg.alfx, cfg.alfz)
        else:
            self.nachbar = R.bnachbar(grid)
            self.smatm = R.bsmatmtri(grid, self.nachbar, cfg.alfx, cfg.alfz)
        # start model (src/bsigm0.f90)
        if cfg.ldiff:  # src/bsigm0.f90:66-69: the reference-state model
            self.sigma = np.exp(np.asarray(m0, np.complex128))
        elif cfg.lrho0:
            s = complex(math.cos(cfg.pha0 / 1e3) / cfg.bet0, -math.sin(cfg.pha0 / 1e3) / cfg.bet0)
            self.sigma = np.full(grid.elanz, s, np.complex128)
        elif sigma_start is not None:
            self.sigma = np.array(sigma_start, np.complex128)
        elif 11 in set(np.asarray(grid.typ).tolist()):  # lbeta: src/bsigm0.f90:87-125
            self.sigma = np.full(grid.elanz, self._start_from_data(backend.kfak()), np.complex128)
        else:
            raise formats.CRError(100, "no start model (src/bsigm0.f90)")
        self.dat = data.dat.copy()
        self.swapped = np.zeros(self.nanz, bool)
        self.rows: List[Row] = []
        self.status = ""
        self.phase_stage = phase_stage  # run the final phase improvement (lfphai)
        self.stage_start = None         # first row of the phase stage
        self.models: List[dict] = []    # every accepted model (an IT / PIT line), for write_models
        self.lam_cri = None             # lambda when the final phase improvement started
        self.lamalt = None              # the last good lambda after run()

    def _start_from_data(self, kfak) -> complex:
        """src/bsigm0.f90:87-125: exp of the weighted mean of the data's
        log apparent conductivities (phases brought into (-pi/2, pi/2]),
        weights sqrt(wmatd) wdfak (all 1 here)."""
        s0 = 0j
        dum = 0.0
        for i in range(self.nanz):
            imdat = self.data.dat[i].imag
            idat = _phase_class(imdat)
            if idat != 0:
                imdat = imdat + idat * _PI
            redat = self.data.dat[i].real - math.log(abs(kfak[i]))
            dum2 = math.sqrt(self.wmatd[i]) * 1.0
            s0 = s0 + complex(redat, imdat) * complex(dum2)
            dum = dum + dum2
        if abs(dum) == 0.0:
            raise formats.CRError(99, "unable to find starting value sigma0")
        return np.exp(s0 / complex(dum))

    # -- pieces -----------------------------------------------------------------
    def _forward(self, sigma):
        sa = np.array(self.b.forward(sigma), np.complex128)
        s = self.swapped  # polarity already changed by chkpol: -ln(-V)
        if s.any():
            im = sa.imag[s]
            sa.imag[s] = np.where(im < 0, im + _PI, im - _PI)
        return sa

    def _chkpol(self, lsetup: bool):
        """src/chkpol.f90 with lpol off: change the polarity of the model
        datum (the potential electrodes swap) and exclude the datum."""
        imdat, imsig = self.dat.imag.copy(), self.sigmaa.imag.copy()
        idat, isig = _phase_classes(imdat), _phase_classes(imsig)
        c1 = (idat == 0) & (isig != 0)
        c2 = (idat != 0) & (isig == 0)
        c3 = (idat != 0) & (isig != 0)
        flip = c1 | c3
        self.swapped[flip] = ~self.swapped[flip]
        imsig[flip] = imsig[flip] + isig[flip] * _PI
        imdat[c1] = imdat[c1] - np.copysign(_PI, imdat[c1])
        imdat[c3] = imdat[c3] + idat[c3] * _PI
        self.sigmaa = self.sigmaa.real + 1j * imsig
        self.dat = self.dat.real + 1j * imdat
        wdfak = np.ones(self.nanz, np.int32)
        wdfak[c1 | c2] = 0
        self.wdfak = wdfak

    def _misfit(self):
        m = dmisft(self.dat, self.sigmaa, self.wmatd, self.data.wmatdr, self.data.wmatdp, self.lfpi, self.lpol,
                   self.doff)
        self.nrmsd, self.betrms, self.pharms, self.npol = m.nrmsd, m.betrms, m.pharms, m.npol
        if self.lrobust:  # src/dmisft.f90:128-176: the weights of the next update
            self.l1rat, w = robust_weights(self.wmatd, m.psi, m.wdlok, self.l1min)
            if w is not None:
                self.wmatd = w

    def _kont2(self, lsetup: bool):
        p = "P" if self.lfpi else ""
        if lsetup or (self.llam and not self.lstep):
            self.models.append(dict(it=self.it, sigma=self.sigma.copy(), sigmaa=self.sigmaa.copy(),
                                    wdfak=self.wdfak.copy(), betrms=self.betrms, pharms=self.pharms))
        l1 = self.l1rat if self.lrobust else None
        if lsetup:
            self.rows.append(Row(p + "IT", self.it, self.nrmsd, betrms=self.betrms, pharms=self.pharms,
                                 npol=self.npol, first=True, l1rat=l1))
        elif self.llam and not self.lstep:
            self.rows.append(Row(p + "IT", self.it, self.nrmsd, self.bdpar, self.lam, self.rough, self.ncg,
                                 self.betrms, self.pharms, self.npol, self.step, l1rat=l1))
        else:
            self.rows.append(Row(p + "UP", self.itr, self.nrmsd, self.bdpar, self.lam, self.rough, self.ncg,
                                 step=self.step, l1rat=l1))

    # -- the loop ---------------------------------------------------------------
    def run(self, max_iterations: Optional[int] = None) -> List[Row]:
        """Runs until a stopping rule of src/inv.f90:560-640 holds; the rule
        is in self.status ('79' iteration limit, '80' target misfit, '81' no
        misfit decrease, '92' minimal step twice, '109' minimal model change;
        'fpi' where the final phase improvement starts, when the Inversion
        was made with phase_stage=False).  With
        max_iterations the run also ends ('max_iterations') once that many
        models have been accepted."""
        cfg, b = self.cfg, self.b
        it = itr = 0
        rmsalt = 0.0
        lamalt = 1.0
        self.bdpar = bdalt = 1.0
        self.lsetup, self.lsetip, self.lfpi = True, False, False
        self.llam, ldlami, self.lstep, lfstep = False, True, False, False
        self.step, stpalt, alam = 1.0, 1.0, 0.0
        self.lam, dlam, dlalt, rmsreg, ldlamf = 0.0, 1.0, 1.0, 0.0, False
        self.rough, self.ncg = 0.0, 0
        dpar = np.zeros(self.manz, np.complex128)
        dpar2 = dpar.copy()
        ncg2 = 0
        sigma2 = self.sigma.copy()
        sgmaa2 = None
        self.wdfak = np.ones(self.nanz, np.int32)
        lfphai = cfg.lfphai
        self.lrobust, self.l1min, self.l1rat = cfg.lrobust, 1.0, 0.0  # src/rall.f90:194
        wmatd2 = self.wmatd.copy()
        while True:
            self.it, self.itr = it, itr
            # modelling (src/inv.f90:342-503)
            try:
                self.sigmaa = self._forward(self.sigma)
            except Exception as e:
                # a zero voltage (src/bvolti.f90, errnr 82) ends the run with the
                # last model (src/inv.f90:495-503); any other error -- e.g. a
                # non-positive DC pivot, errnr 28 -- aborts it, as in the reference
                if getattr(e, "errnr", None) != 82 or sgmaa2 is None:
                    raise
                self.sigma, self.sigmaa = sigma2, sgmaa2
                self.status = "82"
                break
            setup = self.lsetup or self.lsetip
            if setup:
                self._chkpol(setup)
            self._misfit()
            if self.nrmsd < 1e-12:
                self.nrmsd = self.nrmsdm * (1.0 - self.mqrms)
            self._kont2(setup)
            # stopping rules (src/inv.f90:560-640)
            if self.llam and not self.lstep:
                self._chkpol(setup)
                err2 = 0
                if stpalt == 0.0:
                    err2 = 92
                if abs(1.0 - _q(rmsalt, self.nrmsd)) <= self.mqrms:
                    err2 = 81
                if abs(1.0 - _q(self.nrmsd, self.nrmsdm)) <= self.mqrms and ldlamf:
                    err2 = 80
                if it >= cfg.itmax:
                    err2 = 79
                if abs(1.0 - _q(self.bdpar, bdalt)) < self.bdmin:
                    err2 = 109
                if err2 != 0 and not (lfphai and err2 != 79):
                    self.status = str(err2)
                    break
                if err2 != 0:
                    # final phase improvement (src/inv.f90:600-660): phase
                    # weights, a new lambda_0, the phase-only update
                    if not self.phase_stage:
                        self.status = "fpi"
                        break
                    self.wmatd = self.data.wmatdp.copy()
                    self.lam_cri = lamalt  # src/inv.f90:634: the lambda of the complex stage
                    self.lfpi, self.lsetip = True, True
                    lfphai, self.llam, ldlami, lfstep, self.step = False, False, True, True, 1.0
                    self.stage_start = len(self.rows)
                    if cfg.lffhom:  # restart from the start phase, same magnitudes
                        a = np.abs(self.sigma)
                        self.sigma = a * complex(math.cos(cfg.pha0 / 1e3), -math.sin(cfg.pha0 / 1e3))
                        self.lsetup = True
                        continue
                    self.lsetup = False
                    self._misfit()
                    self._kont2(True)
                    setup = True
                else:
                    lamalt = self.lam
                if max_iterations is not None and it >= max_iterations:
                    self.status = "max_iterations"
                    break
            if (self.llam and not self.lstep) or setup:
                it += 1
                itr = 0
                rmsreg, dlam, dlalt, ldlamf = 0.0, 1.0, 1.0, False
                self.bdpar = bdalt = 1.0
                rmsalt = self.nrmsd
                if it > 1:
                    lamalt = self.lam
                sigma2, sgmaa2 = self.sigma.copy(), self.sigmaa.copy()
                if self.lrobust:  # src/inv.f90:727
                    wmatd2 = self.wmatd.copy()
                b.sensitivities()
            else:
                self.sigma, self.sigmaa = sigma2.copy(), sgmaa2.copy()
                if self.lrobust:  # src/inv.f90:760
                    self.wmatd = wmatd2.copy()
            self.it, self.itr = it, itr
            if cfg.itmax == 0:
                self.status = "109"
                break
            # regularisation and step length (src/inv.f90:768-905)
            if cfg.llamf & 1:
                self.lam = cfg.lamfix
                if (cfg.llamf & 2) and it > 1:
                    self.lam = cfg.lamfix / (2.0 * (it - 1))
                self.llam = False
                if self.lsetup or self.lsetip:
                    self.lsetup = self.lsetip = False
            elif not self.lstep:
                if self.llam:
                    self.llam = False
                    self.step = 1.0
                else:
                    itr += 1
                    self.itr = itr
                    nr = self.nrmsd
                    search = ((((nr < rmsreg and itr <= self.nlam) or (dlam > 1.0 and itr <= self.nlam))
                               and (not ldlamf or dlalt <= 1.0)
                               and abs(1.0 - _q(self.bdpar, bdalt)) > self.bdmin
                               and abs(1.0 - _q(rmsreg, self.nrmsdm)) > self.mqrms)
                              or rmsreg == 0.0)
                    if search:
                        if self.lsetup or self.lsetip:
                            self.lam = blam0(cfg, self.lamnull_cri, self.lamnull_fpi, self.manz, self.nanz,
                                             self.lfpi, lambda w, d, p: b.jtj(w, d, p or cfg.ldc), self.wmatd,
                                             self.wdfak)
                            lamalt = self.lam
                        else:
                            dlalt = dlam
                            lr = math.log(nr / self.nrmsdm)
                            if ldlami:
                                ldlami = False
                                alam = max(abs(lr), math.log(1.0 + self.mqrms))
                                dlam = self.fstart
                            else:
                                alam = max(alam, abs(lr))
                                dlam = (math.log(self.fstop) * math.copysign(1.0, lr)
                                        + math.log(self.fstart / self.fstop) * lr / alam)
                                dlam = math.exp(dlam)
                            self.lam *= dlam
                            if dlalt > 1.0 and dlam < 1.0:
                                ldlamf = True
                            if dlam > 1.0:  # src/inv.f90:868
                                self.lrobust = False
                    else:
                        self.llam = True
                        self.lam /= dlam
                        if lfstep:
                            lfstep = False
                        else:
                            self.lstep = True
                            self.step = 0.5
                    if self.lsetup or self.lsetip:
                        self.lsetup = self.lsetip = False
                    elif not self.lstep:
                        rmsreg = self.nrmsd
            else:
                self.lstep = False
                self.step = parfit(rmsalt, self.nrmsd, rmsreg, self.nrmsdm, self.stpmin, self.step)
                if self.step == self.stpmin and stpalt == self.stpmin:
                    stpalt = 0.0
                else:
                    stpalt = self.step
            # update (src/bpar.f90, src/update.f90, src/bsigma.f90, src/brough_mod.f90)
            par = np.log(self.sigma)
            bdalt = self.bdpar
            if not self.llam:
                dpar2, ncg2 = dpar, self.ncg
                # difference inversion: dat - sigmaa - (d0 - fm0) (src/update.f90:241-279)
                dat_eff = self.dat if self.doff is None else self.dat - self.doff
                dpar, self.ncg = b.update(self.wmatd, self.wdfak, dat_eff, self.sigmaa, cfg.ltri, self.smatm,
                                          cfg.nx, self.nachbar, self.lam, self.eps, self.ncgmax, 1.0, par,
                                          phase_only=self.lfpi, dc=cfg.ldc)
                dpar = np.array(dpar, np.complex128)
            else:
                dpar, self.ncg = dpar2, ncg2
            par = par + self.step * dpar
            self.bdpar = float(np.sum((dpar * np.conj(dpar)).real)) * self.step
            self.sigma = np.exp(par)
            self.rough = roughness(par, cfg.ltri, self.smatm, self.nachbar, cfg.nx, self.lfpi)
            if cfg.llamf & 1:
                self.llam = True
        self.it, self.itr = it, itr
        self.lamalt = lamalt  # the last good lambda (src/inv.f90:1065, buncert)
        return self.rows


def format_rows(rows: List[Row]) -> str:
    """The IT/UP lines of inv.ctr, byte for byte as the formats 100-111 of
    src/kont2.f90:33-50 lay them out (T positions, A3, I3, G10.4, G9.3, I6,
    I4, F5.3)."""
    A, I, G, Fx = FIO.fmt_A, FIO.fmt_I, FIO.fmt_G, FIO.fmt_F
    out = []
    for r in rows:
        robust = r.l1rat is not None
        head = [(1, A(r.kind, 3)), (5, I(r.index, 3)), (11, G(r.nrmsd, 10, 4))]
        if r.first:  # formats 100 / 101
            f = head + [(69, G(r.betrms, 10, 4)), (81, G(r.pharms, 10, 4)), (93, I(r.npol, 4))]
            if robust:
                f.append((105, G(r.l1rat, 9, 3)))
        elif r.kind.endswith("IT"):  # formats 110 / 111
            f = head + [(23, G(r.bdpar, 10, 4)), (34, G(r.lam, 10, 4)), (46, G(r.rough, 10, 4)),
                        (58, I(r.ncg, 6)), (69, G(r.betrms, 10, 4)), (81, G(r.pharms, 10, 4)),
                        (93, I(r.npol, 4))]
            f += [(105, G(r.l1rat, 9, 3)), (117, Fx(r.step, 5, 3))] if robust else [(105, Fx(r.step, 5, 3))]
        else:  # formats 105 / 106
            f = head + [(23, G(r.bdpar, 9, 3)), (34, G(r.lam, 10, 4)), (46, G(r.rough, 10, 4)),
                        (58, I(r.ncg, 6))]
            f += [(105, G(r.l1rat, 9, 3)), (117, Fx(r.step, 5, 3))] if robust else [(105, Fx(r.step, 5, 3))]
        out.append(FIO.tab_record(f))
    return "".join(out)


def write_models(inv: "Inversion", ramd: str, ldc: bool = False):
    """The files src/wout.f90:61-200 writes for every accepted model NN, byte
    for byte as gfortran writes them: rhoNN.mag (elanz, TAB, the magnitude
    RMS; centroid x, y, log10 |rho|), rhoNN.pha (the phase RMS; x, y, phase
    of rho in mrad), rhoNN.modl (I7; 1/Re(sigma) and the phase in
    (2(1x,G12.4))), rhoNN.sig (Re, Im of sigma in REAL*8) and voltNN.dat
    (strnr, vnr, |R|, phase in mrad, wdfak)."""
    os.makedirs(ramd, exist_ok=True)
    g = inv.grid
    cx, cy = R._centroids(g)
    r4, r8, i4, rec = FIO.real4, FIO.real8, FIO.int4, FIO.record
    for m in inv.models:
        nn = f"{m['it']:02d}"
        rho = 1.0 / m["sigma"]
        pha = [1e3 * math.atan2(z.imag, z.real) for z in rho]
        with open(os.path.join(ramd, f"rho{nn}.mag"), "w") as fh:
            fh.write(rec([i4(g.elanz), FIO.char("\t"), r8(m["betrms"])]))
            fh.write("".join(rec([r4(cx[i]), r4(cy[i]), r4(math.log10(abs(rho[i])))]) for i in range(g.elanz)))
        with open(os.path.join(ramd, f"rho{nn}.modl"), "w") as fh:
            fh.write(FIO.fmt_I(g.elanz, 7) + "\n")
            # dum2 = real(1d3*datan2(...)): the phase passes through REAL*4
            fh.write("".join(" " + FIO.fmt_G(1.0 / m["sigma"][i].real, 12, 4) + " "
                             + FIO.fmt_G(float(np.float32(pha[i])), 12, 4) + "\n" for i in range(g.elanz)))
        if not ldc:
            with open(os.path.join(ramd, f"rho{nn}.pha"), "w") as fh:
                fh.write(rec([i4(g.elanz), FIO.char("\t"), r8(m["pharms"])]))
                fh.write("".join(rec([r4(cx[i]), r4(cy[i]), r4(pha[i])]) for i in range(g.elanz)))
            with open(os.path.join(ramd, f"rho{nn}.sig"), "w") as fh:
                fh.write(rec([i4(g.elanz), r8(m["betrms"]), r8(m["pharms"])]))
                fh.write("".join(rec([r8(z.real), r8(z.imag)]) for z in m["sigma"]))
        with open(os.path.join(ramd, f"volt{nn}.dat"), "w") as fh:
            fh.write(rec([i4(len(m["sigmaa"]))]))
            for i, sa in enumerate(m["sigmaa"]):
                cols = [r4(1.0 / math.exp(sa.real))] + ([] if ldc else [r4(-1e3 * sa.imag)])
                fh.write(rec([i4(inv.data.strnr[i]), i4(inv.data.vnr[i])] + cols + [i4(m["wdfak"][i])]))


def read_model_mag(path: str):
    """(elanz, rms, x, y, log10 |rho|) of a rhoNN.mag file."""
    with open(path) as fh:
        head = fh.readline().split()
        vals = np.loadtxt(fh)
    return int(head[0]), float(head[1]), vals[:, 0], vals[:, 1], vals[:, 2]


def run_crtomo(exe_dir: str, precision: int = 1, refinement=(8, 1e-10), write: bool = True):
    """CRTomo on a tomodir: reads exe_dir/crtomo.cfg and its
    inputs, inverts on the GPU and (write) puts the IT/UP lines into
    <ramd>/inv.ctr, the final model into <ramd>/rho.dat (magnitude in ohm m
    and phase in mrad, as src/rsigma.f90 reads a model) and every accepted
    model with its data into rhoNN.* / voltNN.dat (write_models).  Returns
    the Inversion."""
    cfg = read_crtomo_cfg(os.path.join(exe_dir, "crtomo.cfg"))

    def p(x):
        return os.path.normpath(os.path.join(exe_dir, x))

    grid = formats.read_elem(p(cfg.delem))
    enr = formats.read_elec(p(cfg.delectr), grid.sanz)
    recs: list = []
    data = read_data(p(cfg.dstrom), cfg, len(enr), recs)
    if write and cfg.noise is not None and recs:
        N.write_records(exe_dir, data.strnr, data.vnr, recs, cfg.ldc)
    survey = formats.Survey(enr=enr, strnr=data.strnr, vnr=data.vnr, strom=np.ones(len(data.strnr)))
    if cfg.swrtr:
        from .crmod import rwaven
        kwn, kwnwi = rwaven(grid, survey)
    else:  # src/rall.f90:818-838
        if 11 in set(np.asarray(grid.typ).tolist()):
            raise formats.CRError(110, "2D with mixed boundaries")
        kwn = np.array([0.0 if cfg.lrandb2 else 1e-6])
        kwnwi = np.zeros(1)
    sigma_start = m0 = None
    if cfg.ldiff:  # the reference state; the wavenumbers above came from all data
        data, m0 = read_difference(data, p(cfg.dd0), p(cfg.dfm0), p(cfg.dm0), grid.elanz, cfg)
        survey = formats.Survey(enr=enr, strnr=data.strnr, vnr=data.vnr, strom=np.ones(len(data.strnr)))
    elif not cfg.lrho0 and cfg.dm0:
        sigma_start = formats.read_rho(p(cfg.dm0), grid.elanz)
    b = DeviceBackend(grid, survey, kwn, kwnwi, cfg.swrtr, cfg.lsink, cfg.nsink, precision, refinement, cfg.ldc)
    try:
        if cfg.lrandb2:
            b.m.set_boundary_values(*formats.read_boundary_values(p(cfg.drandb), grid.sanz))
        inv = Inversion(grid, data, cfg, b, sigma_start=sigma_start, m0=m0)
        inv.run()
        if write:  # coverage and, by mswitch, uncertainty (src/inv.f90:1050-1065)
            from . import uncertainty
            uncertainty.write_all(inv, b, p(cfg.ramd))
    finally:
        b.close()
    if write:
        ramd = p(cfg.ramd)
        os.makedirs(ramd, exist_ok=True)
        with open(os.path.join(ramd, "inv.ctr"), "w") as fh:
            fh.write(format_rows(inv.rows))
        mag = 1.0 / np.abs(inv.sigma)
        pha = -1e3 * np.angle(inv.sigma)  # resistivity phase in mrad
        formats.write_rho(os.path.join(ramd, "rho.dat"), mag, pha)
        write_models(inv, ramd, cfg.ldc)
    return inv
