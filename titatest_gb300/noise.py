"""Synthetic data noise of CRTomo (lnse).

The portable generator of src/make_noise.f90 -- the three linear
congruential sequences with a 97-entry shuffle table of Press et al.
(ran1) and Gaussian deviates by the polar Box-Muller method -- and its use
by src/rdati.f90:110-140, 257-290: one deviate per datum for the magnitude
(seed iseed) and one for the phase (seed -iseed), added as
  R   <- R   + g_r (1e-2 A R + B)
  phi <- phi + g_p (A1 eps_r^B1 + 1e-2 A2 |phi| + p0)      [mrad]
before the data are taken to logarithms.  The noise model is either the
error model itself (a negative relative error in crtomo.cfg, the seed on
the line after the regularisation switch) or the file crt.noisemod
(src/make_noise.f90:50-124).

The arithmetic follows Fortran: INTEGER*4 products (no overflow for these
moduli), MOD and integer division truncating towards zero, and the scale
constants 1./M1 and 1./M2 evaluated in single precision and widened
(src/make_noise.f90:39-40).
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import formats

_N_RND = 97
_M1, _M2, _M3 = 259200, 134456, 243000
_IA1, _IA2, _IA3 = 7141, 8121, 4561
_IC1, _IC2, _IC3 = 54773, 28441, 51349
_RM1 = float(np.float32(1.0) / np.float32(_M1))
_RM2 = float(np.float32(1.0) / np.float32(_M2))


def _fmod(a: int, m: int) -> int:
    """Fortran MOD: the remainder takes the sign of a."""
    r = abs(a) % m
    return r if a >= 0 else -r


def _fdiv(a: int, b: int) -> int:
    """Fortran integer division (truncation towards zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


class PortableRandom:
    """Random_Init / Random_Draw / Random_Gauss of src/make_noise.f90."""

    def __init__(self, iseed: int = 1):
        ix1 = _fmod(_IC1 + iseed, _M1)
        ix1 = _fmod(_IA1 * ix1 + _IC1, _M1)
        ix2 = _fmod(ix1, _M2)
        ix1 = _fmod(_IA1 * ix1 + _IC1, _M1)
        ix3 = _fmod(ix1, _M3)
        self.rnd = [0.0] * _N_RND
        for i in range(_N_RND):
            ix1 = _fmod(_IA1 * ix1 + _IC1, _M1)
            ix2 = _fmod(_IA2 * ix2 + _IC2, _M2)
            self.rnd[i] = (float(ix1) + float(ix2) * _RM2) * _RM1
        self.ix = [ix1, ix2, ix3]

    def draw(self) -> float:
        ix1, ix2, ix3 = self.ix
        while True:
            ix1 = _fmod(_IA1 * ix1 + _IC1, _M1)
            ix2 = _fmod(_IA2 * ix2 + _IC2, _M2)
            ix3 = _fmod(_IA3 * ix3 + _IC3, _M3)
            i = 1 + _fdiv(_N_RND * ix3, _M3)
            if 1 <= i <= _N_RND:
                break
        v = self.rnd[i - 1]
        self.rnd[i - 1] = (float(ix1) + float(ix2) * _RM2) * _RM1
        self.ix = [ix1, ix2, ix3]
        return v

    def gauss(self) -> float:
        while True:
            x = 2.0 * self.draw() - 1.0
            y = 2.0 * self.draw() - 1.0
            z = x * x + y * y
            if z <= 1.0:
                break
        return x * math.sqrt(-2.0 * math.log(z) / z)

    def gauss_n(self, n: int) -> np.ndarray:
        return np.array([self.gauss() for _ in range(n)], np.float64)


def read_noisemodel(path: str, iseed: int = 1):
    """src/make_noise.f90:50-124 (get_noisemodel): the seed (an unreadable
    first line keeps `iseed`, the old file layout), A [%], B [Ohm m], A1,
    B1, A2 [%], p0 [mrad].  A negative entry is error 1 of the caller."""
    with open(path) as fh:
        lines = [ln for ln in fh.read().splitlines() if ln.strip()]
    k = 0
    try:
        iseed = int(lines[0].split()[0])
        k = 1
    except ValueError:
        pass
    vals = [formats._f(lines[k + j].split()[0]) for j in range(6)]
    if iseed < 0 or min(vals) < 0:
        raise formats.CRError(1, "noise model: negative seed or parameter (crt.noisemod)")
    return (iseed, *vals)


def draw(model, nanz: int, ldc: bool):
    """The deviates of rdati (src/rdati.f90:127-138): nanz for the
    magnitudes from seed iseed, and nanz for the phases from seed -iseed."""
    iseed = model[0]
    g_r = PortableRandom(iseed).gauss_n(nanz)
    g_p = None if ldc else PortableRandom(-iseed).gauss_n(nanz)
    return g_r, g_p


def apply(bet: float, pha: float, g_r: float, g_p, model, ldc: bool):
    """Noise on one datum (src/rdati.f90:257-290): (bet_new, pha_new, eps_r,
    eps_p)."""
    _, wa, w0, pa1, pb, pa2, p0 = model
    eps_r = 1e-2 * wa * bet + w0
    eps_p = 0.0
    new_pha = pha
    if not ldc:
        eps_p = pa1 * eps_r ** pb + 1e-2 * pa2 * abs(pha) + p0
        new_pha = pha + g_p * eps_p
    return bet + g_r * eps_r, new_pha, eps_r, eps_p


def _g14_4(x: float) -> str:
    """Fortran G14.4 for the noise records (4 significant digits)."""
    ax = abs(x)
    if ax != 0.0 and (ax < 0.1 or ax >= 1e4):
        m = f"{x:.3E}"
        mant, ex = m.split("E")
        # Fortran's 0.dddE+ee form
        v = float(mant) / 10.0
        e = int(ex) + 1
        return f"{v:.4f}E{e:+03d}".rjust(14)
    if ax == 0.0:
        d = 3
    else:
        d = 4 - (int(math.floor(math.log10(ax))) + 1)
    return (f"{x:.{max(d, 0)}f}" + "    ").rjust(14)


def write_records(exe_dir: str, strnr, vnr, recs, ldc: bool):
    """inv.mynoise_rho, inv.mynoise_pha and inv.mynoise_voltages
    (src/rdati.f90:113-125, 259-285): per datum the deviate, the error, the
    value before and after."""
    with open(os.path.join(exe_dir, "inv.mynoise_rho"), "w") as fr:
        fr.write("#  rnd_r\teps_r\t\tbet(old)\tbet(new)\n")
        for (g_r, _, eps_r, _, bet, _, nb, _) in recs:
            fr.write(" " + "".join(_g14_4(v) + " " for v in (g_r, eps_r, bet)) + _g14_4(nb) + "\n")
    if not ldc:
        with open(os.path.join(exe_dir, "inv.mynoise_pha"), "w") as fp:
            fp.write("#  rnd_p\teps_p\t\tpha(old)\tpha(new)\n")
            for (_, g_p, _, eps_p, _, pha, _, npha) in recs:
                fp.write(" " + "".join(_g14_4(v) + " " for v in (g_p, eps_p, pha)) + _g14_4(npha) + "\n")
    with open(os.path.join(exe_dir, "inv.mynoise_voltages"), "w") as fv:
        fv.write(f"{len(recs):12d}\n")
        for s, v, rec in zip(strnr, vnr, recs):
            fv.write(f" {int(s):11d} {int(v):11d}  {rec[6]!r}  {rec[7]!r}\n")
