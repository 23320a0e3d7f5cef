"""Coverage, model uncertainty and resolution after a CRTomo inversion.

src/bbsens.f90 (coverage.mag) and src/bmcm_mod.f90 buncert (ata.diag,
ata_reg.diag, cov1_m.diag, res_m.diag, cov2_m.diag), chosen by mswitch as
src/rall.f90:528-541 does: +2 MCM 1, +4 resolution, +8 MCM 2 (each implying
the ones before it); the coverage is always written.  The sums and the
dense algebra run on the backend (DeviceBackend: crgpu_column_sums and
crgpu_mcm on the sensitivities left on the device by the last model); this
module picks the weights and lambda of the reference and writes the files.
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import formats
from . import fortran_io as FIO
from . import regularization as R

f4 = formats.f4


r8, i4, ch, rec = FIO.real8, FIO.int4, FIO.char, FIO.record  # list-directed items, as gfortran writes them


def weights(inv):
    """(w_mcm, w_cov, w_cov_fpi): the data weights buncert uses
    (src/bmcm_mod.f90:84-93) and those of the coverage (src/bbsens.f90:40-52)."""
    cfg, d = inv.cfg, inv.data
    lelerr = (not cfg.lfphai and not cfg.ldc) or bool(cfg.mswitch & 32)
    wd = np.asarray(inv.wdfak, np.float64)
    if lelerr:
        w_mcm = d.wmatd_cri
    elif inv.lfpi:
        w_mcm = d.wmatdr
    else:
        w_mcm = inv.wmatd
    if inv.lfpi:
        w_cov = (d.wmatd_cri if lelerr else d.wmatdr)
        w_fpi = inv.wmatd
    else:
        w_cov = inv.wmatd
        w_fpi = inv.wmatd
    return np.asarray(w_mcm, np.float64), np.sqrt(w_cov) * wd, np.sqrt(w_fpi) * wd


def coverage(inv, backend, ramd: str):
    """src/bbsens.f90: coverage.mag (x, y, log10(c_j / max c)) with c_j =
    sum_i |J_ij| sqrt(w_i) wdfak_i; in the final phase improvement also
    coverage.mag_fpi from |Re J|.  Returns (c, c_fpi)."""
    _, wa, wb = weights(inv)
    c1, c2, _ = backend.column_sums(wa, wb, np.zeros_like(wa))
    cx, cy = R._centroids(inv.grid)
    os.makedirs(ramd, exist_ok=True)
    cmax = float(np.max(c1))
    with open(os.path.join(ramd, "coverage.mag"), "w") as fh:
        fh.write(rec([i4(len(c1)), r8(cmax)]))
        fh.write("".join(rec([r8(cx[j]), r8(cy[j]), r8(math.log10(c1[j] / cmax))]) for j in range(len(c1))))
    if inv.lfpi:
        fmax = float(np.max(c2))
        with open(os.path.join(ramd, "coverage.mag_fpi"), "w") as fh:
            fh.write(rec([i4(len(c2))]))
            fh.write("".join(rec([r8(cx[j]), r8(cy[j]), r8(math.log10(c2[j] / fmax))]) for j in range(len(c2))))
            fh.write(rec([ch("Max:"), r8(fmax)]))
    return c1, c2


def buncert(inv, backend, ramd: str, res: bool = True, cov2: bool = True) -> dict:
    """src/bmcm_mod.f90 buncert: lambda of the complex stage after a final
    phase improvement (lam_cri), else the last good lambda; the diagonals of
    ata, ata + lam R, cov = (ata + lam R)^-1, cov ata and cov ata cov, and
    their files.  Returns the diagonals and lambda."""
    cfg = inv.cfg
    lam = inv.lam_cri if inv.lfpi else inv.lamalt
    w_mcm, _, _ = weights(inv)
    out = backend.mcm(w_mcm, inv.wdfak, cfg.ltri, inv.smatm, cfg.nx, inv.nachbar, lam, res, cov2)
    out["lam"] = lam
    sigma = inv.sigma
    os.makedirs(ramd, exist_ok=True)
    n = len(out["ata"])
    d = out["ata"]
    with open(os.path.join(ramd, "ata.diag"), "w") as fh:  # bata
        fh.write(rec([i4(n), r8(d.min()), r8(d.max())]))
        fh.write("".join(rec([r8(v), r8(math.log10(v) - math.log10(d.max()))]) for v in d))
    if inv.lfpi:  # bata: the FPI diagonal sum_i Re(J_ij)^2 wmatdp_i wdfak_i
        _, _, dfpi = backend.column_sums(np.zeros(len(w_mcm)), np.zeros(len(w_mcm)),
                                         inv.data.wmatdp * np.asarray(inv.wdfak, np.float64))
        out["ata_fpi"] = dfpi
        with open(os.path.join(ramd, "ata.diag_fpi"), "w") as fh:
            fh.write(rec([i4(n)]))
            fh.write("".join(rec([r8(v), r8(math.log10(v) - math.log10(dfpi.max()))]) for v in dfpi))
            fh.write(rec([ch("Max/Min:"), r8(dfpi.max()), ch("/"), r8(dfpi.min())]))
    d = out["reg"]
    with open(os.path.join(ramd, "ata_reg.diag"), "w") as fh:  # bata_reg
        fh.write(rec([i4(n), r8(lam)]))
        fh.write("".join(rec([r8(v), r8(math.log10(v))]) for v in d))
        fh.write(rec([ch("Max/Min:"), r8(d.max()), ch("/"), r8(d.min())]))

    def mcm_file(name, dg):  # bmcm, bmcm2
        with open(os.path.join(ramd, name), "w") as fh:
            fh.write(rec([i4(n), r8(lam)]))
            for j in range(n):
                r = math.sqrt(dg[j])
                fh.write(rec([r8(r * 1e2), r8(sigma[j].real * r), r8(sigma[j].imag * r)]))
            fh.write(rec([ch("Max/Min:"), r8(dg.max()), ch("/"), r8(dg.min())]))

    mcm_file("cov1_m.diag", out["cov1"])
    if res:
        d = out["res"]
        with open(os.path.join(ramd, "res_m.diag"), "w") as fh:  # bres
            fh.write(rec([i4(n), r8(lam), r8(d.min()), r8(d.max())]))
            fh.write("".join(rec([r8(abs(v)), r8(math.log10(abs(v)) - math.log10(d.max()))]) for v in d))
        if cov2:
            mcm_file("cov2_m.diag", out["cov2"])
    return out


def read_columns(path: str, ncol: int):
    """The numeric lines of a .diag / coverage file (header and Max/Min lines
    skipped): array (n, ncol)."""
    rows = []
    with open(path) as fh:
        fh.readline()
        for line in fh:
            t = line.split()
            if len(t) < ncol:
                continue
            try:
                rows.append([float(x) for x in t[:ncol]])
            except ValueError:
                continue
    return np.array(rows)


def write_all(inv, backend, ramd: str):
    """What CRTomo writes after the inversion (src/inv.f90:1050-1065) for
    the run's mswitch: the coverage always, the MCM files by bits 1-3."""
    m = inv.cfg.mswitch
    lcov2 = bool(m & 8)
    lres = bool(m & 4) or lcov2
    lcov1 = bool(m & 2) or lres
    coverage(inv, backend, ramd)
    if lcov1:
        return buncert(inv, backend, ramd, res=lres, cov2=lcov2)
    return None
