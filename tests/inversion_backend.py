"""Test infrastructure: the CPU oracle as a backend of
titatest_gb300.inversion.Inversion, and a reader of the IT/UP rows of the
reference's inv.ctr (src/kont2.f90)."""
import os

import numpy as np

from conftest import GOLDEN

from oracle import oracle as O


class OracleBackend:
    """forward + src/bvolti.f90, src/bsensi.f90 and src/update.f90 by the
    oracle (complex128)."""

    def __init__(self, grid, survey, kwn, kwnwi, swrtr=1, lsink=False, nsink=0, ldc=False):
        self.P = O.Problem(grid, survey)
        self.grid, self.kwn, self.kwnwi = grid, kwn, kwnwi
        self.kw = dict(swrtr=swrtr, lsink=lsink, nsink=nsink)
        self.ldc = ldc
        self.P.set_dc(ldc)

    def forward(self, sigma):
        # DC: the real routines read DBLE(sigma) (src/kompadc.f90, src/bsendc.f90)
        self.sigma = np.array(sigma.real if self.ldc else sigma, np.complex128)
        try:
            self.kp = self.P.forward(self.sigma, self.kwn, self.kwnwi, **self.kw)
            hp = self.P.rtrafo(self.kp, self.kwnwi, self.kw["swrtr"])
            self.volt, sa = self.P.bvolt(hp, 2 if self.ldc else 1, None)
        except RuntimeError as e:  # "... errnr N" of the oracle, as the library's errors carry it
            from titatest_gb300.formats import CRError
            raise CRError(int(str(e).split()[-1]), str(e)) from e
        return sa

    def sensitivities(self):
        self.J = self.P.bsens(self.kp, self.kwn, self.kwnwi, self.sigma, self.volt, mode=1,
                              swrtr=self.kw["swrtr"])

    def update(self, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx, nachbar, lam, eps, ncgmax, step, par,
               phase_only=False, dc=False):
        _, dpar, _, _, ncg = O.update(self.J, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx=nx, nachbar=nachbar,
                                      maxnk=self.grid.maxnk, lam=lam, eps=eps, ncgmax=ncgmax, step=step, par=par,
                                      phase_only=phase_only, dc=dc)
        return dpar, ncg

    def mcm(self, wmatd, wdfak, ltri, smatm, nx, nachbar, lam, res, cov2):
        return O.mcm(self.J, wmatd, wdfak, ltri, smatm, nx=nx, nachbar=nachbar, maxnk=self.grid.maxnk, lam=lam,
                     res=res, cov2=cov2)

    def column_sums(self, wa, wb, wc):
        return O.column_sums(self.J, wa, wb, wc)

    def kfak(self):
        return self.P.bkfak()

    def jtj(self, wmatd, wdfak, phase_only):
        """|(J^H W J 1)_j| of src/blam0.f90 from the host Jacobian."""
        w = np.asarray(wmatd) * np.asarray(wdfak, np.float64)
        J = self.J.real if phase_only else self.J
        return np.abs(np.conj(J).T @ (w * (J @ np.ones(J.shape[1]))))


def golden_rows(case):
    """(kind, index, nrmsd, bdpar, lam, rough, ncg, step) of every IT/UP
    (and PIT/PUP) line of the case's inv.ctr; None where the line has no such
    column."""
    rows = []
    with open(os.path.join(GOLDEN, case, "inv.ctr")) as fh:
        for line in fh:
            t = line.split()
            if not t or t[0] not in ("IT", "UP", "PIT", "PUP"):
                continue
            if t[0].endswith("IT") and len(t) == 6:
                rows.append((t[0], int(t[1]), float(t[2]), None, None, None, None, None))
            elif t[0].endswith("IT"):
                rows.append((t[0], int(t[1]), float(t[2]), float(t[3]), float(t[4]), float(t[5]), int(t[6]),
                             float(t[10])))
            else:
                rows.append((t[0], int(t[1]), float(t[2]), float(t[3]), float(t[4]), float(t[5]), int(t[6]),
                             float(t[7])))
    return rows


def inversion_case(case):
    """(grid, survey, data, cfg, kwn, kwnwi) of a golden inversion case."""
    from titatest_gb300 import formats as F
    from titatest_gb300 import inversion as I
    d = os.path.join(GOLDEN, case)
    cfg = I.read_crtomo_cfg(os.path.join(d, "crtomo.cfg"))
    g = F.read_elem(os.path.join(d, "elem.dat"))
    enr = F.read_elec(os.path.join(d, "elec.dat"), g.sanz)
    data = I.read_data(os.path.join(d, "volt.dat"), cfg, len(enr))
    sv = F.Survey(enr=enr, strnr=data.strnr, vnr=data.vnr, strom=np.ones(len(data.strnr)))
    kwn, kwnwi = O.Problem(g, sv).rwaven()
    return g, sv, data, cfg, kwn, kwnwi


# Tolerances against the printed trace (4 significant digits, the step size
# 3).  A trial whose CG ran to its cap (ncg = ncgmax) is a fixed sequence of
# operations: all fields within a few 1e-3.  A trial whose CG stopped on its
# residual test (|r| <= 1e-4 |b|, src/cg_mod.f90) stops wherever rounding puts
# the residual below the bound, and the model it returns can move by the
# system's condition times 1e-4: misfit, roughness and model change within a
# few percent, lambda (set by the earlier misfits) within 1e-2, the CG count
# within 8 steps.  Kind, index and step length always agree.
TIGHT = dict(rms=3e-3, lam=3e-3, rough=5e-3, bdpar=1.5e-2, ncg=0)
LOOSE = dict(rms=5e-2, lam=1e-2, rough=5e-2, bdpar=1e-1, ncg=8)


def _close(x, ref, tol):
    """relative, or against the printed resolution where the trace prints 0"""
    if ref == 0.0:
        return abs(x) < 5e-4
    return abs(x / ref - 1) < tol


def golden_rows_robust(case):
    """The IT/UP lines of a robust inversion's inv.ctr (src/kont2.f90
    formats 100, 106, 110: an L1-ratio column before the step length):
    (kind, index, nrmsd, bdpar, lam, rough, ncg, step, l1rat)."""
    rows = []
    with open(os.path.join(GOLDEN, case, "inv.ctr")) as fh:
        for line in fh:
            t = line.split()
            if not t or t[0] not in ("IT", "UP"):
                continue
            # lines after robust was switched off (src/inv.f90:868) have no L1 column
            if t[0] == "IT" and len(t) in (6, 7):
                rows.append(("IT", int(t[1]), float(t[2]), None, None, None, None, None,
                             float(t[6]) if len(t) == 7 else None))
            elif t[0] == "IT":
                rows.append(("IT", int(t[1]), float(t[2]), float(t[3]), float(t[4]), float(t[5]), int(t[6]),
                             float(t[-1]), float(t[10]) if len(t) == 12 else None))
            else:
                rows.append(("UP", int(t[1]), float(t[2]), float(t[3]), float(t[4]), float(t[5]), int(t[6]),
                             float(t[-1]), float(t[7]) if len(t) == 9 else None))
    return rows


def compare_rows(gold, rows, ncgmax, skip=()):
    """skip: lines compared by kind, index and lambda only."""
    assert len(rows) >= len(gold), (len(rows), len(gold))
    for i, g in enumerate(gold):
        r = rows[i]
        if i in skip:
            assert (r.kind, r.index) == (g[0], g[1]) and abs(r.lam / g[4] - 1) < 1e-2, (i, g[0], g[1])
            continue
        if len(g) > 8 and g[8] is not None:  # robust: the L1 ratio, printed with 3 digits
            assert abs(r.l1rat / g[8] - 1) < 5e-3, (i, r.l1rat, g[8])
        where = (i, g[0], g[1])
        assert (r.kind, r.index) == (g[0], g[1]), where
        t = TIGHT if (g[6] is None or g[6] == ncgmax) else LOOSE
        assert abs(r.nrmsd / g[2] - 1) < t["rms"], (where, r.nrmsd, g[2])
        if g[3] is None:
            continue
        assert _close(r.bdpar, g[3], t["bdpar"]), (where, r.bdpar, g[3])
        assert _close(r.lam, g[4], t["lam"]), (where, r.lam, g[4])
        assert _close(r.rough, g[5], t["rough"]), (where, r.rough, g[5])
        assert abs(r.ncg - g[6]) <= t["ncg"], (where, r.ncg, g[6])
        assert r.step == g[7], (where, r.step, g[7])


def dc_problem(ldc):
    """The DC_Problem tomodir: (grid, survey, data, cfg, kwn, kwnwi) for the
    complex inversion (ldc False) or the DC one (crtomo_dc.cfg)."""
    from titatest_gb300 import inversion as I
    g, sv, data, cfg, kwn, kwnwi = inversion_case("dc_problem")
    if ldc:
        d = os.path.join(GOLDEN, "dc_problem")
        cfg = I.read_crtomo_cfg(os.path.join(d, "crtomo_dc.cfg"))
        data = I.read_data(os.path.join(d, "volt.dat"), cfg, sv.eanz)
    return g, sv, data, cfg, kwn, kwnwi


def golden_rows_file(case, name):
    """golden_rows of another inv.ctr of a case"""
    rows = []
    with open(os.path.join(GOLDEN, case, name)) as fh:
        for line in fh:
            t = line.split()
            if t and t[0] == "IT" and len(t) == 6:
                rows.append((t[0], int(t[1]), float(t[2]), float(t[3]), t[4], int(t[5])))
    return rows


def check_models(case, inv, log10_tol=5e-4, pha_tol_mrad=0.5, volt_tol=1e-3):
    """The accepted models against the reference's rhoNN.mag (log10 |rho|
    per element; the files print 9 digits), rhoNN.pha (phase of rho, mrad)
    and volt01.dat (|R| of the model after iteration 1) of the case.
    Measured: the oracle within 5e-5 in log10 and 0.05 mrad; the GPU within
    2.6e-4 and 0.28 mrad (phases up to 10 mrad on mixed_surf, where the
    phase data carry a 0.1 mrad error: a model difference five times below
    what the data resolve is the phase bound)."""
    from titatest_gb300 import inversion as I
    d = os.path.join(GOLDEN, case)
    checked = 0
    for nn in (1, 2):
        path = os.path.join(d, f"rho{nn:02d}.mag")
        if not os.path.exists(path):
            continue
        m = [mm for mm in inv.models if mm["it"] == nn][0]
        rho = 1.0 / m["sigma"]
        n, rms, x, y, lg = I.read_model_mag(path)
        assert n == len(rho)
        assert np.abs(np.log10(np.abs(rho)) - lg).max() < log10_tol, (case, nn)
        pha_path = os.path.join(d, f"rho{nn:02d}.pha")
        if os.path.exists(pha_path):
            _, _, _, _, ph = I.read_model_mag(pha_path)
            assert np.abs(1e3 * np.angle(rho) - ph).max() < pha_tol_mrad, (case, nn)
        checked += 1
    m1 = [mm for mm in inv.models if mm["it"] == 1][0]
    vals = np.loadtxt(os.path.join(d, "volt01.dat"), skiprows=1)
    ours = np.exp(-m1["sigmaa"].real)
    assert np.abs(ours / vals[:, 2] - 1).max() < volt_tol
    return checked


def check_uncertainty(inv, backend, tmpdir, rel=5e-3):
    """titatest_gb300.uncertainty.write_all against the reference's
    coverage and uncertainty files of minimal (mswitch 15; the reference
    files come from the 2014 build, whose headers differ, the columns not):
    ata, ata + lam R, cov and cov ata cov diagonals relative, the resolution
    diagonal against its largest entry, the coverage in log10."""
    from titatest_gb300 import uncertainty as U
    U.write_all(inv, backend, str(tmpdir))
    d = os.path.join(GOLDEN, "minimal")
    for name, nc, col, kind, tol in (("ata.diag", 2, 0, "rel", rel), ("ata_reg.diag", 2, 0, "rel", rel),
                                     ("cov1_m.diag", 3, 0, "rel", rel), ("cov2_m.diag", 3, 0, "rel", rel),
                                     ("ata.diag_fpi", 2, 0, "rel", rel), ("res_m.diag", 2, 0, "max", 1e-3),
                                     ("coverage.mag", 3, 2, "abs", 5e-3), ("coverage.mag_fpi", 3, 2, "abs", 5e-3)):
        a = U.read_columns(os.path.join(str(tmpdir), name), nc)[:, col]
        r = U.read_columns(os.path.join(d, name), nc)[:, col]
        assert a.shape == r.shape, name
        if kind == "rel":
            err = np.max(np.abs(a / r - 1))
        elif kind == "max":
            err = np.max(np.abs(a - r)) / np.max(np.abs(r))
        else:
            err = np.max(np.abs(a - r))
        assert err < tol, (name, err)


def diff_case():
    """The difference inversion of tests/golden/diff_dc: (grid, survey of the
    kept data, data with d0 / fm0, m0, cfg, kwn, kwnwi).  The wavenumbers
    come from all data (src/rall.f90 calls rwaven before it drops the data
    without a reference-state match)."""
    from titatest_gb300 import formats as F
    from titatest_gb300 import inversion as I
    d = os.path.join(GOLDEN, "diff_dc")
    cfg = I.read_crtomo_cfg(os.path.join(d, "crtomo.cfg"))
    g = F.read_elem(os.path.join(GOLDEN, "robust_dc", "elem.dat"))
    enr = F.read_elec(os.path.join(GOLDEN, "robust_dc", "elec.dat"), g.sanz)
    data = I.read_data(os.path.join(d, "volt.dat"), cfg, len(enr))
    sv_all = F.Survey(enr=enr, strnr=data.strnr, vnr=data.vnr, strom=np.ones(len(data.strnr)))
    kwn, kwnwi = O.Problem(g, sv_all).rwaven()
    data, m0 = I.read_difference(data, os.path.join(d, "d0.dat"), os.path.join(d, "fm0.dat"),
                                 os.path.join(d, "m0.mag"), g.elanz, cfg)
    sv = F.Survey(enr=enr, strnr=data.strnr, vnr=data.vnr, strom=np.ones(len(data.strnr)))
    return g, sv, data, m0, cfg, kwn, kwnwi
