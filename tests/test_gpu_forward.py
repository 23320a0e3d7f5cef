"""GPU parity: the CUDA forward, factor and sensitivities against the oracle.

Tolerances (relative, max-norm over the array):
  plain complex128 mode : 1e-10 for kpot, volt, sensitivities
  mixed complex64+refinement : 1e-6 voltages, 1e-5 sensitivities
"""
import numpy as np
import pytest

from conftest import FORWARD_CASES, load_case, relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-10
MIXED_VOLT_TOL = 1e-6
MIXED_SENS_TOL = 1e-5


def _oracle_forward(g, sv, sig, cfg_swrtr=1, lsink=False, nsink=0):
    P = O.Problem(g, sv)
    if cfg_swrtr:
        kwn, kwnwi = P.rwaven()
    else:
        kwn, kwnwi = np.zeros(1), np.zeros(1)
    kp = P.forward(sig, kwn, kwnwi, swrtr=cfg_swrtr, lsink=lsink, nsink=nsink)
    hp = P.rtrafo(kp, kwnwi, cfg_swrtr)
    volt, sigmaa = P.bvolt(hp, 0, None)
    return P, kwn, kwnwi, kp, hp, volt


@pytest.mark.parametrize("case", FORWARD_CASES)
def test_plain_forward_matches_oracle(gpu_lib, case):
    from titatest_gb300 import PLAIN, CRMod
    g, sv, sig, cfg, _ = load_case(case)
    P, kwn, kwnwi, kp, hp, volt = _oracle_forward(g, sv, sig, cfg.swrtr, cfg.lsink, cfg.nsink)
    with CRMod(g, sv, kwn, kwnwi, swrtr=cfg.swrtr, lsink=cfg.lsink, nsink=cfg.nsink,
               precision=PLAIN) as m:
        out = m.forward(sig, kpot=True, hpot=True)
    gk, gh = out["kpot"], out["hpot"]
    if cfg.swrtr == 0 and not (g.typ == 11).any():
        # 2D with no-flow boundaries only: the system is singular and each
        # potential is fixed only up to a rounding-dependent constant (the
        # reference's too); compare differences to node 1
        gk, kp = gk - gk[..., :1], kp - kp[..., :1]
        gh, hp = gh - gh[..., :1], hp - hp[..., :1]
        tol = 1e-8
    else:
        tol = PLAIN_TOL
    assert relerr(gk, kp) < tol
    assert relerr(gh, hp) < tol
    assert relerr(out["volt"], volt) < tol


@pytest.mark.parametrize("case", ["minimal", "testmodinv"])
def test_plain_factor_matches_oracle_chol(gpu_lib, case):
    from titatest_gb300 import PLAIN, CRMod
    g, sv, sig, cfg, _ = load_case(case)
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN) as m:
        for k, l in [(1, 1), (len(kwn), sv.eanz), (3, 5)]:
            a_ref, fak_ref = P.factor(sig, kwn, k, l)
            a, fak = m.factor_system(sig, k, l)
            np.testing.assert_allclose(fak, fak_ref, rtol=1e-14)
            # entries outside the band start (columns < 1) are unused in both
            for i in range(g.sanz):
                lo = max(0, g.mb - i)
                assert relerr(a[i, lo:], a_ref[i, lo:]) < 1e-11 or np.max(np.abs(a_ref[i, lo:])) < 1e-300


@pytest.mark.parametrize("case", ["minimal", "testmodinv", "mixed_surf"])
def test_mixed_forward_matches_oracle(gpu_lib, case):
    from titatest_gb300 import MIXED, CRMod
    g, sv, sig, cfg, _ = load_case(case)
    P, kwn, kwnwi, kp, hp, volt = _oracle_forward(g, sv, sig)
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED) as m:
        out = m.forward(sig, kpot=True)
        st = m.stats()
    assert relerr(out["volt"], volt) < MIXED_VOLT_TOL
    assert relerr(out["kpot"], kp) < 1e-6
    assert st["refine_iterations"] >= 1


@pytest.fixture(scope="module")
def cfg1():
    from titatest_gb300 import synth
    s = synth.config1()
    P, kwn, kwnwi, kp, hp, volt = _oracle_forward(s.grid, s.survey, s.sigma)
    sens0 = P.bsens(kp, kwn, kwnwi, s.sigma, volt, mode=0)
    sens1 = P.bsens(kp, kwn, kwnwi, s.sigma, volt, mode=1)
    return s, kwn, kwnwi, kp, volt, sens0, sens1


def test_cfg1_plain_forward_and_sensitivities(gpu_lib, cfg1):
    from titatest_gb300 import PLAIN, CRMod
    s, kwn, kwnwi, kp, volt, sens0, sens1 = cfg1
    with CRMod(s.grid, s.survey, kwn, kwnwi, precision=PLAIN) as m:
        out = m.forward(s.sigma, kpot=True)
        assert relerr(out["kpot"], kp) < PLAIN_TOL
        assert relerr(out["volt"], volt) < PLAIN_TOL
        J0 = m.bsens()
        assert relerr(J0, sens0) < PLAIN_TOL
        J1 = m.bsensi()
        assert relerr(J1, sens1) < PLAIN_TOL


def test_cfg1_mixed_forward_and_sensitivities(gpu_lib, cfg1):
    from titatest_gb300 import MIXED, CRMod
    s, kwn, kwnwi, kp, volt, sens0, sens1 = cfg1
    with CRMod(s.grid, s.survey, kwn, kwnwi, precision=MIXED) as m:
        out = m.forward(s.sigma)
        assert relerr(out["volt"], volt) < MIXED_VOLT_TOL
        assert relerr(m.bsens(), sens0) < MIXED_SENS_TOL
        assert relerr(m.bsensi(), sens1) < MIXED_SENS_TOL


def test_volt_matches_reference_golden(gpu_lib):
    """End to end against the reference's own CRMod output (real*4)."""
    from titatest_gb300 import PLAIN, CRMod
    from titatest_gb300 import formats as F
    g, sv, sig, cfg, (bet, pha) = load_case("testmodinv")
    with CRMod(g, sv, precision=PLAIN) as m:
        out = m.forward(sig)
    b2, p2, v2 = F.volt_record(out["sigmaa"], sv.strnr, sv.vnr)
    assert np.array_equal(v2, sv.vnr)
    assert (np.abs(b2 - bet) / np.abs(bet)).max() < 1e-7
    assert np.abs(p2 - pha).max() < 1e-3


def test_zero_conductivity_raises_reference_error(gpu_lib):
    """A zero diagonal (all-zero sigma) reports src/scalab.f90's error 27."""
    from titatest_gb300 import PLAIN, CRMod
    from titatest_gb300._lib import CRGPUError
    g, sv, sig, cfg, _ = load_case("minimal")
    with CRMod(g, sv, precision=PLAIN) as m:
        with pytest.raises(CRGPUError) as ei:
            m.forward(np.zeros_like(sig))
        assert ei.value.errnr == 27
        out = m.forward(sig)  # context still usable
        assert np.all(np.isfinite(out["volt"]))


@pytest.mark.parametrize("prec", [0, 1])
def test_singularity_removal_matches_oracle(gpu_lib, cfg1, prec):
    """mswitch bit 2: src/refsig.f90 + src/potana.f90 + the lsr branch of
    src/kompab.f90 and kpot += pota (src/fem.f90:390-391)."""
    from titatest_gb300 import CRMod
    s, kwn, kwnwi, *_ = cfg1
    P = O.Problem(s.grid, s.survey)
    kp = P.forward(s.sigma, kwn, kwnwi, lsr=True)
    hp = P.rtrafo(kp, kwnwi)
    volt, _ = P.bvolt(hp, 0, None)
    with CRMod(s.grid, s.survey, kwn, kwnwi, precision=prec, lsr=True) as m:
        out = m.forward(s.sigma, kpot=True)
    tol = PLAIN_TOL if prec == 0 else MIXED_VOLT_TOL
    assert relerr(out["kpot"], kp) < (PLAIN_TOL if prec == 0 else 1e-6)
    assert relerr(out["volt"], volt) < tol


def test_singularity_removal_homogeneous_is_analytic(gpu_lib):
    """With a homogeneous model sigma - sigma0 = 0, the removal right-hand side
    vanishes and kpot is the analytic half-space field of src/potana.f90."""
    from titatest_gb300 import PLAIN, CRMod
    g, sv, sig, cfg, _ = load_case("minimal")
    sig = np.full_like(sig, 0.01 + 0.001j)
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN, lsr=True) as m:
        out = m.forward(sig, kpot=True)
    s0 = P.refsig(sig)
    for k in (0, len(kwn) - 1):
        for l in (1, sv.eanz):
            pa = P.potana(l, kwn[k], s0)
            assert relerr(out["kpot"][k, l - 1], pa) < 1e-12


def _wide_band_case(nx=190, nz=6, ne=16, seed=17):
    """A strip in its natural numbering (x fastest): band width nx + 2 at
    only (nx+1)(nz+1) nodes, beyond the register-window kernels."""
    from titatest_gb300 import formats, synth
    xs = np.arange(nx + 1, dtype=float)
    depths = np.arange(nz + 1, dtype=float)
    grid, surface, X, Y = synth._quad_grid(xs, depths)
    area = grid.nrel[: grid.nelanz[0]]
    grid.mb = int((area.max(axis=1) - area.min(axis=1)).max())
    enr = surface[np.linspace(10, nx - 10, ne).astype(int)]
    s, v = synth._encode(synth.dipole_dipole(ne, [1], [1, 2, 3]))
    survey = formats.Survey(enr=enr, strnr=s, vnr=v, strom=np.ones(len(s)))
    mag, pha = synth.random_model(grid, np.random.default_rng(seed))
    return grid, survey, synth._sigma_from(mag, pha)


def test_tensor_core_factor_matches_oracle_chol(gpu_lib):
    """The complex64 tensor-core factor read back through crgpu_factor_system
    (its band rows copied out of the batch buffer), against the oracle's chol
    rows."""
    from titatest_gb300 import MIXED, CRMod
    g, sv, sig, cfg, _ = load_case("testmodinv")
    assert g.mb + 4 <= 128
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED, band_order=0) as m:  # the grid's own band
        m.set_tune(1)  # tensor cores
        for k, l in [(1, 1), (len(kwn), sv.eanz)]:
            a_ref, fak_ref = P.factor(sig, kwn, k, l)
            a, fak = m.factor_system(sig, k, l)
            np.testing.assert_allclose(fak, fak_ref, rtol=1e-14)
            for i in range(g.sanz):
                lo = max(0, g.mb - i)
                assert relerr(a[i, lo:], a_ref[i, lo:]) < 1e-3, (k, l, i)


def _strip_case(nx, nz, ne, seed=23):
    """A strip of nx x nz quads in its natural numbering (x fastest): band
    width nx + 2, (nx+1)(nz+1) nodes, ne surface electrodes."""
    from titatest_gb300 import formats, synth
    grid, surface, X, Y = synth._quad_grid(np.arange(nx + 1, dtype=float), np.arange(nz + 1, dtype=float))
    area = grid.nrel[: grid.nelanz[0]]
    grid.mb = int((area.max(axis=1) - area.min(axis=1)).max())
    enr = surface[np.linspace(0, nx, ne).astype(int)]
    s, v = synth._encode(synth.dipole_dipole(ne, [1], [1, 2]))
    survey = formats.Survey(enr=enr, strnr=s, vnr=v, strom=np.ones(len(s)))
    mag, pha = synth.random_model(grid, np.random.default_rng(seed))
    return grid, survey, synth._sigma_from(mag, pha)


@pytest.mark.parametrize("nx,nz", [(5, 4), (20, 6), (60, 2), (61, 3)])
def test_warp_factor_matches_oracle_chol(gpu_lib, nx, nz):
    """The one-warp-per-system complex64 factor (window in registers) against
    the oracle's chol rows and, through refinement, the complex128 forward:
    fewer nodes than the window (30), odd node counts that are not a multiple
    of the 8-column block (147, 183), the widest band of the two-column step
    (mb = 62) and the widest band of the kernel (mb = 63, one column a step)."""
    from titatest_gb300 import MIXED, PLAIN, CRMod
    g, sv, sig = _strip_case(nx, nz, ne=min(nx + 1, 8))
    assert g.mb == nx + 2 and g.mb <= 63
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED, band_order=0) as m:
        m.set_tune(4)
        assert m.tune()["factor"] == "SIMT warp per system"
        for k, l in [(1, 1), (len(kwn), sv.eanz)]:
            a_ref, fak_ref = P.factor(sig, kwn, k, l)
            a, fak = m.factor_system(sig, k, l)
            np.testing.assert_allclose(fak, fak_ref, rtol=1e-14)
            for i in range(g.sanz):
                lo = max(0, g.mb - i)
                assert relerr(a[i, lo:], a_ref[i, lo:]) < 1e-3, (k, l, i)
        m.set_refinement(10, 1e-10)
        om = m.forward(sig, kpot=True)
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN) as m:
        op = m.forward(sig, kpot=True)
    assert relerr(om["kpot"], op["kpot"]) < MIXED_VOLT_TOL
    assert relerr(om["volt"], op["volt"]) < MIXED_VOLT_TOL


def test_wide_band_mixed_factor_shared_memory_window(gpu_lib):
    """mb = 192: the complex64 factor with its window in shared memory, against
    the oracle's factor and, through refinement, the complex128 forward."""
    from titatest_gb300 import MIXED, PLAIN, CRMod
    g, sv, sig = _wide_band_case()
    assert 176 <= g.mb + 1 <= 208
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    a_ref, fak_ref = P.factor(sig, kwn, 1, 1)
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED, band_order=0) as m:  # the grid's own band
        a, fak = m.factor_system(sig, 1, 1)
        m.set_refinement(10, 1e-10)
        vm = m.forward(sig)["volt"]
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN) as m:
        vp = m.forward(sig)["volt"]
    for i in range(g.sanz):
        lo = max(0, g.mb - i)
        assert relerr(a[i, lo:], a_ref[i, lo:]) < 1e-3, i
    assert relerr(vm, vp) < MIXED_VOLT_TOL


def test_run_tomodir_writes_crmod_outputs(gpu_lib, tmp_path):
    """CRMod on a tomodir (crmod.run_tomodir): volt.dat against the reference's
    golden, and with potentials and sensitivities switched on, one pot and one
    sens file per measurement (src/bpot.f90, src/wpot.f90, src/wsens.f90)."""
    import os
    import shutil

    from conftest import GOLDEN
    from titatest_gb300 import PLAIN
    from titatest_gb300 import formats as F
    from titatest_gb300.crmod import run_tomodir
    src = os.path.join(GOLDEN, "minimal")
    for sub in ("exe", "grid", "rho", "config", "mod"):
        os.makedirs(tmp_path / sub)
    shutil.copyfile(os.path.join(src, "elem.dat"), tmp_path / "grid" / "elem.dat")
    shutil.copyfile(os.path.join(src, "elec.dat"), tmp_path / "grid" / "elec.dat")
    shutil.copyfile(os.path.join(src, "rho.dat"), tmp_path / "rho" / "rho.dat")
    s, v, bet, pha = F.read_volt(os.path.join(src, "volt.dat"))
    F.write_config(str(tmp_path / "config" / "config.dat"), s, v)
    cfg = open(os.path.join(src, "crmod.cfg")).read().splitlines()
    cfg[5] = "T                ! potentials ?"
    cfg[9] = "T               ! sensitivities ?"
    (tmp_path / "exe" / "crmod.cfg").write_text("\n".join(cfg) + "\n")
    out = run_tomodir(str(tmp_path / "exe"), precision=PLAIN)
    s2, v2, bet2, pha2 = F.read_volt(str(tmp_path / "mod" / "volt.dat"))
    assert np.array_equal(s2, s) and np.array_equal(v2, v)
    assert np.max(np.abs(bet2 / bet - 1)) < 1e-6  # real*4 files on both sides
    pots = sorted(os.listdir(tmp_path / "mod" / "pot"))
    sens = sorted(os.listdir(tmp_path / "mod" / "sens"))
    assert len(pots) == len(sens) == len(s) and pots[0] == "pot01.dat" and sens[-1] == "sens12.dat"
    J = out["sens"]
    body = np.loadtxt(tmp_path / "mod" / "sens" / "sens12.dat", skiprows=1)
    assert np.allclose(body[:, 2] + 1j * body[:, 3], J[11], rtol=1e-6, atol=1e-7 * np.abs(J[11]).max())


def test_wide_band_mixed_in_geometric_order(gpu_lib):
    """The same mb = 192 strip with the default band order: the complex64
    factor runs on the tensor cores in the nodes' geometric order (band 8);
    potentials, voltages and sensitivities come back in the grid's order and
    equal the complex128 path's."""
    from titatest_gb300 import MIXED, PLAIN, CRMod
    from titatest_gb300._lib import CRGPUError
    g, sv, sig = _wide_band_case()
    kwn, kwnwi = O.Problem(g, sv).rwaven()
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN) as m:
        op = m.forward(sig, kpot=True, hpot=True)
        Jp = m.bsens()
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED) as m:
        m.set_refinement(10, 1e-10)
        order = m.node_order()
        assert sorted(order.tolist()) == list(range(1, g.sanz + 1)) and np.any(order != np.arange(1, g.sanz + 1))
        om = m.forward(sig, kpot=True, hpot=True)
        Jm = m.bsens()
        with pytest.raises(CRGPUError):
            m.factor_system(sig, 1, 1)
    assert relerr(om["kpot"], op["kpot"]) < MIXED_VOLT_TOL
    assert relerr(om["hpot"], op["hpot"]) < MIXED_VOLT_TOL
    assert relerr(om["volt"], op["volt"]) < MIXED_VOLT_TOL
    assert relerr(Jm, Jp) < MIXED_SENS_TOL
