"""The CPU oracle against the reference's own golden outputs.

The volt.dat goldens are written in real*4 (src/wdatm.f90:76), so they pin
the oracle to float32 precision; the CutMcK goldens are integer-exact."""
import os

import numpy as np
import pytest

from conftest import CUTMCK_CASES, GOLDEN, FORWARD_CASES, load_case

from oracle import oracle as O
from titatest_gb300 import formats as F

# measured pin of each case (two reference builds of the same inputs differ by
# 3.7e-5, so only the cases written by a current build are pinned this tight)
PIN = {"minimal": 1e-7, "testmodinv": 1e-7, "mixed_surf": 1e-6, "decoupling_2d_sink": 1e-7}


@pytest.mark.parametrize("case", FORWARD_CASES)
def test_oracle_reproduces_reference_volt(case):
    g, sv, sig, cfg, (bet, pha) = load_case(case)
    P = O.Problem(g, sv)
    if cfg.swrtr:
        kwn, kwnwi = P.rwaven()
    else:
        kwn, kwnwi = np.zeros(1), np.zeros(1)
    kpot = P.forward(sig, kwn, kwnwi, swrtr=cfg.swrtr, lsr=cfg.lsr, lsink=cfg.lsink, nsink=cfg.nsink)
    hpot = P.rtrafo(kpot, kwnwi, cfg.swrtr)
    volt, sigmaa = P.bvolt(hpot, 0, None)
    b2, p2, v2 = F.volt_record(sigmaa, sv.strnr, sv.vnr)
    assert np.array_equal(v2, sv.vnr), "polarity of the golden measurements must match"
    rel = np.abs(b2 - bet) / np.abs(bet)
    assert rel.max() < PIN[case], rel.max()
    assert np.abs(p2 - pha).max() < 1e-3  # mrad


@pytest.mark.parametrize("case", CUTMCK_CASES)
def test_oracle_cutmck_is_integer_exact(case):
    d = os.path.join(GOLDEN, "cutmck_" + case)
    g0 = F.read_elem(os.path.join(d, "elem.dat.orig"), fix_borders=False)
    e0 = F.read_elec(os.path.join(d, "elec.dat.orig"))
    g1 = F.read_elem(os.path.join(d, "elem.dat"), fix_borders=False)
    e1 = F.read_elec(os.path.join(d, "elec.dat"))
    g2, e2 = O.cutmck(g0, e0)
    assert g2.mb == g1.mb
    assert np.array_equal(g2.snr, g1.snr)
    assert np.array_equal(g2.nrel, g1.nrel)
    assert np.array_equal(e2, e1)


def test_oracle_homogeneous_halfspace_matches_analytic():
    """Second oracle (src/potana.f90): on a homogeneous half-space the FE
    potentials approach the analytic K0 solution away from the source."""
    from titatest_gb300 import synth
    s = synth.config1()
    sig = np.full(s.grid.elanz, 0.01 + 0j)
    P = O.Problem(s.grid, s.survey)
    kwn, kwnwi = P.rwaven()
    kp = P.forward(sig, kwn, kwnwi)
    s0 = P.refsig(sig)
    assert abs(s0 - 0.01) < 1e-12
    x, y = s.grid.node_xy()
    l = 10
    src = s.survey.enr[l - 1] - 1
    for k in (2, 5):
        pa = P.potana(l, kwn[k], s0)
        r = np.hypot(x - x[src], y - y[src])
        far = (r > 3.0) & (r < 12.0)
        rel = np.abs(kp[k, l - 1, far] - pa[far]) / np.abs(pa[far])
        assert np.median(rel) < 0.05


def test_oracle_bessel_tables():
    """A&S 9.8 approximations against scipy's exact K0/K1 (they are accurate
    to ~1e-7 relative, which is the point: parity needs the tables)."""
    sp = pytest.importorskip("scipy.special")
    L = O.lib()
    for x in (0.01, 0.5, 1.9, 2.0, 2.1, 7.0, 40.0):
        assert abs(L.or_bessk0(x) - sp.k0(x)) <= 2e-7 * sp.k0(x) + 1e-300
        assert abs(L.or_bessk1(x) - sp.k1(x)) <= 2e-7 * sp.k1(x) + 1e-300
    assert L.or_bessk0(600.0) == 0.0


def _valued_nodes(g, sv, count, seed, exclude=()):
    rng = np.random.default_rng(seed)
    skip = set(int(e) for e in sv.enr) | set(int(x) for x in exclude)
    pool = [i for i in range(1, g.sanz + 1) if i not in skip]
    return np.sort(rng.choice(pool, size=count, replace=False)).astype(np.int32)


def test_oracle_randb2_keeps_a_system_that_satisfies_its_values():
    """src/randb2.f90 restated: prescribing at some nodes the potential that
    system (k0, 1) has there leaves that system's potential unchanged, and
    every system assembled by kompab (all of them with mixed boundaries)
    returns exactly the prescribed value at those nodes."""
    g, sv, sig, cfg, _ = load_case("minimal")
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    kp = P.forward(sig, kwn, kwnwi)
    nodes = _valued_nodes(g, sv, 12, seed=3)
    k0 = 2
    vals = kp[k0, 0, nodes - 1].copy()
    P.set_boundary_values(nodes, vals)
    kp2 = P.forward(sig, kwn, kwnwi)
    assert np.max(np.abs(kp2[k0, 0] - kp[k0, 0])) < 1e-9 * np.max(np.abs(kp[k0, 0]))
    assert np.array_equal(kp2[:, :, nodes - 1], np.broadcast_to(vals, kp2[:, :, nodes - 1].shape))
    assert np.max(np.abs(kp2[k0 + 1, 1] - kp[k0 + 1, 1])) > 1e-6 * np.max(np.abs(kp[k0 + 1, 1]))


def test_oracle_randb2_values_only_in_kompab_systems():
    """Without mixed boundaries one factor per wavenumber serves all
    electrodes: electrode 1's system is assembled by kompab (values applied),
    the others' right-hand sides by kompb, which leaves the values out, so
    their potential is 0 at the valued nodes (src/fem.f90:355-376)."""
    g, sv, sig, cfg, _ = load_case("decoupling_2d_sink")
    P = O.Problem(g, sv)
    kwn, kwnwi = np.zeros(1), np.zeros(1)
    nodes = _valued_nodes(g, sv, 8, seed=4, exclude=[cfg.nsink])
    vals = np.linspace(0.5, 2.0, len(nodes)) * (1 - 0.1j)
    P.set_boundary_values(nodes, vals)
    kp = P.forward(sig, kwn, kwnwi, swrtr=0, lsink=cfg.lsink, nsink=cfg.nsink)
    assert np.array_equal(kp[0, 0, nodes - 1], vals)
    assert np.all(kp[0, 1:, nodes - 1] == 0)
    assert np.all(np.isfinite(kp))


def test_oracle_randb2_node_out_of_range_is_error_30():
    g, sv, sig, cfg, _ = load_case("minimal")
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    P.set_boundary_values([g.sanz + 1], [1.0])
    with pytest.raises(RuntimeError, match="errnr 30"):
        P.forward(sig, kwn, kwnwi)
