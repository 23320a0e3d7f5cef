"""Host-side logic of the product that needs no GPU: file formats, the
Cuthill-McKee renumbering and the wavenumber rule, and the C ABI exports."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import CUTMCK_CASES, GOLDEN, ROOT, load_case

from titatest_gb300 import formats as F


@pytest.fixture(scope="module")
def built():
    from titatest_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    hdr = open(os.path.join(ROOT, "include", "crtomo_gb300.h")).read()
    names = sorted(set(re.findall(r"\b(crgpu_[a-z_]+)\s*\(", hdr)))
    assert len(names) >= 16
    for n in names:
        assert hasattr(lib, n), n


@pytest.mark.parametrize("case", CUTMCK_CASES)
def test_product_cutmck_is_integer_exact(built, case):
    from titatest_gb300 import cutmck
    d = os.path.join(GOLDEN, "cutmck_" + case)
    g0 = F.read_elem(os.path.join(d, "elem.dat.orig"), fix_borders=False)
    e0 = F.read_elec(os.path.join(d, "elec.dat.orig"))
    g1 = F.read_elem(os.path.join(d, "elem.dat"), fix_borders=False)
    e1 = F.read_elec(os.path.join(d, "elec.dat"))
    g2, e2 = cutmck(g0, e0)
    assert (g2.mb, g2.snr.tolist(), g2.nrel.tolist(), e2.tolist()) == \
        (g1.mb, g1.snr.tolist(), g1.nrel.tolist(), e1.tolist())


@pytest.mark.parametrize("case", ["minimal", "testmodinv", "mixed_surf"])
def test_product_rwaven_matches_oracle(built, case):
    from oracle import oracle as O
    from titatest_gb300 import rwaven
    g, sv, *_ = load_case(case)
    k1, w1 = rwaven(g, sv)
    k2, w2 = O.Problem(g, sv).rwaven()
    assert len(k1) == len(k2)
    np.testing.assert_allclose(k1, k2, rtol=1e-13, atol=0)
    np.testing.assert_allclose(w1, w2, rtol=1e-13, atol=0)


def test_rwaven_duplicate_electrodes_error(built):
    from titatest_gb300 import rwaven
    from titatest_gb300._lib import CRGPUError
    g, sv, *_ = load_case("minimal")
    enr = sv.enr.copy()
    enr[1] = enr[0]  # electrodes 1 and 2 on the same node
    bad = F.Survey(enr=enr, strnr=np.array([10002], np.int32), vnr=np.array([30004], np.int32),
                   strom=np.ones(1))
    bad.strnr[0] = 1 * 10000 + 3
    bad.vnr[0] = 2 * 10000 + 4
    with pytest.raises(CRGPUError) as ei:
        rwaven(g, F.Survey(enr=enr, strnr=np.array([20003], np.int32), vnr=np.array([10004], np.int32),
                           strom=np.ones(1)))
    assert ei.value.errnr == 73


def test_elem_write_read_roundtrip(tmp_path):
    g, *_ = load_case("minimal")
    p = tmp_path / "elem.dat"
    F.write_elem(str(p), g)
    g2 = F.read_elem(str(p))
    assert g2.mb == g.mb and np.array_equal(g2.nrel, g.nrel) and np.array_equal(g2.rnr, g.rnr)
    assert np.allclose(g2.sx, g.sx, atol=1e-3) and np.allclose(g2.sy, g.sy, atol=1e-3)


def test_config_formats(tmp_path):
    p = tmp_path / "config.dat"
    p.write_text("2\n1 2 3 4\n2 3 4 5\n")
    s, v, _ = F.read_config(str(p), 5)
    assert s.tolist() == [10002, 20003] and v.tolist() == [30004, 40005]
    F.write_config(str(p), s, v)
    s2, v2, _ = F.read_config(str(p), 5)
    assert s2.tolist() == s.tolist() and v2.tolist() == v.tolist()
    p.write_text("1\n1 1 3 4\n")
    with pytest.raises(F.CRError) as ei:
        F.read_config(str(p), 5)
    assert ei.value.errnr == 73


def test_rho_reader_phase_convention(tmp_path):
    p = tmp_path / "rho.dat"
    p.write_text("2\n100.0 -10.0\n10.0 0.0\n")
    sig = F.read_rho(str(p), 2)
    phi = -10e-3
    assert abs(sig[0] - complex(np.cos(phi) / 100.0, -np.sin(phi) / 100.0)) < 1e-15
    assert abs(sig[1] - 0.1) < 1e-15


def test_volt_polarity_swap():
    sig = np.array([-2.0 + 0.0j, 1.0 - 0.01j])
    b, p, v = F.volt_record(sig, np.array([10002, 10002]), np.array([30004, 30004]))
    assert v.tolist() == [40003, 30004] and abs(p[0]) < 1e-12 and b[0] == 2.0


def test_border_fix_takes_last_matching_element():
    g, *_ = load_case("minimal")
    g2 = g.copy()
    g2.rnr[:] = 1  # corrupt every pointer
    n = F.fix_border_elements(g2)
    assert n > 0 and np.array_equal(g2.rnr, g.rnr)


def test_boundary_values_file(tmp_path):
    """src/rrandb.f90 (complex case): list-directed complex values, a value
    split over two records, a bare real, the Neumann block read and dropped;
    a node above sanz is errnr 30."""
    p = tmp_path / "boundary.dat"
    p.write_text("3\n5 (1.5, -2.0)\n7 ( 0.25 ,\n 1d-3 )\n9 2.0\n2\n(1,2) (3,4)\n")
    nodes, vals = F.read_boundary_values(str(p), 20)
    assert nodes.tolist() == [5, 7, 9]
    assert np.array_equal(vals, [1.5 - 2j, 0.25 + 1e-3j, 2.0])
    F.write_boundary_values(str(p), nodes, vals)
    n2, v2 = F.read_boundary_values(str(p), 20)
    assert np.array_equal(n2, nodes) and np.array_equal(v2, vals)
    with pytest.raises(F.CRError) as ei:
        F.read_boundary_values(str(p), 8)
    assert ei.value.errnr == 30


def test_potential_and_sensitivity_files(tmp_path):
    """src/wpot.f90 / src/wsens.f90 layouts: numbered names, x y Re Im lines
    (the potential of each measurement's current pair; J per element with
    the |sum| / phase header), read back against the arrays written."""
    from conftest import load_case
    from oracle import oracle as O
    from titatest_gb300 import regularization as R
    assert F.numbered_path("../mod/pot/pot.dat", 7, 12) == "../mod/pot/pot07.dat"
    assert F.numbered_path("sens/sens.dat", 7, 1199) == "sens/sens0007.dat"
    g, sv, sig, cfg, _ = load_case("minimal")
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    hp = P.rtrafo(P.forward(sig, kwn, kwnwi), kwnwi)
    F.write_potentials(str(tmp_path / "pot" / "pot.dat"), hp, sv.strnr, np.ones(sv.nanz), g)
    vals = np.loadtxt(tmp_path / "pot" / "pot03.dat")
    e1, e2 = sv.strnr[2] % 10000, sv.strnr[2] // 10000
    want = hp[e2 - 1] - hp[e1 - 1]
    x, y = g.node_xy()
    assert vals.shape == (g.sanz, 4) and np.allclose(vals[:, 0], x.astype(np.float32))
    assert np.allclose(vals[:, 2] + 1j * vals[:, 3], want, rtol=1e-6, atol=1e-7 * np.abs(want).max())
    rng = np.random.default_rng(1)
    J = rng.normal(size=(sv.nanz, g.elanz)) + 1j * rng.normal(size=(sv.nanz, g.elanz))
    cx, cy = R._centroids(g)
    F.write_sensitivities(str(tmp_path / "sens" / "sens.dat"), J, cx, cy)
    with open(tmp_path / "sens" / "sens05.dat") as fh:
        head = [float(t) for t in fh.readline().split()]
        body = np.loadtxt(fh)
    s = J[4].sum()
    assert abs(head[0] / abs(s) - 1) < 1e-6 and abs(head[1] - 1e3 * np.angle(s)) < 1e-3
    assert np.allclose(body[:, 2] + 1j * body[:, 3], J[4], rtol=1e-6)
