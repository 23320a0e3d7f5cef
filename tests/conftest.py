"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
FORWARD_CASES = ["minimal", "testmodinv", "mixed_surf", "decoupling_2d_sink"]
CUTMCK_CASES = sorted(d[len("cutmck_"):] for d in os.listdir(GOLDEN) if d.startswith("cutmck_"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def load_case(name):
    """(grid, survey, sigma, crmod.cfg, golden volt.dat columns) of a golden
    forward case; the measurement configurations are volt.dat's (strnr, vnr)."""
    from titatest_gb300 import formats as F
    d = os.path.join(GOLDEN, name)
    g = F.read_elem(os.path.join(d, "elem.dat"))
    enr = F.read_elec(os.path.join(d, "elec.dat"), g.sanz)
    s, v, bet, pha = F.read_volt(os.path.join(d, "volt.dat"))
    sig = F.read_rho(os.path.join(d, "rho.dat"), g.elanz)
    cfg = F.read_crmod_cfg(os.path.join(d, "crmod.cfg"))
    sv = F.Survey(enr=enr, strnr=s, vnr=v, strom=np.ones(len(s)))
    return g, sv, sig, cfg, (bet, pha)


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libcrtomo_gb300; GPU tests only."""
    from titatest_gb300 import build
    build.build()
    from titatest_gb300 import _lib
    return _lib.lib()
