"""Autotuner (crgpu_autotune): the kernels it picks give the same results as
the defaults (against the oracle), for a band that fits the tensor-core
window (config 1, mb 33) and one that does not (mb 192); the choice is
cached by problem shape."""
import numpy as np
import pytest

from conftest import relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _oracle(g, sv, sigma):
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    kp = P.forward(sigma, kwn, kwnwi)
    hp = P.rtrafo(kp, kwnwi)
    volt, _ = P.bvolt(hp, 0, None)
    return P, kwn, kwnwi, kp, volt


def test_autotune_config1_matches_oracle(gpu_lib):
    from titatest_gb300 import MIXED, CRMod, synth
    s = synth.config1()
    P, kwn, kwnwi, kp, volt = _oracle(s.grid, s.survey, s.sigma)
    sens0 = P.bsens(kp, kwn, kwnwi, s.sigma, volt, mode=0)
    with CRMod(s.grid, s.survey, kwn, kwnwi, precision=MIXED) as m:
        m.set_refinement(8, 1e-10)
        t = m.autotune(s.sigma, force=True)
        assert t["factor"] in ("tensor cores", "SIMT register tiles")
        assert t["jacobian"] in ("tensor cores", "SIMT")
        out = m.forward(s.sigma)
        assert relerr(out["volt"], volt) < 1e-6
        assert relerr(m.bsens(), sens0) < 1e-5
    with CRMod(s.grid, s.survey, kwn, kwnwi, precision=MIXED) as m2:
        assert m2.autotune(s.sigma) == t  # cached by problem shape


def test_autotune_wide_band_matches_plain(gpu_lib):
    from test_gpu_forward import _wide_band_case
    from titatest_gb300 import MIXED, PLAIN, CRMod
    g, sv, sig = _wide_band_case()
    kwn, kwnwi = O.Problem(g, sv).rwaven()
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN) as m:
        vp = m.forward(sig)["volt"]
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED, band_order=0) as m:  # the grid's own band
        m.set_refinement(10, 1e-10)
        t = m.autotune(sig, force=True)
        assert t["factor"] == "SIMT shared-memory tiles" and t["factor_blocks_per_sm"] in (1, 2)
        vm = m.forward(sig)["volt"]
    assert relerr(vm, vp) < 1e-6
