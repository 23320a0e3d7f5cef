"""Ensembles of uneven meshes (titatest_gb300.ensemble): problems run
concurrently on their contexts' streams must give exactly the results of
running each problem alone, and those must match the oracle (voltages 1e-6,
Jacobian 1e-5 relative, the mixed-precision tolerances)."""
import numpy as np
import pytest

from conftest import relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_ensemble_equals_one_by_one_and_oracle(gpu_lib):
    from titatest_gb300 import MIXED, CRMod, synth
    from titatest_gb300.ensemble import Ensemble
    probs = sorted(synth.config5(count=10), key=lambda p: p.grid.sanz)[:6]  # the smaller ones
    ens = Ensemble(probs, precision=MIXED, workers=3, refine_tol=1e-10)
    res = ens.run(sens_mode=0, keep_sens=True)
    for p, r in zip(probs, res):
        with CRMod(p.grid, p.survey, precision=MIXED) as m:
            m.set_refinement(8, 1e-10)
            v = m.forward(p.sigma)["volt"]
            J = m.bsens()
        assert relerr(r["volt"], v) < 1e-12
        assert relerr(r["sens"], J) < 1e-12
        P = O.Problem(p.grid, p.survey)
        kwn, kwnwi = P.rwaven()
        kp = P.forward(p.sigma, kwn, kwnwi)
        vo, _ = P.bvolt(P.rtrafo(kp, kwnwi), 0, None)
        assert relerr(r["volt"], vo) < 1e-6
        assert relerr(r["sens"], P.bsens(kp, kwn, kwnwi, p.sigma, vo, mode=0)) < 1e-5
