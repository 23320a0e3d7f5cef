"""crgpu_forward_sens_batch: several uneven meshes (config-5 problems: the
smallest, the median, the widest band and two more), their band factors in
one persistent tensor-core launch over a (problem, system) table, against
each problem run alone and against the oracle (mixed-precision tolerances:
voltages 1e-6, Jacobian 1e-5)."""
import numpy as np
import pytest

from conftest import relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_forward_sens_batch_matches_single_and_oracle(gpu_lib):
    from titatest_gb300 import MIXED, CRMod, synth
    from titatest_gb300.crmod import forward_sens_batch
    shapes = synth.config5_shapes()
    by_size = sorted(range(len(shapes)), key=lambda q: shapes[q][0] * shapes[q][1])
    picks = [by_size[0], by_size[len(by_size) // 2], by_size[-1], by_size[10], by_size[200]]
    probs = synth.config5(indices=picks)
    models = [CRMod(p.grid, p.survey, precision=MIXED) for p in probs]
    try:
        for m in models:
            m.set_refinement(8, 1e-10)
        volts = forward_sens_batch(models, [p.sigma for p in probs], sens_mode=0)
        for m, p, v in zip(models, probs, volts):
            Jb = m.bsens()  # from the batch's potentials
            with CRMod(p.grid, p.survey, precision=MIXED) as m1:
                m1.set_refinement(8, 1e-10)
                v1 = m1.forward(p.sigma)["volt"]
                J1 = m1.bsens()
            assert relerr(v, v1) < 1e-10
            assert relerr(Jb, J1) < 1e-9
        p, v = probs[0], volts[0]
        P = O.Problem(p.grid, p.survey)
        kwn, kwnwi = P.rwaven()
        kp = P.forward(p.sigma, kwn, kwnwi)
        vo, _ = P.bvolt(P.rtrafo(kp, kwnwi), 0, None)
        assert relerr(v, vo) < 1e-6
        assert relerr(models[0].bsens(), P.bsens(kp, kwn, kwnwi, p.sigma, vo, mode=0)) < 1e-5
    finally:
        for m in models:
            m.close()


def test_forward_sens_batch_rejects_plain_contexts(gpu_lib):
    from titatest_gb300 import PLAIN, CRMod, synth
    from titatest_gb300._lib import CRGPUError
    from titatest_gb300.crmod import forward_sens_batch
    p = synth.config1()
    with CRMod(p.grid, p.survey, precision=PLAIN) as m:
        with pytest.raises(CRGPUError) as ei:
            forward_sens_batch([m], [p.sigma])
        assert ei.value.errnr == 1002
