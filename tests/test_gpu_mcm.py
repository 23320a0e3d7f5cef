"""Model uncertainty and resolution (crgpu_mcm: src/bmcm_mod.f90 bata,
bata_reg, bmcm, bres, bmcm2) on the library's own dense FP64 kernels, against
the oracle's restatement, on config 1's Jacobian (1200 cells: 19 blocks of
the blocked Cholesky factor and inverse, the last one partial).

Both sides are FP64 with different summation orders; the diagonals agree to
1e-9 relative (the resolution diagonal relative to its largest entry)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ltri", [0, 1])
def test_mcm_dense_kernels_match_oracle(gpu_lib, ltri):
    from titatest_gb300 import PLAIN, CRMod, synth
    from titatest_gb300 import regularization as R
    s = synth.config1()
    g = s.grid
    rng = np.random.default_rng(71)
    with CRMod(g, s.survey, precision=PLAIN) as m:
        m.forward(s.sigma, volt_mode=1)
        J = m.sens(1)  # also kept on the device for crgpu_mcm
        nanz, manz = J.shape
        wmatd = rng.uniform(0.5, 2.0, size=nanz) / 0.03 ** 2
        wdfak = np.ones(nanz, np.int32)
        if ltri == 0:
            smatm, nach = R.bsmatmreg(g, s.nx, s.nz), None
        else:
            nach = R.bnachbar(g)
            smatm = R.bsmatmtri(g, nach)
        d = m.mcm(wmatd, wdfak, ltri, smatm, nx=s.nx, nachbar=nach, lam=30.0)
    o = O.mcm(J, wmatd, wdfak, ltri, smatm, nx=s.nx, nachbar=nach, maxnk=g.maxnk, lam=30.0)
    assert manz == 1200
    for key in ("ata", "reg", "cov1", "cov2"):
        err = np.max(np.abs(d[key] / o[key] - 1))
        assert err < 1e-9, (key, err)
    assert np.max(np.abs(d["res"] - o["res"])) / np.max(np.abs(o["res"])) < 1e-9
