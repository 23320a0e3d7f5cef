"""Synthetic data noise (titatest_gb300/noise.py) against the noise the
reference drew for examples/MGS/01_simple/03_mgs (tests/golden/noise_mgs:
crt.noisemod with seed 1, the clean volt.dat, and the reference's
inv.mynoise_rho / _pha / _voltages)."""
import dataclasses
import os

import numpy as np

from titatest_gb300 import inversion as I
from titatest_gb300 import noise as N

G = os.path.join(os.path.dirname(__file__), "golden", "noise_mgs")
CFG = os.path.join(os.path.dirname(__file__), "golden", "mixed_surf", "crtomo.cfg")


def _records(name):
    with open(os.path.join(G, name)) as fh:
        return [ln.rstrip("\n") for ln in fh if not ln.startswith("#")]


def test_generator_matches_reference_deviates():
    rho, pha = _records("inv.mynoise_rho"), _records("inv.mynoise_pha")
    g_r = N.PortableRandom(1).gauss_n(len(rho))
    g_p = N.PortableRandom(-1).gauss_n(len(pha))
    assert [N._g14_4(x).strip() for x in g_r] == [ln.split()[0] for ln in rho]
    assert [N._g14_4(x).strip() for x in g_p] == [ln.split()[0] for ln in pha]


def test_noise_model_file():
    assert N.read_noisemodel(os.path.join(G, "crt.noisemod")) == (1, 0.4, 1e-4, 0.0, 0.0, 0.0, 0.0)


def _cfg():
    cfg = I.read_crtomo_cfg(CFG)
    return dataclasses.replace(cfg, ldc=False, noise=N.read_noisemodel(os.path.join(G, "crt.noisemod")))


def test_noisy_data_and_records(tmp_path):
    cfg = _cfg()
    recs = []
    data = I.read_data(os.path.join(G, "volt.dat"), cfg, 10000, recs)
    ref = np.array([[float(x) for x in ln.split()[2:4]] for ln in _records("inv.mynoise_voltages")[1:]])
    new_bet = np.array([r[6] for r in recs])
    # the reference's build contracts some products into FMAs: within one ulp
    np.testing.assert_allclose(new_bet, ref[:, 0], rtol=3e-16, atol=0)
    np.testing.assert_array_equal(np.array([r[7] for r in recs]), ref[:, 1])  # zero phase noise
    np.testing.assert_allclose(data.dat.real, -np.log(ref[:, 0]), rtol=1e-14)
    # the weights keep the clean data's error model
    bet0 = np.array([r[4] for r in recs])
    np.testing.assert_allclose(data.wmatdr, 1.0 / (1e-2 * cfg.stabw0 + cfg.stabm0 / bet0) ** 2, rtol=1e-15)
    N.write_records(str(tmp_path), data.strnr, data.vnr, recs, False)
    for name in ("inv.mynoise_rho", "inv.mynoise_pha"):
        ours = [ln.rstrip("\n") for ln in open(tmp_path / name) if not ln.startswith("#")]
        assert [ln.split() for ln in ours] == [ln.split() for ln in _records(name)]
