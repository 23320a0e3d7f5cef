"""Differentiable forward (titatest_gb300.autograd) and the adjoint solve.

CPU: the complex-gradient convention of the autograd wrapper on a linear
stand-in model (V = M sigma), against PyTorch's own differentiation.
GPU: crgpu_adjoint against central finite differences of the forward, against
the reference's J^T g (src/bsens.f90) where reciprocity is exact (no mixed
boundary), the batched (refactoring) path against the resident one, and the
CRTomo misfit gradient in both precisions.
"""
import numpy as np
import pytest
import torch

from conftest import load_case, relerr


class _LinearModel:
    """Stand-in with the model interface the wrapper uses: V = M sigma."""

    def __init__(self, M):
        self.M = M

        class _S:
            nanz = M.shape[0]
        self.survey = _S()

    def forward(self, sigma):
        return {"volt": self.M @ sigma}

    def adjoint(self, g):
        return self.M.T @ g


def test_autograd_complex_convention_cpu():
    from titatest_gb300.autograd import volt
    rng = np.random.default_rng(7)
    M = rng.normal(size=(9, 6)) + 1j * rng.normal(size=(9, 6))
    d = rng.normal(size=9) + 1j * rng.normal(size=9)
    w = rng.uniform(0.5, 2.0, size=9)
    m0 = torch.tensor(rng.normal(size=6) * 0.1 + 1j * rng.normal(size=6) * 0.1, dtype=torch.complex128)

    m1 = m0.clone().requires_grad_(True)
    v = volt(_LinearModel(M), torch.exp(m1))
    loss = torch.sum(torch.as_tensor(w) * torch.abs(-torch.log(v) - torch.as_tensor(d)) ** 2)
    loss.backward()

    m2 = m0.clone().requires_grad_(True)
    v2 = torch.as_tensor(M) @ torch.exp(m2)
    loss2 = torch.sum(torch.as_tensor(w) * torch.abs(-torch.log(v2) - torch.as_tensor(d)) ** 2)
    loss2.backward()
    assert torch.allclose(m1.grad, m2.grad, rtol=1e-12, atol=1e-14)


def _forward_volt(m, sig):
    return m.forward(sig)["volt"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["minimal", "testmodinv"])
def test_adjoint_matches_central_differences(gpu_lib, case):
    """sum_i g_i dV_i/dsigma_e by the adjoint vs fourth-order central
    differences, including elements on mixed boundaries.  Step 1e-2 |sigma_e|:
    the O(h^4) truncation is ~1e-9 there, while below ~1e-3 the rounding of
    the forward (condition number times 1e-16, divided by h) dominates."""
    from titatest_gb300 import PLAIN, CRMod
    g_, sv, sig, cfg, _ = load_case(case)
    rng = np.random.default_rng(11)
    sig = sig * np.exp(1j * rng.uniform(-0.03, 0.0, size=sig.shape))  # complex model
    g = rng.normal(size=sv.nanz) + 1j * rng.normal(size=sv.nanz)
    with CRMod(g_, sv, precision=PLAIN) as m:
        v0 = _forward_volt(m, sig)
        grad = m.adjoint(g)
        nb = m.grid.elanz
        elems = sorted(set(rng.choice(nb, size=8, replace=False).tolist() + [0, nb - 1]))
        def F(e, d):
            sp = sig.copy()
            sp[e] += d
            return np.sum(g * _forward_volt(m, sp))

        for e in elems:
            h = 1e-2 * abs(sig[e])
            fd = (8 * (F(e, h) - F(e, -h)) - (F(e, 2 * h) - F(e, -2 * h))) / (12 * h)
            assert abs(grad[e] - fd) <= 1e-7 * max(abs(fd), 1e-3 * np.abs(grad).max()), (e, grad[e], fd)
        assert np.all(np.isfinite(v0))


@pytest.mark.gpu
def test_adjoint_equals_reference_jt_g_without_mixed_boundaries(gpu_lib):
    """2D problem with no-flow boundaries only: reciprocity is exact, so the
    reference's J (src/bsens.f90, unit current) gives the same J^T g."""
    from titatest_gb300 import PLAIN, CRMod
    g_, sv, sig, cfg, _ = load_case("decoupling_2d_sink")
    rng = np.random.default_rng(5)
    g = rng.normal(size=sv.nanz) + 1j * rng.normal(size=sv.nanz)
    with CRMod(g_, sv, swrtr=cfg.swrtr, lsink=cfg.lsink, nsink=cfg.nsink, precision=PLAIN) as m:
        m.forward(sig)
        grad = m.adjoint(g)
        J = m.bsens()
    strom = np.asarray(sv.strom) if getattr(sv, "strom", None) is not None else np.ones(sv.nanz)
    jtg = (g / strom) @ J
    assert relerr(grad, jtg) < 1e-8


@pytest.mark.gpu
def test_adjoint_refactoring_path_equals_resident(gpu_lib):
    """A forward that needs several batches keeps no factors: the adjoint
    refactors batch by batch and must give the resident result."""
    from titatest_gb300 import PLAIN, CRMod
    g_, sv, sig, cfg, _ = load_case("testmodinv")
    rng = np.random.default_rng(3)
    g = rng.normal(size=sv.nanz) + 1j * rng.normal(size=sv.nanz)
    with CRMod(g_, sv, precision=PLAIN) as m:
        m.forward(sig)
        g1 = m.adjoint(g)
        nb1 = m.stats()["nbatches"]
    with CRMod(g_, sv, precision=PLAIN) as m:
        n, w = g_.sanz, g_.mb + 1
        per = n * w * 16 + n * 16 * 40
        m.set_memory_budget(per * 7)  # a handful of systems per batch
        m.forward(sig)
        nb2 = m.stats()["nbatches"]
        g2 = m.adjoint(g)
    assert nb1 == 1 and nb2 > 1
    assert relerr(g2, g1) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-5), (1, 1e-4)])
def test_crtomo_misfit_gradient_matches_central_differences(gpu_lib, prec, tol):
    """dphi/dm of phi(m) = sum w |-log V(exp m) - dobs|^2 by autograd vs
    central differences in the real and imaginary parts of m_e."""
    from titatest_gb300 import CRMod, synth
    from titatest_gb300.autograd import CRTomoMisfit
    s = synth.config1()
    rng = np.random.default_rng(9)
    with CRMod(s.grid, s.survey, precision=prec) as m:
        m.set_refinement(20, 1e-12)
        dobs = -np.log(m.forward(s.sigma)["volt"])
        dobs = dobs + 0.01 * rng.normal(size=dobs.shape)
        wmatd = np.full(dobs.shape, 1.0)
        phi = CRTomoMisfit(m, dobs, wmatd).cuda()
        m0 = torch.full((s.grid.elanz,), complex(np.log(0.01), -0.01), dtype=torch.complex128, device="cuda")
        mm = m0.clone().requires_grad_(True)
        loss = phi(mm)
        loss.backward()
        grad = mm.grad.cpu().numpy()
        for e in rng.choice(s.grid.elanz, size=6, replace=False):
            h = 1e-6
            vals = []
            for d in (h, -h, 1j * h, -1j * h):
                mp = m0.clone()
                mp[e] += d
                vals.append(float(phi(mp)))
            fd = complex((vals[0] - vals[1]) / (2 * h), (vals[2] - vals[3]) / (2 * h))
            assert abs(grad[e] - fd) <= tol * max(abs(fd), 1e-2 * np.abs(grad).max()), (e, grad[e], fd)
