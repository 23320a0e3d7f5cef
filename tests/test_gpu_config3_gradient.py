"""The differentiable forward on the 250x100 split-triangle mesh (50000
triangles, 25351 nodes, 64 electrodes, 2000 dipole-dipole quadrupoles).

The CRTomo data misfit phi(m) = sum_i w_i |(-log V_i(exp m)) - d_i|^2 on
complex log-conductivities m, with d the model's response plus 3% Gaussian
magnitude noise and 1 mrad phase noise (w = 1/0.03^2), is differentiated by
the adjoint behind torch.autograd (titatest_gb300.autograd) and checked:

  * against central finite differences of phi at step h = 1e-6 on 50 seeded
    elements, in complex64 + FP64 refinement (phi at m_e +- h and m_e +- i h)
    and in complex128 (the voltage vector at m_e +- h: V is holomorphic in
    m_e, so dV/dm_e along the real axis is the complex derivative, and both
    partial derivatives of phi follow from it by the chain rule);
  * against the reference's own gradient, 2 J^H W r with J of
    src/bsensi.f90:23-194 (J = d(-log V)/dm, as src/update.f90:236-293 forms
    J^H W (d - f)).  That J assumes reciprocity across the electrode-dependent
    mixed boundary (src/beta.f90), so it differs from the exact derivative;
    the gap is measured and bounded here.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

H = 1e-6
N_ELEM = 50
# |adjoint - central difference| / max(|central difference|, 1e-2 max|gradient|):
# at h = 1e-6 the differences carry the forward's rounding divided by h, about
# 1e-5 .. 1e-4 here (measured worst: 3.2e-5 complex64, 8.0e-5 complex128)
FD_TOL = 2e-4


@pytest.fixture(scope="module")
def cfg3():
    from titatest_gb300 import PLAIN, CRMod, synth
    s = synth.config3()
    rng = np.random.default_rng(3003)
    with CRMod(s.grid, s.survey, precision=PLAIN) as m:
        v = m.forward(s.sigma)["volt"]
    d = -np.log(v)
    dobs = d - np.log1p(0.03 * rng.normal(size=d.shape)) - 1j * 1e-3 * rng.normal(size=d.shape)
    w = np.full(d.shape, 1.0 / 0.03 ** 2)
    # start model: the homogeneous model of the mean log-conductivity
    m0 = np.full(s.grid.elanz, np.mean(np.log(s.sigma)), np.complex128)
    elems = np.sort(rng.choice(s.grid.elanz, size=N_ELEM, replace=False))
    return s, dobs, w, m0, elems


def _autograd(m, dobs, w, m0):
    from titatest_gb300.autograd import CRTomoMisfit
    phi = CRTomoMisfit(m, dobs, w).cuda()
    mm = torch.tensor(m0, device="cuda").requires_grad_(True)
    phi(mm).backward()
    return phi, mm.grad.cpu().numpy()


def test_config3_gradient_mixed_against_central_differences(gpu_lib, cfg3):
    from titatest_gb300 import MIXED, CRMod
    s, dobs, w, m0, elems = cfg3
    with CRMod(s.grid, s.survey, precision=MIXED) as m:
        m.set_refinement(20, 1e-12)
        phi, grad = _autograd(m, dobs, w, m0)
        base = torch.tensor(m0, device="cuda")

        def f(e, dm):
            mp = base.clone()
            mp[e] += dm
            return float(phi(mp))

        gmax = np.abs(grad).max()
        worst = 0.0
        for e in elems:
            fd = complex((f(e, H) - f(e, -H)) / (2 * H), (f(e, 1j * H) - f(e, -1j * H)) / (2 * H))
            worst = max(worst, abs(grad[e] - fd) / max(abs(fd), 1e-2 * gmax))
        print(f"complex64 + refinement: worst relative gradient error {worst:.2e} over {len(elems)} elements")
        assert worst < FD_TOL


def test_config3_gradient_plain_against_central_differences(gpu_lib, cfg3):
    from titatest_gb300 import PLAIN, CRMod
    s, dobs, w, m0, elems = cfg3
    with CRMod(s.grid, s.survey, precision=PLAIN) as m:
        phi, grad = _autograd(m, dobs, w, m0)
        sig0 = np.exp(m0)
        v0 = m.forward(sig0)["volt"]
        r = -np.log(v0) - dobs
        gmax = np.abs(grad).max()
        worst = 0.0
        for e in elems:
            vp = m.forward(sig0 * np.where(np.arange(len(m0)) == e, np.exp(H), 1.0))["volt"]
            vm = m.forward(sig0 * np.where(np.arange(len(m0)) == e, np.exp(-H), 1.0))["volt"]
            dfdm = -(np.log(vp) - np.log(vm)) / (2 * H)  # d(-log V)/dm_e, holomorphic
            # phi = sum w |r|^2:  dphi/dRe m_e = 2 Re sum w conj(r) df,  dphi/dIm m_e = 2 Re sum w conj(r) i df
            fd = complex(2 * np.sum(w * (np.conj(r) * dfdm).real), 2 * np.sum(w * (np.conj(r) * 1j * dfdm).real))
            worst = max(worst, abs(grad[e] - fd) / max(abs(fd), 1e-2 * gmax))
        print(f"complex128: worst relative gradient error {worst:.2e} over {len(elems)} elements")
        assert worst < FD_TOL


def test_config3_gradient_against_reference_jacobian(gpu_lib, cfg3):
    """Exact adjoint gradient against 2 J^H W r with the reference's J: the
    gap is the mixed-boundary term that the reference's reciprocity omits."""
    from titatest_gb300 import PLAIN, CRMod
    s, dobs, w, m0, elems = cfg3
    with CRMod(s.grid, s.survey, precision=PLAIN) as m:
        phi, grad = _autograd(m, dobs, w, m0)
        v0 = m.forward(np.exp(m0))["volt"]
        J = m.bsensi()  # d(-log V)/dm by src/bsensi.f90
    r = -np.log(v0) - dobs
    gref = 2 * (np.conj(J).T @ (w * r))
    gap = np.abs(grad - gref)
    rel_l2 = float(np.linalg.norm(grad - gref) / np.linalg.norm(grad))
    # elements with a node on the mixed (type 11) boundary
    g = s.grid
    E = g.elanz
    bnodes = set(g.nrel[E + int(g.nelanz[1]):, :2].ravel().tolist())  # nodes of the type-11 lines
    on_b = np.array([any(int(x) in bnodes for x in g.nrel[e, :3]) for e in range(E)])
    rel_in = float(np.linalg.norm((grad - gref)[~on_b]) / np.linalg.norm(grad[~on_b]))
    rel_b = float(np.linalg.norm((grad - gref)[on_b]) / np.linalg.norm(grad[on_b]))
    print(f"reference J^H W r vs exact gradient: relative L2 gap {rel_l2:.2e} (interior {rel_in:.2e}, "
          f"mixed-boundary elements {rel_b:.2e}), max gap {gap.max():.3e} of max |grad| {np.abs(grad).max():.3e}")
    assert rel_l2 < 0.02 and rel_in < 2e-3
