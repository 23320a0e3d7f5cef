"""Dirichlet boundary values (src/randb2.f90) on the GPU against the oracle's
restatement: plain complex128 at 1e-10, mixed precision at the voltage
tolerance.  The values enter the systems that src/kompab.f90 assembles; with
no mixed boundary (decoupling_2d_sink) the electrodes after the first take
src/kompb.f90's right-hand side, which leaves them out.  The valued nodes
also make that 2D no-flow problem well posed, so it is compared directly."""
import numpy as np
import pytest

from conftest import load_case, relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-10
MIXED_VOLT_TOL = 1e-6


def _values(g, sv, count, seed, exclude=()):
    rng = np.random.default_rng(seed)
    skip = set(int(e) for e in sv.enr) | set(int(x) for x in exclude)
    pool = [i for i in range(1, g.sanz + 1) if i not in skip]
    nodes = np.sort(rng.choice(pool, size=count, replace=False)).astype(np.int32)
    vals = rng.uniform(0.2, 2.0, count) * np.exp(1j * rng.uniform(-0.05, 0.0, count))
    return nodes, vals


def _oracle(g, sv, sig, nodes, vals, swrtr=1, lsink=False, nsink=0, lsr=False):
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven() if swrtr else (np.zeros(1), np.zeros(1))
    P.set_boundary_values(nodes, vals)
    kp = P.forward(sig, kwn, kwnwi, swrtr=swrtr, lsink=lsink, nsink=nsink, lsr=lsr)
    hp = P.rtrafo(kp, kwnwi, swrtr)
    volt, _ = P.bvolt(hp, 0, None)
    return kwn, kwnwi, kp, hp, volt


@pytest.mark.parametrize("case", ["minimal", "testmodinv", "decoupling_2d_sink"])
def test_plain_forward_with_boundary_values_matches_oracle(gpu_lib, case):
    from titatest_gb300 import PLAIN, CRMod
    g, sv, sig, cfg, _ = load_case(case)
    nodes, vals = _values(g, sv, 10, seed=len(case), exclude=[cfg.nsink] if cfg.lsink else [])
    kwn, kwnwi, kp, hp, volt = _oracle(g, sv, sig, nodes, vals, cfg.swrtr, cfg.lsink, cfg.nsink)
    with CRMod(g, sv, kwn, kwnwi, swrtr=cfg.swrtr, lsink=cfg.lsink, nsink=cfg.nsink, precision=PLAIN) as m:
        m.set_boundary_values(nodes, vals)
        out = m.forward(sig, kpot=True, hpot=True)
    assert relerr(out["kpot"], kp) < PLAIN_TOL
    assert relerr(out["hpot"], hp) < PLAIN_TOL
    assert relerr(out["volt"], volt) < PLAIN_TOL
    assert np.array_equal(out["kpot"][:, 0, nodes - 1], np.broadcast_to(vals, (len(kwn), len(vals))))


def test_boundary_values_repeated_node_and_removal(gpu_lib):
    """A node listed twice: b takes the last value, the moved column the
    first (the second pass of src/randb2.f90 finds the column removed).
    Removing the values restores the plain forward."""
    from titatest_gb300 import PLAIN, CRMod
    g, sv, sig, cfg, _ = load_case("minimal")
    nodes, vals = _values(g, sv, 6, seed=9)
    nodes = np.concatenate([nodes, nodes[2:3]])
    vals = np.concatenate([vals, [0.7 - 0.02j]])
    kwn, kwnwi, kp, hp, volt = _oracle(g, sv, sig, nodes, vals)
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN) as m:
        v_plain = m.forward(sig)["volt"]
        m.set_boundary_values(nodes, vals)
        out = m.forward(sig, kpot=True)
        assert relerr(out["kpot"], kp) < PLAIN_TOL
        assert relerr(out["volt"], volt) < PLAIN_TOL
        m.set_boundary_values(None, None)
        assert relerr(m.forward(sig)["volt"], v_plain) < 1e-14


def test_mixed_forward_with_boundary_values_matches_oracle(gpu_lib):
    from titatest_gb300 import MIXED, CRMod
    g, sv, sig, cfg, _ = load_case("testmodinv")
    nodes, vals = _values(g, sv, 16, seed=21)
    kwn, kwnwi, kp, hp, volt = _oracle(g, sv, sig, nodes, vals)
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED) as m:
        m.set_refinement(8, 1e-10)
        m.set_boundary_values(nodes, vals)
        out = m.forward(sig)
    assert relerr(out["volt"], volt) < MIXED_VOLT_TOL


def test_singularity_removal_with_boundary_values_matches_oracle(gpu_lib):
    from titatest_gb300 import PLAIN, CRMod
    g, sv, sig, cfg, _ = load_case("minimal")
    nodes, vals = _values(g, sv, 8, seed=5)
    kwn, kwnwi, kp, hp, volt = _oracle(g, sv, sig, nodes, vals, lsr=True)
    with CRMod(g, sv, kwn, kwnwi, precision=PLAIN, lsr=True) as m:
        m.set_boundary_values(nodes, vals)
        out = m.forward(sig, kpot=True)
    assert relerr(out["kpot"], kp) < PLAIN_TOL
    assert relerr(out["volt"], volt) < PLAIN_TOL


def test_adjoint_with_boundary_values_matches_central_differences(gpu_lib):
    """With prescribed values the moved column depends on sigma: the adjoint
    keeps the potential at the valued nodes (lambda is 0 there)."""
    from titatest_gb300 import PLAIN, CRMod
    g_, sv, sig, cfg, _ = load_case("minimal")
    rng = np.random.default_rng(12)
    sig = sig * np.exp(1j * rng.uniform(-0.03, 0.0, size=sig.shape))
    nodes, vals = _values(g_, sv, 10, seed=13)
    g = rng.normal(size=sv.nanz) + 1j * rng.normal(size=sv.nanz)
    with CRMod(g_, sv, precision=PLAIN) as m:
        m.set_boundary_values(nodes, vals)
        m.forward(sig)
        grad = m.adjoint(g)
        nb = g_.elanz

        def F(e, d):
            sp = sig.copy()
            sp[e] += d
            return np.sum(g * m.forward(sp)["volt"])

        for e in sorted(set(rng.choice(nb, size=8, replace=False).tolist() + [0, nb - 1])):
            h = 1e-2 * abs(sig[e])
            fd = (8 * (F(e, h) - F(e, -h)) - (F(e, 2 * h) - F(e, -2 * h))) / (12 * h)
            assert abs(grad[e] - fd) <= 1e-7 * max(abs(fd), 1e-3 * np.abs(grad).max()), (e, grad[e], fd)


def test_boundary_value_node_out_of_range_is_error_30(gpu_lib):
    from titatest_gb300 import PLAIN, CRMod
    from titatest_gb300._lib import CRGPUError
    g, sv, sig, cfg, _ = load_case("minimal")
    with CRMod(g, sv, precision=PLAIN) as m:
        with pytest.raises(CRGPUError) as ei:
            m.set_boundary_values([g.sanz + 1], [1.0])
        assert ei.value.errnr == 30
