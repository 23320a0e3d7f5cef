"""Mixed-precision Jacobian: the tensor-core Gram-form contraction (eanz <= 128)
and the SIMT contraction it falls back to (eanz > 128), against the oracle's
src/bsens.f90 / src/bsensi.f90 restatement in FP64.

Meshes of linear triangles (element type 3, nk = 3) with electrode counts
whose 2 eanz is not a multiple of 16 exercise the padded MMA rows; a quad
mesh with 140 electrodes takes the fallback."""
import numpy as np
import pytest

from conftest import relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_SENS_TOL = 1e-5


def _mesh(nx, nz, ne, triangles, seed):
    from titatest_gb300 import synth
    rng = np.random.default_rng(seed)
    xs = np.arange(nx + 1, dtype=float) - 4.0
    depths = np.arange(nz + 1, dtype=float) * 0.8
    if triangles:
        grid, surface, X, Y = synth._quad_grid(xs, depths, triangles=True, jitter=0.15, rng=rng)
    else:
        grid, surface, X, Y = synth._quad_grid(xs, depths)
    mag, pha = synth.random_model(grid, rng)
    enodes = np.arange(4, 4 + ne)
    quads = synth._subsample(synth.dipole_dipole(ne, range(1, 3), range(1, 6)), 300, rng)
    return synth._finish("t", grid, surface, enodes, quads, mag, pha, nx, nz, triangles=triangles)


@pytest.mark.parametrize("nx,nz,ne,tri", [(48, 10, 37, True), (26, 8, 8, True), (150, 6, 140, False)])
def test_mixed_jacobian_matches_oracle(gpu_lib, nx, nz, ne, tri):
    from titatest_gb300 import MIXED, CRMod
    s = _mesh(nx, nz, ne, tri, seed=nx * 100 + ne)
    g, sv = s.grid, s.survey
    P = O.Problem(g, sv)
    kwn, kwnwi = P.rwaven()
    kp = P.forward(s.sigma, kwn, kwnwi)
    hp = P.rtrafo(kp, kwnwi)
    volt, _ = P.bvolt(hp, 0, None)
    sens0 = P.bsens(kp, kwn, kwnwi, s.sigma, volt, mode=0)
    sens1 = P.bsens(kp, kwn, kwnwi, s.sigma, volt, mode=1)
    with CRMod(g, sv, kwn, kwnwi, precision=MIXED) as m:
        m.set_refinement(8, 1e-10)
        m.forward(s.sigma)
        assert relerr(m.bsens(), sens0) < MIXED_SENS_TOL
        assert relerr(m.bsensi(), sens1) < MIXED_SENS_TOL
