"""crgpu_factor_system_noalloc against crgpu_factor_system and the oracle's chol.

The no-alloc entry point serves callers that cannot allocate device memory
when they call: a framework that hands out all device memory from its own
pool, or a host that must avoid the device-wide synchronisation of
cudaMalloc/cudaFree in the middle of its work.  It takes caller-owned device
buffers and keeps its scratch in one fixed array inside the library.  Its
factor and scaling vector must equal those of the allocating entry point and
of the oracle's src/chol.f90 restatement, call after call (the scratch keeps
the previous call's contents), on the context's stream and on a stream the
caller owns.

This file is collected last so that a failure here does not hide the rest of
the suite in a run that stops at the first failure.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case, relerr

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _band_err(a, a_ref, mb):
    """Largest row-wise relative difference over the entries inside the matrix
    (columns before the first row are outside it in both layouts)."""
    worst = 0.0
    for i in range(a.shape[0]):
        lo = max(0, mb - i)
        ref = a_ref[i, lo:]
        if np.max(np.abs(ref)) < 1e-300:
            continue
        worst = max(worst, relerr(a[i, lo:], ref))
    return worst


@pytest.mark.parametrize("own_stream", [False, True])
def test_factor_system_noalloc_matches_allocating_entry_and_oracle(gpu_lib, own_stream):
    import torch

    from titatest_gb300 import PLAIN, CRMod
    from titatest_gb300._lib import lib

    g, sv, sig, cfg, _ = load_case("testmodinv")
    P = O.Problem(g, sv)
    L = lib()
    with CRMod(g, sv, precision=PLAIN) as m:
        n, w = g.sanz, g.mb + 1
        stream = torch.cuda.Stream() if own_stream else None
        sig_dev = torch.from_numpy(np.ascontiguousarray(sig).view(np.float64).copy()).cuda()
        a_dev = torch.zeros(2 * n * w, dtype=torch.float64, device="cuda")
        fak_dev = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        handle = C.c_void_p(stream.cuda_stream) if stream is not None else None
        for k, l in [(1, 1), (m.kwnanz, sv.eanz)]:  # two calls in a row
            rc = L.crgpu_factor_system_noalloc(m._h, C.c_void_p(sig_dev.data_ptr()), k, l,
                                               C.c_void_p(a_dev.data_ptr()), C.c_void_p(fak_dev.data_ptr()),
                                               handle)
            assert rc == 0, L.crgpu_last_error(m._h).decode()
            a_ref, fak_ref = m.factor_system(sig, k, l)
            a_or, fak_or = P.factor(sig, m.kwn, k, l)
            a = a_dev.cpu().numpy().view(np.complex128).reshape(n, w)
            fak = fak_dev.cpu().numpy()
            assert relerr(fak, fak_ref) < 1e-10
            assert relerr(fak, fak_or) < 1e-10
            assert _band_err(a, a_ref, g.mb) < 1e-10
            assert _band_err(a, a_or, g.mb) < 1e-10


def test_factor_system_noalloc_rejects_mixed_and_dc_contexts(gpu_lib):
    import torch

    from titatest_gb300 import MIXED, PLAIN, CRMod
    from titatest_gb300._lib import lib

    g, sv, sig, cfg, _ = load_case("minimal")
    L = lib()
    buf = torch.zeros(2 * g.sanz * (g.mb + 1), dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    with CRMod(g, sv, precision=MIXED) as m:
        assert L.crgpu_factor_system_noalloc(m._h, p, 1, 1, p, p, None) == 1002
    with CRMod(g, sv, precision=PLAIN) as m:
        m.set_dc(True)
        assert L.crgpu_factor_system_noalloc(m._h, p, 1, 1, p, p, None) == 1002
