"""crgpu_factor_system_noalloc against crgpu_factor_system.

The no-alloc entry point serves callers that cannot allocate device memory
when they call (for example while a CUDA graph is being captured, or inside a
framework that owns every device allocation): it takes caller-owned device
buffers and keeps its scratch in one fixed array inside the library.  Its
factor and scaling vector must equal those of the allocating entry point,
call after call (the scratch keeps the previous call's contents).

This file is collected last so that a failure here does not hide the rest of
the suite in a run that stops at the first failure.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case, relerr

pytestmark = pytest.mark.gpu


def test_factor_system_noalloc_matches_allocating_entry(gpu_lib):
    import torch

    from titatest_gb300 import PLAIN, CRMod
    from titatest_gb300._lib import lib

    g, sv, sig, cfg, _ = load_case("testmodinv")
    L = lib()
    with CRMod(g, sv, precision=PLAIN) as m:
        n, w = g.sanz, g.mb + 1
        sig_dev = torch.from_numpy(np.ascontiguousarray(sig).view(np.float64).copy()).cuda()
        a_dev = torch.zeros(2 * n * w, dtype=torch.float64, device="cuda")
        fak_dev = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for k, l in [(1, 1), (m.kwnanz, sv.eanz)]:  # two calls in a row
            rc = L.crgpu_factor_system_noalloc(m._h, C.c_void_p(sig_dev.data_ptr()), k, l,
                                               C.c_void_p(a_dev.data_ptr()), C.c_void_p(fak_dev.data_ptr()),
                                               None)
            assert rc == 0, L.crgpu_last_error(m._h).decode()
            a_ref, fak_ref = m.factor_system(sig, k, l)
            a = a_dev.cpu().numpy().view(np.complex128).reshape(n, w)
            fak = fak_dev.cpu().numpy()
            assert relerr(fak, fak_ref) < 1e-10
            # columns before the first row are outside the matrix in both layouts
            for i in range(n):
                lo = max(0, g.mb - i)
                assert relerr(a[i, lo:], a_ref[i, lo:]) < 1e-10


def test_factor_system_noalloc_rejects_mixed_context(gpu_lib):
    import torch

    from titatest_gb300 import MIXED, CRMod
    from titatest_gb300._lib import lib

    g, sv, sig, cfg, _ = load_case("minimal")
    L = lib()
    with CRMod(g, sv, precision=MIXED) as m:
        buf = torch.zeros(2 * g.sanz * (g.mb + 1), dtype=torch.float64, device="cuda")
        rc = L.crgpu_factor_system_noalloc(m._h, C.c_void_p(buf.data_ptr()), 1, 1, C.c_void_p(buf.data_ptr()),
                                           C.c_void_p(buf.data_ptr()), None)
        assert rc == 1002
