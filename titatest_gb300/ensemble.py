"""Forward + Jacobian of many independent problems (uneven meshes) at once.

Each problem gets its own context (its own band width, pattern and batch
buffers).  Problems are sorted by their band-factor work (n * mb^2 * number of
systems), largest first, and handed to a pool of worker threads.  Each worker
owns a CUDA stream, so the kernels of different problems run concurrently on
the GPU.  The C ABI releases the GIL, so the workers do not serialise on the
host.

The per-worker memory budget is the free device memory divided by the number
of workers.  A problem whose band factors do not fit is processed in batches
by its own context.
"""
from __future__ import annotations

import threading
from concurrent.futures import ThreadPoolExecutor
from typing import List, Optional, Sequence

import numpy as np

from . import MIXED, CRMod
from ._lib import device_memory


def problem_work(p) -> float:
    """Band-factor flops of one forward: 4 n mb^2 per (k, l) system (approximate k count)."""
    g = p.grid
    return 4.0 * g.sanz * g.mb * g.mb * max(1, p.survey.eanz)


class Ensemble:
    """Forward (and Jacobian) of `problems`: objects with .grid, .survey and
    .sigma, e.g. those of titatest_gb300.synth.config5()."""

    def __init__(self, problems: Sequence, precision: int = MIXED, workers: int = 8,
                 refine_maxit: int = 8, refine_tol: float = 1e-6, budget_bytes: Optional[int] = None,
                 autotune: bool = False):
        self.problems = list(problems)
        self.precision = precision
        self.workers = max(1, int(workers))
        self.refine = (refine_maxit, refine_tol)
        self.autotune = autotune  # per problem shape, cached by the library after the first run
        if budget_bytes is None:
            free, _ = device_memory()
            budget_bytes = int(0.5 * free / self.workers)
        self.budget = budget_bytes
        self.order = sorted(range(len(self.problems)), key=lambda i: -problem_work(self.problems[i]))
        self._tls = threading.local()

    def _stream(self):
        import torch
        if not hasattr(self._tls, "stream"):
            self._tls.stream = torch.cuda.Stream()
        return self._tls.stream

    def _one(self, i: int, sens_mode: Optional[int], keep_sens: bool):
        import torch

        p = self.problems[i]
        st = self._stream()
        with torch.cuda.stream(st):
            sig = torch.from_numpy(np.ascontiguousarray(p.sigma, np.complex128)).to("cuda", non_blocking=False)
            volt = torch.empty(p.survey.nanz, dtype=torch.complex128, device="cuda")
            with CRMod(p.grid, p.survey, precision=self.precision) as m:
                m.set_stream(st.cuda_stream)
                m.set_refinement(*self.refine)
                m.set_memory_budget(self.budget)
                if self.autotune:
                    m.autotune(p.sigma)
                m.forward_device(sig.data_ptr(), volt.data_ptr())
                out = {"index": i, "nanz": p.survey.nanz, "elanz": p.grid.elanz}
                if sens_mode is not None:
                    sens = torch.empty((p.grid.elanz, p.survey.nanz), dtype=torch.complex128, device="cuda")
                    m.sens_device(int(sens_mode), sens.data_ptr())
                    if keep_sens:
                        out["sens"] = sens.T.cpu().numpy()
                    else:  # a checksum keeps the result observable without the copy
                        out["sens_abs_sum"] = float(sens.abs().sum())
                out["stats"] = m.stats()
            out["volt"] = volt.cpu().numpy()
        st.synchronize()
        return out

    def run(self, sens_mode: Optional[int] = 0, keep_sens: bool = False) -> List[dict]:
        """Runs every problem; returns one dict per problem in input order."""
        results: List[Optional[dict]] = [None] * len(self.problems)
        with ThreadPoolExecutor(max_workers=self.workers) as ex:
            for r in ex.map(lambda i: self._one(i, sens_mode, keep_sens), self.order):
                results[r["index"]] = r
        return results  # type: ignore[return-value]
