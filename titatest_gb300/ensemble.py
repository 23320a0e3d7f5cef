"""Forward + Jacobian of many independent problems (uneven meshes) at once.

Each problem gets its own context (its own band width, pattern, batch
buffers and CUDA stream).  Problems are sorted by their band-factor work
(n * mb^2 * number of systems), largest first, and handed to a pool of
worker threads; every context issues its work on its own stream, so the
kernels of different problems run concurrently on the GPU.  The C ABI
releases the GIL, so the workers do not serialise on the host.  Only the C
ABI is used: sigma and the voltages cross as host arrays, and the Jacobian
stays on the device (crgpu_sens with no host buffer) unless it is asked for.

The per-worker memory budget is the free device memory divided by the number
of workers.  A problem whose band factors do not fit is processed in batches
by its own context.
"""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor
from typing import List, Optional, Sequence

import numpy as np

from . import MIXED, CRMod
from ._lib import CRGPUError, device_memory
from .crmod import forward_sens_batch


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

    def _one(self, i: int, sens_mode: Optional[int], keep_sens: bool):
        p = self.problems[i]
        with CRMod(p.grid, p.survey, precision=self.precision) as m:
            m.set_refinement(*self.refine)
            m.set_memory_budget(self.budget)
            if self.autotune:
                m.autotune(p.sigma)
            out = {"index": i, "nanz": p.survey.nanz, "elanz": p.grid.elanz}
            out["volt"] = m.forward(p.sigma)["volt"]
            if sens_mode is not None:
                if keep_sens:
                    out["sens"] = m.sens(int(sens_mode))
                else:
                    m.sens_on_device(int(sens_mode))
            out["stats"] = m.stats()
        return out

    def run(self, sens_mode: Optional[int] = 0, keep_sens: bool = False) -> List[dict]:
        """Runs every problem; returns one dict per problem in input order."""
        results: List[Optional[dict]] = [None] * len(self.problems)
        with ThreadPoolExecutor(max_workers=self.workers) as ex:
            for r in ex.map(lambda i: self._one(i, sens_mode, keep_sens), self.order):
                results[r["index"]] = r
        return results  # type: ignore[return-value]

    def run_batched(self, sens_mode: Optional[int] = 0, reserve_frac: float = 0.1) -> List[dict]:
        """Runs every problem in waves that fit device memory: per wave one
        crgpu_forward_sens_batch (all band factors of the wave in one
        persistent launch, longest systems first).  The contexts of a wave are
        created by the worker threads (the C ABI releases the GIL).  Problems
        the batched call does not take (bands beyond the tensor-core window)
        run one by one."""
        results: List[Optional[dict]] = [None] * len(self.problems)
        _, total = device_memory()
        reserve = int(reserve_frac * total)
        order = list(self.order)

        def create(q):
            p = self.problems[q]
            m = CRMod(p.grid, p.survey, precision=self.precision)
            m.set_refinement(*self.refine)
            return q, m, m.memory_need()

        def run_wave(wave):
            try:
                volts = forward_sens_batch([m for _, m in wave], [self.problems[q].sigma for q, _ in wave],
                                           sens_mode=-1 if sens_mode is None else int(sens_mode))
                for (q, m), v in zip(wave, volts):
                    results[q] = {"index": q, "volt": v, "stats": m.stats()}
            except CRGPUError:
                for q, m in wave:  # one by one
                    results[q] = self._one(q, sens_mode, False)
            finally:
                for _, m in wave:
                    m.close()

        with ThreadPoolExecutor(max_workers=self.workers) as ex:
            i = 0
            while i < len(order):
                wave, pending = [], 0
                while i < len(order):
                    made = list(ex.map(create, order[i:i + self.workers]))
                    free, _ = device_memory()  # the contexts made so far hold their own memory
                    stop = False
                    for q, m, need in made:
                        if stop or (wave and need + pending > free - reserve):
                            m.close()
                            stop = True
                            continue
                        wave.append((q, m))
                        pending += need
                        i += 1
                    if stop:
                        break
                run_wave(wave)
        return results  # type: ignore[return-value]
