"""Run one forward (and optionally the Jacobian) of a synthetic configuration.

A small driver for profilers (ncu) and quick timing:

    python -m titatest_gb300.profile_case --config 2 --precision mixed \
        --batch 152 --repeat 1 [--sens]

--batch limits the number of band systems per batch (one factor launch per
batch), so a profiler can capture a single launch of known size.
--update-steps N adds the CRTomo Jacobian (bsensi, kept on the device) and one
Gauss-Newton update with at most N CG steps (structured smoothness) on data
that are the model's response times 1.03: the CG kernels for a profiler;
--mcm then also times the model uncertainty (crgpu_mcm).
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from . import MIXED, PLAIN, CRMod, synth


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--precision", choices=["mixed", "plain"], default="mixed")
    ap.add_argument("--batch", type=int, default=0, help="systems per batch (0: as many as fit)")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--sens", action="store_true")
    ap.add_argument("--refine-tol", type=float, default=1e-8)
    ap.add_argument("--update-steps", type=int, default=0)
    ap.add_argument("--mcm", action="store_true", help="with --update-steps: time crgpu_mcm (uncertainty)")
    a = ap.parse_args(argv)
    s = synth.make(a.config)
    prec = MIXED if a.precision == "mixed" else PLAIN
    with CRMod(s.grid, s.survey, precision=prec) as m:
        m.set_refinement(8, a.refine_tol)
        if a.batch:
            g = s.grid
            esz = 8 if prec == MIXED else 16
            per = g.sanz * (g.mb + 1) * esz + (g.sanz * 12 * 16) + g.sanz * 8 + g.sanz * (3 * 16 + esz) + 64
            m.set_memory_budget(int(per * a.batch + per // 2))
        for _ in range(a.repeat):
            t = time.time()
            out = m.forward(s.sigma)
            st = m.stats()
            msg = f"forward {1e3 * (time.time() - t):.1f} ms, batches {st['nbatches']}, factor {st['ms_factor']:.1f} ms, " \
                  f"solve {st['ms_solve']:.1f} ms, refinement {st['refine_iterations']}"
            if a.sens:
                J = m.sens(0)
                msg += f", sens {m.stats()['ms_sens']:.1f} ms, |J|max {np.abs(J).max():.3e}"
            print(msg, flush=True)
        assert np.all(np.isfinite(out["volt"]))
        if a.update_steps:
            from . import regularization as R
            sa = m.forward(s.sigma, volt_mode=1)["sigmaa"]
            m.sens_on_device(1)
            dat = sa - np.log(1.03)
            w = np.full(len(sa), 1.0 / 0.03 ** 2)
            sm = R.bsmatmreg(s.grid, s.nx, s.nz)
            t = time.time()
            _, dpar, _, _, ncg = m.update(w, np.ones(len(sa), np.int32), dat, sa, 0, sm, nx=s.nx, lam=300.0,
                                          eps=1e-4, ncgmax=a.update_steps, par=np.log(s.sigma))
            print(f"update {1e3 * (time.time() - t):.1f} ms, {ncg} CG steps, |dpar|max {np.abs(dpar).max():.3e}",
                  flush=True)
            if a.mcm:
                t = time.time()
                d = m.mcm(w, np.ones(len(sa), np.int32), 0, sm, nx=s.nx, lam=300.0)
                print(f"mcm {1e3 * (time.time() - t):.1f} ms for manz {len(d['cov1'])} (ata, ata_reg, Cholesky "
                      f"inverse, resolution, cov2), min cov1 {d['cov1'].min():.3e}", flush=True)


if __name__ == "__main__":
    main()
