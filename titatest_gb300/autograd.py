"""Differentiable forward modelling: torch.autograd on top of the GPU forward.

`volt(model, sigma)` maps complex conductivities (elanz, complex128) to the
measured voltages V (nanz, complex128) of src/bvolt.f90 through
`crgpu_forward_device`.  Its backward is `crgpu_adjoint_device`: one adjoint
solve per (wavenumber, current electrode) system, reusing the forward's band
factors, and an element-wise contraction into dL/dsigma.  That is the exact
derivative of the discrete forward, including the electrode-dependent mixed
boundary that the reference's Jacobian (src/bsens.f90, src/bsensi.f90)
approximates by reciprocity.

V is holomorphic in sigma, so with PyTorch's convention for complex tensors
(gradients are conjugate Wirtinger derivatives of a real loss) the backward
returns conj(J)^T grad_V with J = dV/dsigma.

`CRTomoMisfit` is the CRTomo data term on log-conductivities m = log(sigma)
(src/update.f90: data d = -log V, weights wmatd): phi(m) = sum_i wmatd_i
|d_i(m) - dobs_i|^2.
"""
from __future__ import annotations

import numpy as np
import torch

from .crmod import CRMod  # noqa: F401  (the model type this module wraps)


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def _run_forward(model, s: torch.Tensor) -> torch.Tensor:
    if s.device.type == "cuda":
        model.set_stream(torch.cuda.current_stream(s.device).cuda_stream)
        v = torch.empty(model.survey.nanz, dtype=torch.complex128, device=s.device)
        model.forward_device(_ptr(s), _ptr(v))
    else:
        v = torch.from_numpy(np.ascontiguousarray(model.forward(s.numpy())["volt"]))
    model._autograd_id = getattr(model, "_autograd_id", 0) + 1
    return v


class _VoltFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sigma: torch.Tensor, model):
        s = sigma.detach().to(torch.complex128).resolve_conj().contiguous()
        v = _run_forward(model, s)
        ctx.model = model
        ctx.forward_id = model._autograd_id
        ctx.save_for_backward(s)
        return v

    @staticmethod
    def backward(ctx, grad_v: torch.Tensor):
        model = ctx.model
        (s,) = ctx.saved_tensors
        if getattr(model, "_autograd_id", None) != ctx.forward_id:
            _run_forward(model, s)  # another forward ran on this model since: recompute this one
        g = grad_v.to(torch.complex128).conj().resolve_conj().contiguous()  # physical conjugate
        if g.device.type == "cuda":
            grad = torch.empty(s.shape[0], dtype=torch.complex128, device=g.device)
            model.set_stream(torch.cuda.current_stream(g.device).cuda_stream)
            model.adjoint_device(_ptr(g), _ptr(grad))
        else:
            grad = torch.from_numpy(np.ascontiguousarray(model.adjoint(g.numpy())))
        return torch.conj(grad), None


def volt(model: CRMod, sigma: torch.Tensor) -> torch.Tensor:
    """Voltages V(sigma) (nanz, complex128), differentiable in sigma."""
    return _VoltFunction.apply(sigma, model)


class CRTomoMisfit(torch.nn.Module):
    """phi(m) = sum_i wmatd_i |(-log V_i(exp m)) - dobs_i|^2 on complex
    log-conductivities m (elanz), the data term of src/update.f90."""

    def __init__(self, model: CRMod, dobs, wmatd):
        super().__init__()
        self.model = model
        self.register_buffer("dobs", torch.as_tensor(np.asarray(dobs), dtype=torch.complex128))
        self.register_buffer("wmatd", torch.as_tensor(np.asarray(wmatd), dtype=torch.float64))

    def forward(self, m: torch.Tensor) -> torch.Tensor:
        v = volt(self.model, torch.exp(m))
        r = -torch.log(v) - self.dobs.to(v.device)
        return torch.sum(self.wmatd.to(v.device) * (r.real ** 2 + r.imag ** 2))
