"""The GL free energy as a differentiable PyTorch function.

``GLEnergy(problem, n_images)(a, psi_1, psi_2, theta)`` returns the per-image
free energies (float64, shape (F,)) of fields held in CUDA tensors of shape
(F, ny, nx, 2) in the reference's device layout.  The forward pass is the
library's energy kernel (computeFreeEnergy, mepgl/src/nlcg.cu:217-240); the
backward pass is its hand-written gradient kernel (gradientPsi / gradientA,
nlcg.cu:504-888) scaled by the incoming per-image weights, and the
parameter-adjoint kernel for ``theta``:

* ``theta`` = (H_shift, eta, gamma), float64, shape (3,): a uniform shift
  added to the problem's applied field h, and the couplings eta and gamma.
  ``None`` means (0, problem.eta, problem.gamma) and no parameter gradient.

There is no PyTorch fallback: every number comes from libmepgl_gb300.so.
"""
from __future__ import annotations

import numpy as np
import torch

from . import native
from .problem import Problem


class GLEnergy:
    """Per-image GL free energy F_n(A, psi; H_shift, eta, gamma) on the GPU."""

    def __init__(self, prob: Problem, n_images: int, precision: str = "fp64", **options):
        self.prob = prob
        self.F = int(n_images)
        self.precision = precision
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.options = options
        self._key = None
        self._ctx = None

    def context(self, theta=None) -> native.StringContext:
        """The library context for parameters theta (rebuilt when they change)."""
        key = (0.0, float(self.prob.eta), float(self.prob.gamma)) if theta is None else \
            tuple(float(v) for v in theta)
        if key != self._key:
            if self._ctx is not None:
                self._ctx.close()
            p = self.prob.with_(h=self.prob.h + key[0], eta=key[1], gamma=key[2])
            self._ctx = native.StringContext(p, self.F, self.precision, **self.options)
            self._key = key
        return self._ctx

    def __call__(self, a, psi_1, psi_2=None, theta=None):
        if theta is None:
            theta_t = torch.tensor([0.0, self.prob.eta, self.prob.gamma], dtype=torch.float64)
        else:
            theta_t = theta
        return _FreeEnergy.apply(a, psi_1, psi_2, theta_t, self)

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None
            self._key = None


def _check_fields(g: GLEnergy, tensors):
    shape = (g.F, g.prob.ny, g.prob.nx, 2)
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda or t.dtype != g.dtype or tuple(t.shape) != shape or not t.is_contiguous():
            raise ValueError(f"fields must be contiguous CUDA {g.dtype} tensors of shape {shape}")


def _load(g: GLEnergy, theta, a, p1, p2) -> native.StringContext:
    c = g.context(theta.detach().cpu().numpy())
    torch.cuda.current_stream().synchronize()      # the library works on its own stream
    c.set_state_device(a.data_ptr(), p1.data_ptr(), None if p2 is None else p2.data_ptr())
    return c


class _FreeEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, psi_1, psi_2, theta, g: GLEnergy):
        if g.prob.multicomponent and psi_2 is None:
            raise ValueError("two-component problem needs psi_2")
        psi_2 = psi_2 if g.prob.multicomponent else None
        _check_fields(g, (a, psi_1, psi_2))
        c = _load(g, theta, a, psi_1, psi_2)
        e = c.compute_free_energy()
        ctx.g = g
        ctx.save_for_backward(a, psi_1, psi_2, theta)
        return torch.from_numpy(e).to(a.device)

    @staticmethod
    def backward(ctx, grad_out):
        a, p1, p2, theta = ctx.saved_tensors
        g: GLEnergy = ctx.g
        c = _load(g, theta, a, p1, p2)
        w = grad_out.detach().to(torch.float64)
        ga = gp1 = gp2 = gth = None
        need_fields = ctx.needs_input_grad[0] or ctx.needs_input_grad[1] or ctx.needs_input_grad[2]
        if need_fields:
            ta, t1 = torch.empty_like(a), torch.empty_like(p1)
            t2 = torch.empty_like(p2) if p2 is not None else None
            c.energy_grad_device(ta.data_ptr(), t1.data_ptr(), None if t2 is None else t2.data_ptr(),
                                 with_energy=False)
            scale = w.to(device=a.device, dtype=a.dtype).view(-1, 1, 1, 1)
            ga = ta * scale if ctx.needs_input_grad[0] else None
            gp1 = t1 * scale if ctx.needs_input_grad[1] else None
            gp2 = t2 * scale if (t2 is not None and ctx.needs_input_grad[2]) else None
        if ctx.needs_input_grad[3]:
            adj = torch.from_numpy(np.ascontiguousarray(c.param_adjoint()))   # (F, 3)
            gth = (w.cpu().view(-1, 1) * adj).sum(0).to(theta.device, theta.dtype)
        return ga, gp1, gp2, gth, None
