"""torch.autograd bridge for the adjoint gradient (smat_fdtd_adjoint_grad).

A thin Function: forward runs the FDTD and its adjoint once (the C ABI does
both) and returns J; backward hands back dJ/d eps_r of the design cells.
Tensors are plumbing only -- the work runs in the library's CUDA kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import fdtd as F
from . import workloads as W


def _plan(design: W.Design, eps, precision, nsteps, src, phase, mode, dt_factor):
    s = design.with_eps(eps)
    pr = W.prepare(s, dt_factor=dt_factor)
    p = F.Plan.create(s.L, s.iBc, (design.iB, design.iT, design.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi,
                      pr.sigma, precision=precision, batch=1)
    Hinc, Einc = mode
    p.set_incident(0, Hinc, Einc)
    p.set_schedule(src[:nsteps], planes=(design.iB, design.iT), phase=phase[:nsteps])
    return p


def objective_and_grad(design: W.Design, eps, *, precision=F.FP32, nsteps=6000, K=64, mode=None, src=None,
                       phase=None, dt_factor=1.0 / 0.99, autotune=True):
    """J = |overlap of the output-port DFT with `mode`|^2 and dJ/d eps_r (design box).
    autotune: pick the FP32 forward's launch form (cached per grid and GPU)."""
    eps = np.asarray(eps, dtype=np.float64)
    p = _plan(design, eps, precision, nsteps, src, phase, mode, dt_factor)
    try:
        if autotune and precision == F.FP32:
            p.autotune(4)
        Hinc, Einc = mode
        t = np.concatenate([Hinc[0::2], Hinc[1::2], -Einc[1::2], Einc[0::2]])
        J, g, _ = p.adjoint_grad(nsteps, K, 0, 1, t, design.box)
    finally:
        p.close()
    return J, g / eps


class PortOverlap(torch.autograd.Function):
    """J(eps) for a Design; eps is a (nz, ny, nx) float64 tensor of eps_r."""

    @staticmethod
    def forward(ctx, eps, design, kwargs):
        J, dJ = objective_and_grad(design, eps.detach().cpu().numpy(), **kwargs)
        ctx.save_for_backward(torch.from_numpy(dJ).to(eps.device))
        return torch.tensor(J, dtype=torch.float64, device=eps.device)

    @staticmethod
    def backward(ctx, gJ):
        (dJ,) = ctx.saved_tensors
        return gJ * dJ, None, None
