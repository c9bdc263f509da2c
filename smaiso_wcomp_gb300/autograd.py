"""torch.autograd.Function over the C ABI, used only for gradient checks.

forward: (psi0, coeffs = [alpha, beta, gamma, nu, rho_0]) -> psi(T) after `nsteps`
FP64 steps (swc_set_state + swc_step); backward: swc_backward. Every evaluation
creates a fresh context because the coefficients are fixed at swc_create.
"""
import numpy as np
import torch

from . import abi
from .engine import Engine

COEFFS = ("alpha", "beta", "gamma", "nu", "rho_0")


def _params(base, coeffs, ckpt):
    p = abi.SwcParams.from_buffer_copy(base)
    for name, v in zip(COEFFS, coeffs):
        setattr(p, name, float(v))
    p.precision = abi.SWC_PREC_FP64
    p.adjoint_ckpt = ckpt
    return p


class StepFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi0, coeffs, base, nsteps, rho0, ckpt):
        p = _params(base, coeffs.detach().cpu().numpy(), ckpt)
        e = Engine(p)
        e.set_state(psi0.detach().cpu().numpy(), rho0)
        e.step(nsteps)
        out = torch.from_numpy(e.field("psi").copy())
        ctx.engine = e
        return out

    @staticmethod
    def backward(ctx, grad_out):
        e = ctx.engine
        g = e.backward(dpsi=grad_out.detach().cpu().numpy())
        gc = torch.tensor([g[n] for n in COEFFS], dtype=torch.float64)
        return torch.from_numpy(g["psi0"]), gc, None, None, None, None
