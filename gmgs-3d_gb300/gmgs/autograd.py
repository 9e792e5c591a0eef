"""torch.autograd.Function over the libgmgs adjoint (extension beyond the
reference, which has no density field and no gradients).

    J = compliance(rho, solver)                 # F^T U(rho)
    J = displacement_functional(rho, solver, ell)   # ell^T U(rho)
    J.backward()                                # rho.grad = dJ/drho from gmgs_grad

The forward pass sets the per-voxel stiffness scale rho^penal on the finest
level (gmgs_set_density), solves with the handle's PCG and returns J; the
backward pass calls gmgs_grad, which for compliance uses U itself and for a
displacement functional solves the adjoint system K lambda = ell with the same
PCG, then reduces -penal rho^(penal-1) lambda_e^T Ke0 u_e per voxel on the GPU.
The handle keeps the state of the last forward pass, so call backward before
the next forward on the same solver.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Solver


class _Functional(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho: torch.Tensor, solver: Solver, penal: float, ell):
        r = rho.detach().to("cpu", torch.float64).numpy().ravel()
        solver.set_density(r, penal)
        u = solver.solve()
        if ell is None:
            J = float(solver.load_vector() @ u)
        else:
            J = float(np.asarray(ell, dtype=np.float64).ravel() @ u)
        ctx.solver = solver
        ctx.ell = ell
        ctx.rho_meta = (rho.shape, rho.dtype, rho.device)
        return torch.tensor(J, dtype=rho.dtype, device=rho.device)

    @staticmethod
    def backward(ctx, gout):
        shape, dtype, device = ctx.rho_meta
        g = ctx.solver.grad(ctx.ell)
        grad = torch.as_tensor(g, dtype=dtype, device=device).reshape(shape) * gout
        return grad, None, None, None


def compliance(rho: torch.Tensor, solver: Solver, penal: float = 3.0) -> torch.Tensor:
    """F^T U for the stiffness scale rho^penal (one entry per solid voxel)."""
    return _Functional.apply(rho, solver, penal, None)


def displacement_functional(rho: torch.Tensor, solver: Solver, ell, penal: float = 3.0) -> torch.Tensor:
    """ell^T U; ell is a 3*num_nodes interleaved vector (e.g. one tip DOF)."""
    return _Functional.apply(rho, solver, penal, ell)
