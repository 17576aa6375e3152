"""Differentiable linear-elastic solve: u = K(E)^-1 P f on the GPU.

Forward: assemble K from per-tet Young's moduli (clamped DOFs: identity rows
and columns, as SetFixedBC makes them), ILU(0), and solve K u = P f (P zeroes
the clamped DOFs of the load). Backward (hand-written adjoint, no reference
counterpart): K is symmetric, so lam = K^-1 dL/du is one more solve on the
SAME factors; then
    dL/df   = P lam
    dL/dE_e = -(P lam)_e^T (dK_e/dE_e) u_e        (K_e is linear in E_e)
with the element term computed by dfm2g_tetmesh_dLdE.
"""
from __future__ import annotations

import torch

from .ls import Solve_PCG, Solve_PCG_Mixed
from .problem import StaticElasticProblem


def _solve(P: StaticElasticProblem, rhs: torch.Tensor, precision: str, tol: float) -> torch.Tensor:
    x = torch.zeros_like(rhs)
    if precision == "fp64":
        r = rhs.clone()
        Solve_PCG(r, x, tol, 100000, P.K, P.ilu)
    elif precision in ("mixed", "reliable", "restart"):
        method = "restart" if precision == "restart" else "reliable"
        Solve_PCG_Mixed(rhs, x, tol, P.K, P.ilu, inner_tol=1e-4, method=method)
    else:
        raise ValueError(f"unknown precision {precision!r}")
    return x


class LinearElasticSolve(torch.autograd.Function):
    """u = K(E)^-1 P f. Inputs: young (ntet,) and f (ndof,), float64 CUDA tensors."""

    @staticmethod
    def forward(ctx, young, f, problem: StaticElasticProblem, precision: str = "mixed", tol: float = 1e-10):
        P = problem
        P.assemble_stiffness(young.detach().contiguous())
        if not P.factor():
            raise RuntimeError("ILU(0): more than 10 singular pivots")
        mask = P.free_mask(f)
        u = _solve(P, (f.detach() * mask).contiguous(), precision, tol)
        ctx.problem, ctx.precision, ctx.tol = P, precision, tol
        ctx.token = object()
        P._factored_for = ctx.token  # the factors in P now belong to this forward
        ctx.save_for_backward(young, u, mask)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        P = ctx.problem
        young, u, mask = ctx.saved_tensors
        if getattr(P, "_factored_for", None) is not ctx.token:
            # another forward re-assembled K since: rebuild this forward's factors
            P.assemble_stiffness(young.detach().contiguous())
            P.factor()
            P._factored_for = ctx.token
        lam = _solve(P, grad_u.detach().contiguous(), ctx.precision, ctx.tol)
        lam_free = (lam * mask).contiguous()
        grad_E = None
        if ctx.needs_input_grad[0]:
            grad_E = torch.zeros_like(young)
            P.mesh.dLdE(P.nu, u.contiguous(), lam_free, grad_E)
        grad_f = lam_free if ctx.needs_input_grad[1] else None
        return grad_E, grad_f, None, None, None


def linear_elastic_solve(young, f, problem: StaticElasticProblem, precision: str = "mixed", tol: float = 1e-10):
    """Differentiable u = K(E)^-1 P f (see LinearElasticSolve)."""
    return LinearElasticSolve.apply(young, f, problem, precision, tol)
