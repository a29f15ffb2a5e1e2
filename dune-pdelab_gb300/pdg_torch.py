"""PyTorch autograd wrapper of the GPU DG solve and its hand-written adjoint.

``solve_dg(logK, fc, problem)`` returns u(logK, fc), the solution of the SIPG
problem R(u; K, f) = 0 (StationaryLinearProblemSolver semantics).  Its
backward pass runs one adjoint Krylov solve J^T lambda = dL/du
(pdg_adjoint_solve) and the fused per-cell gradient kernels
(pdg_grad_logK, pdg_grad_source):

    dL/dlogK_e = -lambda^T dR/dlogK_e,      dL/dfc_e = -lambda^T dR/dfc_e.

Everything stays on the GPU; tensors are float64 CUDA tensors.
"""
from __future__ import annotations

import torch

import pdg


class DGProblem:
    """A GridOperator plus solver options used by ``solve_dg``."""

    def __init__(self, go: "pdg.GridOperator", method=pdg.CG, preconditioner=pdg.PREC_BJ_FDM,
                 reduction=1e-12, mixed=True, inner_reduction=1e-3, maxit=20000,
                 inner_maxit=None):
        self.go = go
        self.opts = pdg.default_options(method=method, preconditioner=preconditioner,
                                        reduction=reduction, mixed=int(mixed),
                                        inner_reduction=inner_reduction, maxit=maxit,
                                        inner_maxit=inner_maxit or maxit, max_outer=60)
        self.last_forward = None
        self.last_adjoint = None

    def forward_solve(self, logK, fc):
        go = self.go
        go.set_permeability(logK.detach().contiguous(), is_log=True)
        if fc is not None:
            go.set_source(fc=fc.detach().cpu().numpy())
        u = torch.zeros(go.ndof, dtype=torch.float64, device=logK.device)
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=self.opts.method,
                                                 preconditioner=self.opts.preconditioner,
                                                 maxiter=self.opts.maxit,
                                                 mixed=bool(self.opts.mixed),
                                                 inner_reduction=self.opts.inner_reduction)
        ls.opts.inner_maxit = self.opts.inner_maxit
        ls.opts.max_outer = self.opts.max_outer
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, self.opts.reduction)
        slp.apply()
        self.last_forward = slp.result().as_dict()
        if not slp.result().converged:
            raise pdg.PDGError(pdg.PDG_ENOTCONVERGED, "forward solve did not converge")
        return u


class _SolveDG(torch.autograd.Function):
    @staticmethod
    def forward(ctx, logK, fc, problem):
        u = problem.forward_solve(logK, fc)
        ctx.problem = problem
        ctx.has_fc = fc is not None
        ctx.save_for_backward(u, logK)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        u, logK = ctx.saved_tensors
        problem = ctx.problem
        go = problem.go
        # the operator must be the one of the forward solve
        go.set_permeability(logK.detach().contiguous(), is_log=True)
        lam = torch.zeros_like(u)
        res = go.adjoint_solve(grad_u.contiguous(), lam, problem.opts)
        problem.last_adjoint = res.as_dict()
        if not res.converged:
            raise pdg.PDGError(pdg.PDG_ENOTCONVERGED, "adjoint solve did not converge")
        g = torch.zeros(go.ncell, dtype=torch.float64, device=u.device)
        go.grad_logK(u, lam, g)
        gf = None
        if ctx.has_fc:
            gf = torch.zeros(go.ncell, dtype=torch.float64, device=u.device)
            go.grad_source(lam, gf)
        return g, gf, None


def solve_dg(logK, fc, problem: DGProblem):
    """u = solve(logK, fc); differentiable w.r.t. logK and fc (None = keep the
    source set on the problem's GridOperator)."""
    return _SolveDG.apply(logK, fc, problem)
