"""Nonlinear operator (NonlinearConvectionDiffusionDG: + int q(u) psi) and
Newton (NewtonMethod with Hackbusch-Reusken line search) on the GPU against
the oracle, including the reference's matrix_free_nonlinear test problem."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def pdg():
    import __graft_entry__
    __graft_entry__.build()
    import pdg as m
    return m


def _pair(pdg, oracle, dim, k, nc, seed, coef=(0.3, -0.5, 2.0), method=1, react=False):
    rng = np.random.default_rng(seed)
    ncell = int(np.prod(nc))
    K = np.exp(0.5 * rng.standard_normal(ncell))
    go = pdg.GridOperator(dim, k, nc, alpha=3.0, method=method)
    go.set_permeability(K)
    P = oracle.Problem(dim, k, nc, alpha=3.0, method=method, K=K)
    if react:
        c = rng.uniform(0.5, 1.5, ncell)
        go.set_reaction(c)
        P.set(c=c)
    go.set_nonlinearity(list(coef))
    P.set_nonlinearity(list(coef))
    return go, P, rng


@pytest.mark.parametrize("dim,k,nc", [(2, 1, (5, 4)), (2, 3, (3, 3)), (3, 2, (3, 4, 2)),
                                      (3, 4, (2, 2, 2))])
def test_nonlinear_residual_and_jacobian(pdg, oracle, dim, k, nc):
    go, P, rng = _pair(pdg, oracle, dim, k, nc, seed=41 + k, react=True)
    x = rng.uniform(-1, 1, go.ndof)
    z = rng.uniform(-1, 1, go.ndof)
    r = go.residual(x, np.zeros(go.ndof))
    assert _rel(r, P.residual(x)) <= 1e-12
    y = go.jacobian_apply_nonlinear(x, z, np.zeros(go.ndof))
    P.set_linearization_point(x)
    assert _rel(y, P.jacobian_apply(z)) <= 1e-12
    # assembled blocks at the linearization point
    go.jacobian_assemble()
    ours = go.matrix_apply(z, np.zeros(go.ndof))
    assert _rel(ours, P.blocks_apply(P.assemble_jacobian(), z)) <= 1e-12


def test_nonlinear_jacobian_f32_and_transpose(pdg, oracle):
    import torch
    go, P, rng = _pair(pdg, oracle, 3, 2, (5, 4, 3), seed=47, method=0)
    x = rng.uniform(-1, 1, go.ndof)
    z = rng.uniform(-1, 1, go.ndof)
    go.set_linearization_point(x)
    P.set_linearization_point(x)
    zt = torch.tensor(z, dtype=torch.float32, device="cuda")
    yt = torch.zeros(go.ndof, dtype=torch.float32, device="cuda")
    go.jacobian_apply_f32(zt, yt)
    torch.cuda.synchronize()
    assert _rel(yt.cpu().double().numpy(), P.jacobian_apply(z)) <= 2e-5
    y = go.jacobian_apply_transpose(z, np.zeros(go.ndof))
    assert _rel(y, P.blocks_apply(P.assemble_jacobian(), z, transpose=True)) <= 1e-12


def _reference_problem(pdg, oracle, n=16):
    # matrix_free_nonlinear.cc:24-70: q(u) = mu u^2 (mu = 2), g = |x|^2 on
    # the whole boundary, f = -4 + mu g^2; 2D Q1, SIPG, weightsOn, alpha 3
    go = pdg.GridOperator(2, 1, (n, n), alpha=3.0)
    P = oracle.Problem(2, 1, (n, n), alpha=3.0)
    for obj in (go, P):
        obj.set_nonlinearity([0.0, 0.0, 2.0])
    xv = go.volume_points().reshape(-1, 2)
    g = (xv ** 2).sum(1)
    fq = -4.0 + 2.0 * g * g
    xb = go.boundary_points().reshape(-1, 2)
    gb = (xb ** 2).sum(1)
    go.set_source(fq=fq)
    go.set_boundary_data(g=gb)
    P.set(fq=fq, gq=gb)
    return go, P


@pytest.mark.parametrize("kind", [2, 16 | 2, 16 | 3])
def test_newton_reference_problem(pdg, oracle, kind):
    go, P = _reference_problem(pdg, oracle)
    uref, rres, st = P.newton(oracle.prec_config(kind), solver="bicgstab")
    assert st == 0 and rres.converged
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB, preconditioner=kind)
    u = np.zeros(go.ndof)
    nm = pdg.NewtonMethod(go, ls)
    nm.apply(u)
    r = nm.result()
    assert r.converged and r.iterations == rres.iterations
    assert abs(r.linear_solver_iterations - rres.linear_iterations) <= 10
    # both stop at the Newton reduction 1e-8: agreement to that level
    assert _rel(u, uref) <= 1e-6
    # the reference test's own assertion: L2 error^2 against g = |x|^2 below 1e-6
    xyz, w, val = P.eval_points(u, 6)
    err2 = float((w * (val - (xyz ** 2).sum(-1)) ** 2).sum())
    assert err2 < 1e-6


def test_newton_mixed_3d(pdg, oracle):
    # 3D Q2, q = u + u^3, FP32 inner solves with block SOR
    go, P, rng = _pair(pdg, oracle, 3, 2, (4, 4, 4), seed=53, coef=(0.0, 1.0, 0.0, 1.0))
    go.set_source(fc=5.0 * np.ones(go.ncell))
    P.set(fc=5.0 * np.ones(go.ncell))
    uref, rres, st = P.newton(oracle.prec_config(2), solver="bicgstab", reduction=1e-10)
    assert st == 0 and rres.converged
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                             preconditioner=pdg.PREC_SOR | pdg.PREC_BJ_DENSE,
                                             mixed=True, inner_reduction=1e-1)
    ls.opts.inner_maxit = 30
    u = np.zeros(go.ndof)
    nm = pdg.NewtonMethod(go, ls, reduction=1e-10)
    nm.apply(u)
    assert nm.result().converged
    assert _rel(u, uref) <= 1e-7


def test_newton_errors(pdg):
    go = pdg.GridOperator(2, 1, (4, 4))
    with pytest.raises(pdg.PDGError):
        go.set_nonlinearity([1.0, 2.0, 3.0, 4.0, 5.0, 6.0])
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB, preconditioner=2)
    with pytest.raises(pdg.PDGError):
        pdg.NewtonMethod(go, ls, max_iterations=0).apply(np.zeros(go.ndof))
