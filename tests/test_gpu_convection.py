"""Convection-diffusion-reaction (upwind DG, config C5 at test size):
the CUDA operator with a divergence-free Fourier velocity against the oracle."""
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


def _pair(pdg, oracle, k, n, seed, method=1, bct=None, react=True):
    rng = np.random.default_rng(seed)
    nc = (n,) * 3 if np.isscalar(n) else tuple(n)
    ncell = int(np.prod(nc))
    K = np.exp(rng.standard_normal(ncell))
    c = np.ones(ncell) if react else None
    modes = pdg.fourier_velocity_modes(seed)
    go = pdg.GridOperator(3, k, nc, alpha=3.0, method=method, bctype=bct)
    go.set_permeability(K)
    if react:
        go.set_reaction(c)
    go.set_velocity_modes(modes)
    P = oracle.Problem(3, k, nc, alpha=3.0, method=method, bctype=bct, K=K, c=c, modes=modes)
    return go, P, rng


def test_velocity_is_divergence_free_and_bounded(pdg):
    m = pdg.fourier_velocity_modes(5)
    assert np.allclose((m[:, :3] * m[:, 4:]).sum(1), 0)
    assert np.linalg.norm(m[:, 4:], axis=1).sum() <= 10 + 1e-12


@pytest.mark.parametrize("k,n", [(1, 4), (2, 3), (3, 3), (4, 2), (2, (4, 3, 2))])
def test_convection_apply_f64(pdg, oracle, k, n):
    go, P, rng = _pair(pdg, oracle, k, n, seed=40 + k)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x, y0.copy())) <= 1e-12


@pytest.mark.parametrize("method", [0, 1])
def test_convection_transpose(pdg, oracle, method):
    go, P, rng = _pair(pdg, oracle, 2, 3, seed=50 + method, method=method)
    A = P.assemble_jacobian()
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, y)
    assert _rel(y, P.blocks_apply(A, x, transpose=True)) <= 1e-12


def test_convection_f32_and_boundary_types(pdg, oracle):
    import torch
    bct = [1, -1, 1, -3, 1, -1]
    go, P, rng = _pair(pdg, oracle, 3, 3, seed=61, bct=bct)
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply(x, y)
    yref = P.jacobian_apply(x)
    assert _rel(y, yref) <= 1e-12
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    yt = torch.zeros_like(xt)
    go.jacobian_apply_f32(xt, yt)
    torch.cuda.synchronize()
    assert _rel(yt.cpu().double().numpy(), yref) <= 2e-5


def test_outflow_on_inflow_is_an_error(pdg):
    # every side outflow: b.n < 0 somewhere -> PDG_EOUTFLOW (convectiondiffusiondg.hh:802-806)
    go = pdg.GridOperator(3, 2, (3, 3, 3), bctype=[-2] * 6)
    with pytest.raises(pdg.PDGError) as e:
        go.set_velocity_modes(pdg.fourier_velocity_modes(1))
    assert e.value.status == pdg.PDG_EOUTFLOW


def test_convection_residual_with_inflow_data(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 2, 3, seed=71)
    g = rng.standard_normal(go.nq_boundary)
    fc = rng.standard_normal(go.ncell)
    go.set_boundary_data(g=g)
    go.set_source(fc=fc)
    P.set(gq=g, fc=fc)
    x = rng.uniform(-1, 1, go.ndof)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= 1e-12


def test_convection_block_jacobi_dense(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 2, 3, seed=81)
    lu, piv = P.lu(P.block_diagonal())
    d = rng.uniform(-1, 1, go.ndof)
    prec = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE)
    prec.pre()
    v = np.zeros(go.ndof)
    prec.apply(v, d)
    assert _rel(v, P.lu_apply(lu, piv, d)) <= 1e-10


@pytest.mark.parametrize("mixed", [False, True])
def test_convection_bicgstab_solve(pdg, oracle, mixed):
    go, P, rng = _pair(pdg, oracle, 2, 4, seed=91)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="bicgstab", op=0, reduction=1e-10)
    assert rres.converged
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                             preconditioner=pdg.PREC_BJ_DENSE, mixed=mixed)
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    assert ls.result().converged
    if not mixed:
        assert abs(ls.result().iterations - rres.iterations) <= 1
    assert _rel(u, uref) <= 1e-8


@pytest.mark.parametrize("mixed", [False, True])
def test_gmres_solve_nonsymmetric(pdg, oracle, mixed):
    # restarted GMRES(m) as the outer (FP64) and as the inner (FP32) method
    go, P, rng = _pair(pdg, oracle, 2, 4, seed=93, method=0)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="bicgstab", op=0, reduction=1e-12)
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.GMRES if not mixed else pdg.BICGSTAB,
                                             preconditioner=pdg.PREC_BJ_DENSE, mixed=mixed)
    ls.opts.restart = 20
    ls.opts.inner_method = pdg.GMRES
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    assert ls.result().converged
    assert _rel(u, uref) <= 1e-8


@pytest.mark.parametrize("mode,inner", [(2, 1), (3, 1), (3, 2), (1, 1)])
def test_mixed_outer_modes(pdg, oracle, mode, inner):
    # mixed = 2: FP64 defect correction; 3 (and 1 for BiCGStab): FP64 flexible
    # GMRES whose preconditioner is a short FP32 inner solve
    go, P, rng = _pair(pdg, oracle, 2, 4, seed=95)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="bicgstab", op=0, reduction=1e-12)
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                             preconditioner=pdg.PREC_BJ_DENSE, mixed=True,
                                             inner_reduction=1e-1)
    ls.opts.mixed = mode
    ls.opts.inner_method = inner
    ls.opts.inner_maxit = 20
    ls.opts.restart = 10
    ls.opts.max_outer = 40
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    r = ls.result()
    assert r.converged and r.outer_iterations >= 1 and r.iterations >= r.outer_iterations
    assert _rel(u, uref) <= 1e-8


def test_mixed_flexible_adjoint_solve(pdg, oracle):
    # J^T lam = rhs with the flexible outer loop (transposed FP32 operator and
    # block Jacobi inside), checked through the FP64 transposed operator
    go, P, rng = _pair(pdg, oracle, 2, 3, seed=97)
    rhs = rng.uniform(-1, 1, go.ndof)
    o = pdg.default_options(method=pdg.BICGSTAB, preconditioner=pdg.PREC_BJ_DENSE,
                            reduction=1e-11, mixed=3, inner_reduction=1e-1, inner_maxit=20,
                            max_outer=40, restart=20)
    lam = np.zeros(go.ndof)
    res = go.adjoint_solve(rhs, lam, o)
    assert res.converged and res.outer_iterations >= 1
    A = P.assemble_jacobian()
    assert _rel(P.blocks_apply(A, lam, transpose=True), rhs) <= 1e-9


def test_dense_block_jacobi_fp16_storage(pdg, oracle):
    # FP32 dense block Jacobi with the inverses stored in FP16 (one FP32 scale
    # per block): within FP16 rounding of the FP32 inverse, and the mixed
    # BiCGStab solve that uses it for its inner solves reaches the FP64 solution
    import torch
    go, P, rng = _pair(pdg, oracle, 3, (4, 4, 3), seed=81)
    go.set_source(fc=np.ones(go.ncell))
    d = torch.tensor(rng.uniform(-1, 1, go.ndof), dtype=torch.float32, device="cuda")
    out = {}
    for half in (0, 1):
        go.set_prec_options(dense_fp16=half)
        prec = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE, precision=pdg.F32)
        prec.pre()
        v = torch.zeros_like(d)
        torch.cuda.synchronize()
        prec.apply(v, d)
        torch.cuda.synchronize()
        out[half] = v.cpu().double().numpy()
    assert _rel(out[1], out[0]) <= 4e-3
    assert _rel(out[1], out[0]) > 0          # the FP16 path really ran
    # mixed solve (FP64 flexible GMRES around FP32 BiCGStab) with FP16 blocks
    go.set_prec_options(dense_fp16=1)
    sols = {}
    for mixed in (0, 1):
        pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE,
                                       precision=pdg.F32 if mixed else pdg.F64).pre()
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                                 preconditioner=pdg.PREC_BJ_DENSE, mixed=mixed,
                                                 maxiter=5000, inner_reduction=1e-1)
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        slp.apply()
        assert slp.result().converged
        sols[mixed] = u
    assert _rel(sols[1], sols[0]) <= 1e-8
    # the transposed FP16 block apply, inside the mixed adjoint solve
    rhs = rng.uniform(-1, 1, go.ndof)
    lam = {}
    for mixed in (0, 1):
        o = pdg.default_options(method=pdg.BICGSTAB, preconditioner=pdg.PREC_BJ_DENSE,
                                reduction=1e-11, mixed=mixed, maxit=20000, inner_reduction=1e-1)
        lam[mixed] = np.zeros(go.ndof)
        assert go.adjoint_solve(rhs, lam[mixed], o).converged
    assert _rel(lam[1], lam[0]) <= 1e-8
