"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances: FP64 operator results <= 1e-12 relative (max-norm); FP32
operator results <= 2e-5 relative; solves to 1e-10 agree to 1e-8 relative;
mixed-precision solves to 1e-10 agree with the FP64 solution to 1e-8.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def pdg():
    import __graft_entry__
    __graft_entry__.build()
    import pdg as m
    return m


def _pair(pdg, oracle, dim, k, n, seed=0, method=1, weights=0, alpha=3.0, bctype=None,
          react=False, K=True):
    rng = np.random.default_rng(seed)
    nc = (n,) * dim if np.isscalar(n) else tuple(n)
    ncell = int(np.prod(nc))
    Kv = np.exp(rng.standard_normal(ncell)) if K else np.ones(ncell)
    c = rng.uniform(0.5, 2.0, ncell) if react else None
    go = pdg.GridOperator(dim, k, nc, method=method, weights=weights, alpha=alpha, bctype=bctype)
    go.set_permeability(Kv)
    if react:
        go.set_reaction(c)
    P = oracle.Problem(dim, k, nc, method=method, weights=weights, alpha=alpha, bctype=bctype,
                       K=Kv, c=c)
    return go, P, rng


CASES = [(2, 1, 6), (2, 2, 5), (2, 3, 4), (2, 4, 3), (3, 1, 4), (3, 2, 3), (3, 3, 3), (3, 4, 2),
         (3, 2, (5, 3, 2))]


@pytest.mark.parametrize("dim,k,n", CASES)
def test_jacobian_apply_f64(pdg, oracle, dim, k, n):
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=dim * 10 + k)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply(x, y)                       # accumulate semantics
    yref = P.jacobian_apply(x, y0.copy())
    assert _rel(y, yref) <= TOL64


@pytest.mark.parametrize("dim,k,n,conv", [(2, 2, 5, False), (3, 2, 3, False), (3, 3, 3, True)])
def test_on_the_fly_operator_apply_and_applyscaleadd(pdg, oracle, dim, k, n, conv):
    """OnTheFlyOperator (seqistlsolverbackend.hh:66-90): apply(x, y) sets
    y = J x; applyscaleadd(alpha, x, y) adds alpha J x to y (the reference's
    temp = J x; y += alpha temp)."""
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=40 + dim * k, react=conv)
    if conv:
        m = pdg.fourier_velocity_modes(4)
        go.set_velocity_modes(m)
        P.set_modes(m)
    op = pdg.OnTheFlyOperator(go)
    x = rng.uniform(-1, 1, go.ndof)
    Jx = P.jacobian_apply(x)
    y = rng.uniform(-1, 1, go.ndof)
    op.apply(x, y)                                # overwrites y
    assert _rel(y, Jx) <= TOL64
    for alpha in (-0.7, 2.5):
        y0 = rng.uniform(-1, 1, go.ndof)
        y = y0.copy()
        op.applyscaleadd(alpha, x, y)
        ref = y0 + alpha * Jx
        assert float(np.max(np.abs(y - ref))) <= TOL64 * float(np.max(np.abs(alpha * Jx)))
    # the transposed apply of the convection operator against the oracle's
    # matrix-free transpose
    yt = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, yt)
    assert _rel(yt, P.jacobian_apply_transpose(x)) <= TOL64


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("weights", [0, 1])
def test_methods_and_weights(pdg, oracle, method, weights):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=method * 2 + weights, method=method,
                       weights=weights, react=True)
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x)) <= TOL64


@pytest.mark.parametrize("bct", [[1, -1, 1, -3, -1, 1], [-1, -1, -1, -1, 1, 1],
                                 [-3, 1, -1, 1, 1, -3]])
def test_boundary_types(pdg, oracle, bct):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=5, bctype=bct)
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x)) <= TOL64


@pytest.mark.parametrize("method", [0, 1, 2])
def test_transpose_apply(pdg, oracle, method):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=11, method=method, weights=method % 2,
                       react=True)
    A = P.assemble_jacobian()
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, y)
    assert _rel(y, P.blocks_apply(A, x, transpose=True)) <= TOL64


@pytest.mark.parametrize("dim,k,n", CASES)
def test_transpose_apply_every_degree(pdg, oracle, dim, k, n):
    # the transposed operator of the non-symmetric method (NIPG, weights on)
    # with reaction and mixed boundary types, accumulated onto y0, against the
    # oracle's matrix-free transpose (convectiondiffusiondg.hh:191-195,
    # 474-481, 892-899 with the roles of trial and test functions exchanged)
    bct = [1, -1, -3, 1, -1, 1][:2 * dim]
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=40 + dim * 10 + k, method=0, weights=1,
                       react=True, bctype=bct)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply_transpose(x, y)
    assert _rel(y, y0 + P.jacobian_apply_transpose(x)) <= TOL64


@pytest.mark.parametrize("dim,k,n", [(2, 1, 6), (3, 2, 3), (3, 3, 3), (3, 4, 2)])
def test_jacobian_apply_f32(pdg, oracle, dim, k, n):
    import torch
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=3)
    x = rng.uniform(-1, 1, go.ndof)
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    yt = torch.zeros(go.ndof, dtype=torch.float32, device="cuda")
    go.jacobian_apply_f32(xt, yt)
    torch.cuda.synchronize()
    assert _rel(yt.cpu().double().numpy(), P.jacobian_apply(x)) <= TOL32


@pytest.mark.parametrize("k,nc,method,weights,react,bct", [
    (1, (7, 6, 5), 1, 0, True, None),
    (2, (9, 5, 4), 1, 0, True, [1, -1, 1, -2, -1, 1]),
    (3, (11, 4, 3), 0, 1, False, None),
    (4, (5, 4, 3), 2, 0, True, [-1, 1, 1, 1, -2, 1]),
    (2, (1, 1, 1), 1, 0, False, None),
    (2, (43, 1, 2), 1, 0, True, None),
    (3, (13, 7, 5), 1, 0, True, [1, -1, -2, 1, 1, -1]),
    (3, (33, 2, 3), 2, 1, False, None),
    (3, (1, 1, 1), 1, 0, False, None),
    (3, (5, 9, 11), 0, 0, True, None),
])
def test_jacobian_apply_f32_staged(pdg, oracle, k, nc, method, weights, react, bct):
    # the 3D FP32 kernel stages runs of CPB consecutive cells and their y/z
    # neighbour runs: grids larger than one run, runs that cross rows and
    # planes, every boundary type, reaction, all methods
    import torch
    go, P, rng = _pair(pdg, oracle, 3, k, nc, seed=31 + k, method=method, weights=weights,
                       bctype=bct, react=react)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    yt = torch.tensor(y0, dtype=torch.float32, device="cuda")
    go.jacobian_apply_f32(xt, yt)     # accumulates: y0 + J x
    torch.cuda.synchronize()
    ref = P.jacobian_apply(x, y0.copy())
    assert _rel(yt.cpu().double().numpy(), ref) <= TOL32


@pytest.mark.parametrize("k,nc,method,weights,react,bct", [
    (1, (7, 6, 5), 1, 0, True, None),
    (2, (9, 5, 4), 2, 1, True, [1, -1, 1, -2, -1, 1]),
    (3, (11, 4, 3), 0, 1, False, None),
    (3, (13, 7, 5), 1, 0, True, [1, -1, -2, 1, 1, -1]),
    (3, (33, 2, 3), 2, 1, False, None),
    (3, (1, 1, 1), 1, 0, False, None),
    (3, (5, 9, 11), 0, 0, True, None),
])
def test_jacobian_apply_transpose_f32_staged(pdg, oracle, k, nc, method, weights, react, bct):
    # the transposed FP32 operator (inner operator of the mixed adjoint solve)
    # against the oracle's matrix-free transpose
    import torch
    go, P, rng = _pair(pdg, oracle, 3, k, nc, seed=57 + k, method=method, weights=weights,
                       bctype=bct, react=react)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    yt = torch.tensor(y0, dtype=torch.float32, device="cuda")
    go.jacobian_apply_transpose_f32(xt, yt)     # accumulates: y0 + J^T x
    torch.cuda.synchronize()
    ref = y0 + P.jacobian_apply_transpose(x)
    assert _rel(yt.cpu().double().numpy(), ref) <= TOL32


@pytest.mark.parametrize("k,nc,method,weights,react,bct", [
    (3, (11, 4, 3), 0, 1, False, None),
    (3, (13, 7, 5), 1, 0, True, [1, -1, -2, 1, 1, -1]),
    (3, (33, 2, 3), 2, 1, False, None),
    (3, (1, 1, 1), 1, 0, False, None),
    (3, (5, 9, 11), 0, 0, True, None),
    (3, (40, 37, 12), 1, 0, True, None),
    (2, (9, 5, 4), 1, 0, True, [1, -1, 1, -2, -1, 1]),
])
def test_apply_f32_overwrites(pdg, oracle, k, nc, method, weights, react, bct):
    # y = J x in FP32 (the inner CG's operator; at Q3 the persistent kernel with
    # two staging regions per block, several runs per block on the larger grid)
    import torch
    go, P, rng = _pair(pdg, oracle, 3, k, nc, seed=71 + k, method=method, weights=weights,
                       bctype=bct, react=react)
    x = rng.uniform(-1, 1, go.ndof)
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    yt = torch.full((go.ndof,), 7.0, dtype=torch.float32, device="cuda")
    go.apply_f32(xt, yt)
    torch.cuda.synchronize()
    assert _rel(yt.cpu().double().numpy(), P.jacobian_apply(x)) <= TOL32


def test_device_pointers_match_host(pdg, oracle):
    import torch
    go, P, rng = _pair(pdg, oracle, 3, 3, 3, seed=4)
    x = rng.uniform(-1, 1, go.ndof)
    xt = torch.tensor(x, dtype=torch.float64, device="cuda")
    yt = torch.zeros(go.ndof, dtype=torch.float64, device="cuda")
    go.jacobian_apply(xt, yt)
    y = np.zeros(go.ndof)
    go.jacobian_apply(x, y)
    assert np.array_equal(yt.cpu().numpy(), y)


@pytest.mark.parametrize("dim,k,n", [(2, 1, 8), (2, 3, 4), (2, 4, 3), (3, 2, 3), (3, 3, 2),
                                     (3, 4, 2)])
def test_residual_with_data(pdg, oracle, dim, k, n):
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=8, react=True)
    fq = rng.standard_normal((go.ncell, go.nq_volume))
    fc = rng.standard_normal(go.ncell)
    g = rng.standard_normal(go.nq_boundary)
    go.set_source(fq=fq, fc=fc)
    go.set_boundary_data(g=g)
    P.set(fq=fq, fc=fc, gq=g)
    x = rng.uniform(-1, 1, go.ndof)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64
    assert np.allclose(go.volume_points(), P.volume_points(), rtol=0, atol=1e-15)
    assert np.allclose(go.boundary_points(), P.boundary_points(), rtol=0, atol=1e-15)


def test_residual_neumann_outflow_data(pdg, oracle):
    bct = [1, -1, -1, 1, 1, -1]
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=9, bctype=bct)
    j = rng.standard_normal(go.nq_boundary)
    g = rng.standard_normal(go.nq_boundary)
    go.set_boundary_data(g=g, j=j)
    P.set(gq=g, jq=j)
    x = rng.uniform(-1, 1, go.ndof)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64


@pytest.mark.parametrize("kind", ["fdm", "dense"])
@pytest.mark.parametrize("dim,k,n", [(2, 1, 5), (2, 3, 3), (3, 2, 3), (3, 4, 2)])
def test_block_jacobi(pdg, oracle, kind, dim, k, n):
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=12, react=True)
    lu, piv = P.lu(P.block_diagonal())
    d = rng.uniform(-1, 1, go.ndof)
    vref = P.lu_apply(lu, piv, d)
    prec = pdg.GridOperatorPreconditioner(
        go, kind=pdg.PREC_BJ_FDM if kind == "fdm" else pdg.PREC_BJ_DENSE)
    prec.pre()
    v = np.zeros(go.ndof)
    prec.apply(v, d)
    assert _rel(v, vref) <= 1e-10


def test_block_jacobi_dense_nonsymmetric(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=13, method=0, react=True)
    lu, piv = P.lu(P.block_diagonal())
    d = rng.uniform(-1, 1, go.ndof)
    prec = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE)
    prec.pre()
    v = np.zeros(go.ndof)
    prec.apply(v, d)
    assert _rel(v, P.lu_apply(lu, piv, d)) <= 1e-10


def _mfl(pdg, oracle, n=16):
    # matrix_free_linear.cc problem (2D Q1 SIPG alpha=3, g = exp(-|x-1/2|^2))
    go = pdg.GridOperator(2, 1, (n, n), alpha=3.0)
    P = oracle.Problem(2, 1, (n, n), alpha=3.0)
    vp = go.volume_points()
    c = (0.5 - vp[..., 0]) ** 2 + (0.5 - vp[..., 1]) ** 2
    bp = go.boundary_points()
    cb = (0.5 - bp[:, 0]) ** 2 + (0.5 - bp[:, 1]) ** 2
    f, g = 4 * (1 - c) * np.exp(-c), np.exp(-cb)
    go.set_source(fq=f)
    go.set_boundary_data(g=g)
    P.set(fq=f, gq=g)
    return go, P


@pytest.mark.parametrize("solver", ["cg", "bicgstab"])
def test_matrix_free_linear_solve(pdg, oracle, solver):
    go, P = _mfl(pdg, oracle)
    method = pdg.CG if solver == "cg" else pdg.BICGSTAB
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=method, preconditioner=pdg.PREC_BJ_FDM)
    u = np.zeros(go.ndof)
    slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-12)
    slp.apply()
    res = slp.result()
    uref, rres, st = P.solve(solver=solver, op=0, reduction=1e-12)
    assert res.converged and rres.converged
    assert abs(res.iterations - rres.iterations) <= 1
    assert _rel(u, uref) <= 1e-9
    # L2 error threshold of matrix_free_linear.cc:387-391
    xyz, w, val = P.eval_points(u, 6)
    ce = (0.5 - xyz[..., 0]) ** 2 + (0.5 - xyz[..., 1]) ** 2
    assert np.sum(w * (val - np.exp(-ce)) ** 2) < 1e-6


def test_c1_sin_source_solve(pdg, oracle):
    """The 2D Q1 64^2 workload: K = 1, alpha = 3, homogeneous Dirichlet,
    f = sin(2 pi x) sin(2 pi y) + eps_cell with eps_cell i.i.d. normal of
    variance 0.01 (standard deviation 0.1, the N(mu, sigma^2) reading),
    CG + cell-block Jacobi to 1e-10: iterations within one of the oracle's
    CG and the solutions within 1e-8."""
    import bench
    go, fq = bench.c1_problem(pdg, np, 0)
    P = oracle.Problem(2, 1, (64, 64), alpha=3.0, fq=fq)
    uref, rres, st = P.solve(solver="cg", op=0, reduction=1e-10)
    assert st == 0 and rres.converged
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, preconditioner=pdg.PREC_BJ_FDM)
    u = np.zeros(go.ndof)
    slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
    slp.apply()
    res = slp.result()
    assert res.converged
    assert abs(res.iterations - rres.iterations) <= 1, (res.iterations, rres.iterations)
    assert _rel(u, uref) <= 1e-8
    # the true FP64 defect of the GPU solution
    r, r0 = np.zeros(go.ndof), np.zeros(go.ndof)
    go.residual(u, r)
    go.residual(np.zeros(go.ndof), r0)
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(r0)
    go.close()


def test_solve_3d_cg_fp64_and_mixed(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 3, 2, 4, seed=21)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="cg", op=0, reduction=1e-10)
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG)
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    assert ls.result().converged
    assert abs(ls.result().iterations - rres.iterations) <= 1
    assert _rel(u, uref) <= 1e-8
    lsm = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, mixed=True)
    um = np.zeros(go.ndof)
    slp = pdg.StationaryLinearProblemSolver(go, lsm, um, 1e-10)
    slp.apply()
    assert slp.result().converged and slp.result().outer_iterations >= 2
    assert _rel(um, u) <= 1e-8
    # true residual of the mixed solution
    r = np.zeros(go.ndof)
    go.residual(um, r)
    r0 = np.zeros(go.ndof)
    go.residual(np.zeros(go.ndof), r0)
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(r0)


def test_bicgstab_nonsymmetric_dense(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=22, method=0, react=True)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="bicgstab", op=0, reduction=1e-10)
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                             preconditioner=pdg.PREC_BJ_DENSE)
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    assert ls.result().converged
    assert _rel(u, uref) <= 1e-8


@pytest.mark.parametrize("dim,k,n", [(2, 1, 5), (2, 4, 3), (3, 1, 3), (3, 2, 3), (3, 3, 2),
                                     (3, 4, 2)])
def test_grad_logK_matches_oracle(pdg, oracle, dim, k, n):
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=31)
    g = rng.standard_normal(go.nq_boundary)
    go.set_boundary_data(g=g)
    P.set(gq=g)
    u = rng.uniform(-1, 1, go.ndof)
    lam = rng.uniform(-1, 1, go.ndof)
    gg = np.zeros(go.ncell)
    go.grad_logK(u, lam, gg)
    gref = P.grad_logK(u, lam)
    assert _rel(gg, gref) <= 1e-11
    gs = np.zeros(go.ncell)
    go.grad_source(lam, gs)
    assert _rel(gs, P.grad_fc(lam)) <= 1e-12


def test_errors_are_status_codes(pdg):
    go = pdg.GridOperator(3, 2, (2, 2, 2))
    with pytest.raises(pdg.PDGError) as e:
        pdg.load().pdg_jacobian_apply(go.handle, None, None)
        pdg._check(pdg.load().pdg_jacobian_apply(go.handle, None, None))
    assert e.value.status == pdg.PDG_EINVAL
    prec = pdg.GridOperatorPreconditioner(pdg.GridOperator(3, 2, (2, 2, 2), method=pdg.NIPG))
    with pytest.raises(pdg.PDGError) as e:
        prec.pre()
    assert e.value.status == pdg.PDG_EUNSUPPORTED
    # maxit = 1: reported as non-convergence, not an exception
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, maxiter=1)
    go.set_source(fc=np.ones(go.ncell))
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-12).apply()
    assert not ls.result().converged and ls.result().iterations == 1


@pytest.mark.parametrize("k,nc", [(2, (6, 5, 4)), (3, (7, 5, 4))])
def test_mixed_adjoint_solve_uses_fp32_transpose(pdg, oracle, k, nc):
    # NIPG: J^T != J, so the FP32 inner solves of the mixed adjoint solve run
    # the transposed FP32 operator; the FP64 outer loop must land on the
    # FP64 adjoint solution
    go, P, rng = _pair(pdg, oracle, 3, k, nc, seed=60 + k, method=0, react=True)
    rhs = rng.uniform(-1, 1, go.ndof)
    lam = {}
    for mixed in (0, 1):
        o = pdg.default_options(method=pdg.BICGSTAB, preconditioner=pdg.PREC_BJ_DENSE,
                                reduction=1e-11, mixed=mixed, maxit=20000)
        pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE,
                                       precision=pdg.F32 if mixed else pdg.F64).pre()
        lam[mixed] = np.zeros(go.ndof)
        assert go.adjoint_solve(rhs, lam[mixed], o).converged
    assert _rel(lam[1], lam[0]) <= 1e-8
    # the FP64 adjoint solution against the oracle's transposed operator
    A = P.assemble_jacobian()
    r = P.blocks_apply(A, lam[0], transpose=True)
    assert np.linalg.norm(r - rhs) <= 1e-9 * np.linalg.norm(rhs)


@pytest.mark.parametrize("k,nc,inner_maxit", [(1, (9, 7, 6), 0), (2, (6, 5, 4), 0),
                                               (3, (5, 4, 4), 0), (2, (6, 5, 4), 20)])
def test_mixed_cg_fused_dots_match_unfused(pdg, oracle, k, nc, inner_maxit):
    # The FP32 inner CG computes <p, A p> inside the operator kernel and
    # <M^-1 r, r> inside the FDM block Jacobi kernel.  The dense block Jacobi
    # is the same exact block inverse but takes the separate dot kernels, so
    # both runs must agree (iteration counts up to FP32 rounding).
    go, P, rng = _pair(pdg, oracle, 3, k, nc, seed=70 + k, react=True)
    go.set_source(fc=rng.standard_normal(go.ncell))
    sols, its = {}, {}
    for kind in (pdg.PREC_BJ_FDM, pdg.PREC_BJ_DENSE):
        pdg.GridOperatorPreconditioner(go, kind=kind, precision=pdg.F32).pre()
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, preconditioner=kind,
                                                 mixed=True, inner_reduction=1e-4,
                                                 maxiter=20000)
        if inner_maxit:       # inner solves stopped by the iteration cap
            ls.opts.inner_maxit = inner_maxit
            ls.opts.max_outer = 2000
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        slp.apply()
        assert slp.result().converged
        sols[kind], its[kind] = u, slp.result().iterations
    assert abs(its[pdg.PREC_BJ_FDM] - its[pdg.PREC_BJ_DENSE]) <= max(2, its[pdg.PREC_BJ_DENSE] // 20)
    assert _rel(sols[pdg.PREC_BJ_FDM], sols[pdg.PREC_BJ_DENSE]) <= 1e-8


@pytest.mark.parametrize("k,nc", [(3, (7, 5, 3)), (3, (40, 3, 2)), (3, (1, 1, 1)), (2, (6, 5, 4))])
def test_block_jacobi_fdm_f32(pdg, oracle, k, nc):
    # the FP32 FDM block Jacobi (Q3: one z-plane per thread, partial blocks of
    # 32 cells) against the FP64 one
    import torch
    go, P, rng = _pair(pdg, oracle, 3, k, nc, seed=90 + k, react=True)
    d = rng.uniform(-1, 1, go.ndof)
    ref = np.zeros(go.ndof)
    p64 = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM, precision=pdg.F64)
    p64.pre()
    p64.apply(ref, d)
    p32 = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM, precision=pdg.F32)
    p32.pre()
    dt = torch.tensor(d, dtype=torch.float32, device="cuda")
    vt = torch.zeros_like(dt)
    torch.cuda.synchronize()
    p32.apply(vt, dt)
    torch.cuda.synchronize()
    assert _rel(vt.cpu().double().numpy(), ref) <= TOL32


def test_apply_f32_q3_unaligned_vectors(pdg, oracle):
    # the Q3 FP32 operator stages its runs with TMA copies from 16-byte
    # aligned vectors; vectors one float off that alignment take the
    # per-thread copy path; both must agree with the oracle
    import torch
    go, P, rng = _pair(pdg, oracle, 3, 3, (9, 5, 4), seed=95, react=True)
    x = rng.uniform(-1, 1, go.ndof)
    ref = P.jacobian_apply(x)
    for off in (0, 1):
        xb = torch.zeros(go.ndof + 4, dtype=torch.float32, device="cuda")
        yb = torch.zeros(go.ndof + 4, dtype=torch.float32, device="cuda")
        xt, yt = xb[off:off + go.ndof], yb[off:off + go.ndof]
        xt.copy_(torch.tensor(x, dtype=torch.float32))
        torch.cuda.synchronize()
        go.jacobian_apply_f32(xt, yt)
        torch.cuda.synchronize()
        assert _rel(yt.cpu().double().numpy(), ref) <= TOL32, off
