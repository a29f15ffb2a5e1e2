"""Legendre and Gauss-Lobatto QkDG bases on the GPU against the oracle.

QkDGLocalFiniteElementMap<..., QkDGBasisPolynomial::legendre / lobatto>
(finiteelementmap/qkdg.hh:18-160): the Lobatto basis is nodal and runs the
kernels with its own 1D tables; the Legendre basis runs them between
per-cell changes of basis.  Tolerances as in test_gpu_parity: FP64 operator
<= 1e-12, FP32 <= 2e-5, solves <= 1e-8 relative (max norm).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5
BASES = ["legendre", "lobatto"]


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def pdg():
    import __graft_entry__
    __graft_entry__.build()
    import pdg as m
    return m


def _pair(pdg, oracle, basis, dim, k, n, seed=0, method=1, react=False, bctype=None):
    b = pdg.LEGENDRE if basis == "legendre" else pdg.LOBATTO
    rng = np.random.default_rng(seed)
    nc = (n,) * dim if np.isscalar(n) else tuple(n)
    ncell = int(np.prod(nc))
    K = np.exp(rng.standard_normal(ncell))
    c = rng.uniform(0.5, 2.0, ncell) if react else None
    go = pdg.GridOperator(dim, k, nc, method=method, alpha=3.0, bctype=bctype, basis=b)
    go.set_permeability(K)
    if react:
        go.set_reaction(c)
    P = oracle.Problem(dim, k, nc, method=method, alpha=3.0, bctype=bctype, K=K, c=c, basis=b)
    return go, P, rng


CASES = [(2, 1, 6), (2, 2, 5), (2, 4, 3), (3, 1, 4), (3, 2, 3), (3, 3, 3), (3, 4, 2),
         (3, 2, (5, 3, 2))]


@pytest.mark.parametrize("basis", BASES)
@pytest.mark.parametrize("dim,k,n", CASES)
def test_apply_f64(pdg, oracle, basis, dim, k, n):
    go, P, rng = _pair(pdg, oracle, basis, dim, k, n, seed=dim * 10 + k, react=True)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x, y0.copy())) <= TOL64
    go.close()


@pytest.mark.parametrize("basis", BASES)
@pytest.mark.parametrize("method", [0, 2])
def test_transpose_apply(pdg, oracle, basis, method):
    go, P, rng = _pair(pdg, oracle, basis, 3, 2, 3, seed=5 + method, method=method, react=True)
    A = P.assemble_jacobian()
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, y)
    assert _rel(y, P.blocks_apply(A, x, transpose=True)) <= TOL64
    go.close()


@pytest.mark.parametrize("basis", BASES)
@pytest.mark.parametrize("k,nc", [(1, (6, 5, 4)), (2, (5, 4, 3)), (3, 3), (4, 2)])
def test_apply_f32(pdg, oracle, basis, k, nc):
    import torch
    go, P, rng = _pair(pdg, oracle, basis, 3, k, nc, seed=40 + k)
    x = rng.uniform(-1, 1, go.ndof)
    xt = torch.tensor(x, dtype=torch.float32, device="cuda")
    yt = torch.zeros(go.ndof, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    go.jacobian_apply_f32(xt, yt)
    torch.cuda.synchronize()
    assert _rel(yt.cpu().double().numpy(), P.jacobian_apply(x)) <= TOL32
    go.close()


@pytest.mark.parametrize("basis", BASES)
@pytest.mark.parametrize("dim,k,n", [(2, 3, 4), (3, 2, 3), (3, 4, 2)])
def test_residual_with_data(pdg, oracle, basis, dim, k, n):
    bct = [1, -1, 1, -2, 1, 1]
    go, P, rng = _pair(pdg, oracle, basis, dim, k, n, seed=8, react=True, bctype=bct)
    fq = rng.standard_normal((go.ncell, go.nq_volume))
    fc = rng.standard_normal(go.ncell)
    g = rng.standard_normal(go.nq_boundary)
    j = rng.standard_normal(go.nq_boundary)
    go.set_source(fq=fq, fc=fc)
    go.set_boundary_data(g=g, j=j)
    P.set(fq=fq, fc=fc, gq=g, jq=j)
    x = rng.uniform(-1, 1, go.ndof)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64
    go.close()


@pytest.mark.parametrize("basis", BASES)
@pytest.mark.parametrize("kind", ["fdm", "dense"])
def test_block_jacobi(pdg, oracle, basis, kind):
    go, P, rng = _pair(pdg, oracle, basis, 3, 3, 2, seed=12, react=True)
    lu, piv = P.lu(P.block_diagonal())
    d = rng.uniform(-1, 1, go.ndof)
    prec = pdg.GridOperatorPreconditioner(
        go, kind=pdg.PREC_BJ_FDM if kind == "fdm" else pdg.PREC_BJ_DENSE)
    prec.pre()
    v = np.zeros(go.ndof)
    prec.apply(v, d)
    assert _rel(v, P.lu_apply(lu, piv, d)) <= 1e-10
    go.close()


@pytest.mark.parametrize("basis", BASES)
def test_solves_fp64_and_mixed(pdg, oracle, basis):
    go, P, rng = _pair(pdg, oracle, basis, 3, 2, 4, seed=21)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="cg", op=0, reduction=1e-10)
    assert st == 0
    for mixed in (False, True):
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, mixed=mixed)
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        slp.apply()
        assert slp.result().converged
        if not mixed:
            assert abs(slp.result().iterations - rres.iterations) <= 1
        assert _rel(u, uref) <= 1e-8
    go.close()


@pytest.mark.parametrize("basis", BASES)
def test_mass_and_gradients(pdg, oracle, basis):
    go, P, rng = _pair(pdg, oracle, basis, 3, 3, 3, seed=31)
    g = rng.standard_normal(go.nq_boundary)
    go.set_boundary_data(g=g)
    P.set(gq=g)
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.mass_apply(x, y)
    assert _rel(y, P.mass_apply(x)) <= TOL64
    u = rng.uniform(-1, 1, go.ndof)
    lam = rng.uniform(-1, 1, go.ndof)
    gg = np.zeros(go.ncell)
    go.grad_logK(u, lam, gg)
    assert _rel(gg, P.grad_logK(u, lam)) <= 1e-11
    gs = np.zeros(go.ncell)
    go.grad_source(lam, gs)
    assert _rel(gs, P.grad_fc(lam)) <= 1e-12
    go.close()


def test_legendre_unsupported_features_raise(pdg):
    go = pdg.GridOperator(3, 2, (3, 3, 3), basis=pdg.LEGENDRE)
    with pytest.raises(pdg.PDGError) as e:
        pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM | pdg.PREC_SOR).pre()
    assert e.value.status == pdg.PDG_EUNSUPPORTED
    with pytest.raises(pdg.PDGError) as e:
        go.set_nonlinearity([0.0, 1.0])
    assert e.value.status == pdg.PDG_EUNSUPPORTED
    go.close()


def test_advection_basis_independence(pdg, oracle):
    """3D version of testdglegendre.cc: pure advection (A = 0, b = (1, 1/3, 0)),
    Dirichlet inflow data g = [y >= x/3 + 1/4], SIPG alpha = 2, degree 1; the
    Legendre, Lobatto and Lagrange solutions are the same function
    (L2 difference squared < 1e-14, testdglegendre.cc:190)."""
    n = 6
    D, O = pdg.BC_DIRICHLET, pdg.BC_OUTFLOW
    bct = [D, O, D, O, O, O]
    modes = np.array([[0, 0, 0, np.pi / 2, 1.0, 1.0 / 3.0, 0.0]])
    sols = {}
    for name, b in (("lagrange", pdg.LAGRANGE), ("legendre", pdg.LEGENDRE),
                    ("lobatto", pdg.LOBATTO)):
        go = pdg.GridOperator(3, 1, (n, n, n), alpha=2.0, bctype=bct, basis=b)
        go.set_permeability(np.zeros(go.ncell))
        go.set_velocity_modes(modes)
        bp = go.boundary_points()
        go.set_boundary_data(g=np.where(bp[:, 1] < bp[:, 0] / 3.0 + 0.25, 0.0, 1.0))
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                                 preconditioner=pdg.PREC_BJ_DENSE)
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-12)
        slp.apply()
        assert slp.result().converged, name
        P = oracle.Problem(3, 1, (n, n, n), alpha=2.0, bctype=bct, basis=b)
        sols[name] = P.eval_points(u, 4)
        go.close()
    _, w, vl = sols["lagrange"]
    assert np.max(vl) > 0.5 and np.min(vl) < 0.5
    for name in ("legendre", "lobatto"):
        assert float(np.sum(w * (sols[name][2] - vl) ** 2)) < 1e-14, name
