"""GPU parity for parameter fields beyond A = K I, through the C ABI.

The reference evaluates A(cell, x) as a d x d tensor at the cell centre, or
at every quadrature point when permeabilityIsConstantPerCell() is false, and
b(cell, x), c(cell, x) at every quadrature point
(localoperator/convectiondiffusiondg.hh:124-146, 178-181, 305-382, 425-426,
710-761; convectiondiffusionparameter.hh:143-183).  The GPU evaluates these
forms at the same Gauss points (pdg_general.cu); the oracle restates the
reference's loops.  Tolerances: FP64 <= 1e-12 relative (max norm), FP32
<= 2e-5, solves to 1e-10 within 1e-8 and iteration counts within one.
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


def _spd(rng, n, d, aniso=4.0, full=True):
    out = np.zeros((n, d, d))
    for e in range(n):
        lam = rng.uniform(1.0, aniso, d)
        if full:
            q, _ = np.linalg.qr(rng.standard_normal((d, d)))
            out[e] = (q * lam) @ q.T
        else:
            out[e] = np.diag(lam)
    return out * np.exp(rng.standard_normal(n))[:, None, None]


def _pair(pdg, oracle, dim, k, n, method=1, weights=0, bctype=None, seed=0):
    nc = (n,) * dim
    go = pdg.GridOperator(dim, k, nc, method=method, weights=weights, alpha=3.0, bctype=bctype)
    P = oracle.Problem(dim, k, nc, method=method, weights=weights, alpha=3.0, bctype=bctype)
    return go, P, np.random.default_rng(seed)


def _check_apply(go, P, rng, transpose=True):
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x, y0.copy())) <= TOL64
    if transpose:
        yt = np.zeros(go.ndof)
        go.jacobian_apply_transpose(x, yt)
        assert _rel(yt, P.jacobian_apply_transpose(x)) <= TOL64
    return x


CASES = [(2, 1, 5), (2, 2, 4), (2, 3, 3), (2, 4, 3), (3, 1, 4), (3, 2, 3), (3, 3, 3), (3, 4, 2)]


@pytest.mark.parametrize("dim,k,n", CASES)
def test_full_tensor_per_cell(pdg, oracle, dim, k, n):
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=dim * 10 + k)
    A = _spd(rng, go.ncell, dim)
    go.set_permeability_tensor(A)
    P.set(Acell=A)
    x = _check_apply(go, P, rng)
    # FP32 operator (the inner operator of mixed-precision solves; device
    # vectors only)
    import torch
    x32 = torch.tensor(x, dtype=torch.float32, device="cuda")
    y32 = torch.zeros(go.ndof, dtype=torch.float32, device="cuda")
    go.jacobian_apply_f32(x32, y32)
    assert _rel(y32.double().cpu().numpy(), P.jacobian_apply(x)) <= TOL32
    go.close()


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("weights", [0, 1])
def test_tensor_methods_weights_and_boundaries(pdg, oracle, method, weights):
    bct = [1, -1, 1, -3, 1, 1]
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, method=method, weights=weights, bctype=bct,
                       seed=method * 2 + weights)
    A = _spd(rng, go.ncell, 3)
    c = rng.uniform(0.5, 2.0, go.ncell)
    go.set_permeability_tensor(A)
    go.set_reaction(c)
    P.set(Acell=A, c=c)
    _check_apply(go, P, rng)
    go.close()


@pytest.mark.parametrize("dim,k,n", [(2, 2, 4), (3, 1, 3), (3, 2, 3), (3, 3, 2)])
def test_diagonal_anisotropic_tensor(pdg, oracle, dim, k, n):
    go, P, rng = _pair(pdg, oracle, dim, k, n, seed=7 + k)
    A = _spd(rng, go.ncell, dim, full=False)
    go.set_permeability_tensor(A)
    P.set(Acell=A)
    _check_apply(go, P, rng)
    go.close()


@pytest.mark.parametrize("dim,k,n,method", [(2, 2, 4, 1), (2, 3, 3, 0), (3, 1, 3, 1),
                                            (3, 2, 3, 2), (3, 3, 2, 1)])
def test_tensor_per_point(pdg, oracle, dim, k, n, method):
    """permeabilityIsConstantPerCell() == false: a different tensor at every
    volume point and at every cell's own face points."""
    go, P, rng = _pair(pdg, oracle, dim, k, n, method=method, bctype=[1, 1, -1, 1, 1, 1],
                       seed=30 + k)
    nqv, nqf = P.nq_volume, P.nq_face
    Av = _spd(rng, go.ncell * nqv, dim).reshape(go.ncell, nqv, dim, dim)
    Af = _spd(rng, go.ncell * 2 * dim * nqf, dim).reshape(go.ncell, 2 * dim, nqf, dim, dim)
    go.set_permeability_points(Av, Af)
    P.set(Aq_vol=Av, Aq_face=Af)
    _check_apply(go, P, rng)
    go.close()


def test_point_coordinates_match_oracle(pdg, oracle):
    for dim, k, n in ((2, 2, 3), (3, 3, 2)):
        go, P, _ = _pair(pdg, oracle, dim, k, n)
        assert np.max(np.abs(go.face_lattice_points() - P.face_lattice_points())) < 1e-15
        assert np.max(np.abs(go.cell_face_points() - P.cell_face_points())) < 1e-15
        go.close()


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_reaction_and_velocity_per_point(pdg, oracle, k):
    """c per volume point (added to the per-cell c) and b given as point data
    at the volume points and the face-lattice points (3D)."""
    n = 3 if k < 4 else 2
    go, P, rng = _pair(pdg, oracle, 3, k, n, bctype=[1, -2, 1, 1, 1, 1], seed=50 + k)
    K = np.exp(rng.standard_normal(go.ncell))
    go.set_permeability(K)
    P.set(K=K)
    c = rng.uniform(0.5, 2.0, go.ncell)
    cq = rng.uniform(0.0, 1.0, (go.ncell, P.nq_volume))
    go.set_reaction(c)
    go.set_reaction_points(cq)
    P.set(c=c, cq=cq)
    # a divergence-free field with b.n >= 0 on the outflow side +x
    def b_at(x):
        b = np.zeros(x.shape[:-1] + (3,))
        b[..., 0] = 2.0 + np.sin(2 * np.pi * x[..., 1])
        b[..., 1] = np.cos(2 * np.pi * x[..., 2])
        b[..., 2] = np.sin(2 * np.pi * x[..., 0])
        return b
    bv, bf = b_at(go.volume_points()), b_at(go.face_lattice_points())
    go.set_velocity_points(bv, bf)
    P.set(bq_vol=bv, bq_face=bf)
    _check_apply(go, P, rng)
    go.close()


def test_tensor_residual_with_dirichlet_data(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, bctype=[1, 1, -1, 1, 1, 1], seed=61)
    A = _spd(rng, go.ncell, 3)
    go.set_permeability_tensor(A)
    P.set(Acell=A)
    f = rng.uniform(-1, 1, (go.ncell, P.nq_volume))
    nb = P.nbpts_total()
    g, j = rng.uniform(-1, 1, nb), rng.uniform(-1, 1, nb)
    go.set_source(fq=f)
    go.set_boundary_data(g=g, j=j)
    P.set(fq=f, gq=g, jq=j)
    x = rng.uniform(-1, 1, go.ndof)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64
    # and per point
    nqv, nqf = P.nq_volume, P.nq_face
    Av = _spd(rng, go.ncell * nqv, 3).reshape(go.ncell, nqv, 3, 3)
    Af = _spd(rng, go.ncell * 6 * nqf, 3).reshape(go.ncell, 6, nqf, 3, 3)
    go.set_permeability_points(Av, Af)
    P.set(Acell=None, Aq_vol=Av, Aq_face=Af)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64
    go.close()


def test_tensor_solves(pdg, oracle):
    """SIPG with a symmetric tensor: CG + dense cell-block Jacobi against the
    oracle's CG, FP64 and mixed precision; the FDM block Jacobi is refused."""
    go, P, rng = _pair(pdg, oracle, 3, 2, 4, seed=70)
    A = _spd(rng, go.ncell, 3)
    go.set_permeability_tensor(A)
    go.set_source(fc=np.ones(go.ncell))
    P.set(Acell=A, fc=np.ones(go.ncell))
    with pytest.raises(pdg.PDGError):
        pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM).pre()
    uref, rres, st = P.solve(solver="cg", op=0, reduction=1e-10)
    assert st == 0 and rres.converged
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, preconditioner=pdg.PREC_BJ_DENSE)
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    res = ls.result()
    assert res.converged
    assert abs(res.iterations - rres.iterations) <= 1, (res.iterations, rres.iterations)
    assert _rel(u, uref) <= 1e-8
    lsm = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, preconditioner=pdg.PREC_BJ_DENSE,
                                              mixed=True)
    um = np.zeros(go.ndof)
    slp = pdg.StationaryLinearProblemSolver(go, lsm, um, 1e-10)
    slp.apply()
    assert slp.result().converged
    assert _rel(um, u) <= 1e-8
    r, r0 = np.zeros(go.ndof), np.zeros(go.ndof)
    go.residual(um, r)
    go.residual(np.zeros(go.ndof), r0)
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(r0)
    go.close()


def test_scalar_permeability_drops_tensor(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 3, 2, 3, seed=80)
    go.set_permeability_tensor(_spd(rng, go.ncell, 3))
    K = np.exp(rng.standard_normal(go.ncell))
    go.set_permeability(K)          # back to A = K I, the Kronecker kernels
    P.set(K=K)
    _check_apply(go, P, rng)
    pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM).pre()   # separable again
    go.close()


def test_diagonal_tensor_keeps_fdm_and_mixed_solve(pdg, oracle):
    """A diagonal tensor per cell stays separable (K per direction in the
    Kronecker records): the FDM block Jacobi is exact for it, and the FP64 and
    mixed-precision CG solves match the oracle's CG."""
    go, P, rng = _pair(pdg, oracle, 3, 3, 4, seed=90)
    A = _spd(rng, go.ncell, 3, full=False)
    go.set_permeability_tensor(A)
    go.set_source(fc=np.ones(go.ncell))
    P.set(Acell=A, fc=np.ones(go.ncell))
    # the FDM block inverse against the oracle's LU of the diagonal blocks
    prec = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM)
    prec.pre()
    d = rng.uniform(-1, 1, go.ndof)
    v = np.zeros(go.ndof)
    prec.apply(v, d)
    lu, piv = P.lu(P.block_diagonal())
    assert _rel(v, P.lu_apply(lu, piv, d)) <= 1e-10
    uref, rres, st = P.solve(solver="cg", op=0, reduction=1e-10)
    assert st == 0 and rres.converged
    for mixed in (False, True):
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, preconditioner=pdg.PREC_BJ_FDM,
                                                 mixed=mixed)
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        slp.apply()
        assert slp.result().converged
        if not mixed:
            assert abs(slp.result().iterations - rres.iterations) <= 1
        assert _rel(u, uref) <= 1e-8
    go.close()


@pytest.mark.parametrize("dim,k,nc", [(3, 2, (3, 2, 4)), (3, 1, (1, 1, 1)), (2, 3, (1, 5)),
                                      (2, 2, (4, 1))])
def test_tensor_non_cubic_and_single_cell(pdg, oracle, dim, k, nc):
    rng = np.random.default_rng(sum(nc) + 10 * k)
    go = pdg.GridOperator(dim, k, nc, alpha=3.0, bctype=[1, -1, 1, 1, -1, 1])
    P = oracle.Problem(dim, k, nc, alpha=3.0, bctype=[1, -1, 1, 1, -1, 1])
    A = _spd(rng, go.ncell, dim)
    go.set_permeability_tensor(A)
    P.set(Acell=A)
    _check_apply(go, P, rng)
    go.close()


@pytest.mark.parametrize("basis", [1, 2])
def test_tensor_with_legendre_and_lobatto(pdg, oracle, basis):
    rng = np.random.default_rng(120 + basis)
    go = pdg.GridOperator(3, 2, (3, 3, 2), alpha=3.0, basis=basis)
    P = oracle.Problem(3, 2, (3, 3, 2), alpha=3.0, basis=basis)
    A = _spd(rng, go.ncell, 3)
    go.set_permeability_tensor(A)
    P.set(Acell=A)
    _check_apply(go, P, rng)
    go.close()
