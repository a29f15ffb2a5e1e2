"""Matrix-free block preconditioners beyond block Jacobi on the GPU:
block SOR (BlockSORPreconditionerLocalOperator) and iterative block Jacobi
(IterativeBlockJacobiPreconditionerLocalOperator), against the oracle's
sequential sweep and per-block dune-istl BiCGStab."""
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


def _pair(pdg, oracle, dim, k, nc, seed, method=1, conv=False):
    rng = np.random.default_rng(seed)
    ncell = int(np.prod(nc))
    K = np.exp(rng.standard_normal(ncell))
    c = rng.uniform(0.5, 1.5, ncell)
    go = pdg.GridOperator(dim, k, nc, alpha=3.0, method=method)
    go.set_permeability(K)
    go.set_reaction(c)
    kw = dict(K=K, c=c)
    if conv:
        modes = pdg.fourier_velocity_modes(seed)
        go.set_velocity_modes(modes)
        kw["modes"] = modes
    P = oracle.Problem(dim, k, nc, alpha=3.0, method=method, **kw)
    return go, P, rng


def _oracle_kind(pdg, kind):
    # the oracle's block kinds: 1/2 LU (FDM and dense invert the same block)
    return kind


KINDS = [
    ("iterative", 3),
    ("sor_dense", 16 | 2),
    ("sor_fdm", 16 | 1),
    ("sor_iterative", 16 | 3),
    ("sor_none", 16 | 0),
]


@pytest.mark.parametrize("name,kind", KINDS)
@pytest.mark.parametrize("transpose", [False, True])
def test_prec_apply_matches_oracle(pdg, oracle, name, kind, transpose):
    go, P, rng = _pair(pdg, oracle, 3, 2, (3, 4, 2), seed=21)
    omega = 1.0 if kind != (16 | 2) else 1.3
    go.set_prec_options(omega=omega)
    prec = pdg.GridOperatorPreconditioner(go, kind=kind)
    prec.pre()
    d = rng.uniform(-1, 1, go.ndof)
    v = np.zeros(go.ndof)
    if transpose:
        pdg._check(pdg.load().pdg_prec_apply_transpose(go.handle, pdg._ptr(d), pdg._ptr(v)))
    else:
        prec.apply(v, d)
    pc = oracle.prec_config(kind, omega=omega)
    vref, its = P.prec_apply_cfg(pc, d, transpose=transpose)
    assert _rel(v, vref) <= 1e-9
    if kind & 15 == 3:
        ours = go.prec_block_iterations()
        assert np.mean(ours == its) >= 0.95 and np.max(np.abs(ours - its)) <= 1


@pytest.mark.parametrize("dim,k,nc,method,conv,kind", [
    (2, 3, (5, 4), 1, False, 16 | 2),
    (2, 1, (6, 5), 0, False, 3),
    (3, 2, (3, 3, 3), 1, True, 16 | 2),
    (3, 2, (3, 3, 3), 1, True, 3),
    (3, 1, (4, 3, 3), 2, False, 16 | 3),
])
def test_prec_apply_variants(pdg, oracle, dim, k, nc, method, conv, kind):
    go, P, rng = _pair(pdg, oracle, dim, k, nc, seed=23, method=method, conv=conv)
    prec = pdg.GridOperatorPreconditioner(go, kind=kind)
    prec.pre()
    d = rng.uniform(-1, 1, go.ndof)
    v = np.zeros(go.ndof)
    prec.apply(v, d)
    vref, _ = P.prec_apply_cfg(oracle.prec_config(kind), d)
    assert _rel(v, vref) <= 1e-9


@pytest.mark.parametrize("kind,solver", [(16 | 2, "bicgstab"), (3, "bicgstab"),
                                         (16 | 3, "bicgstab"), (3, "cg")])
def test_solve_with_block_preconditioners(pdg, oracle, kind, solver):
    go, P, rng = _pair(pdg, oracle, 3, 2, (4, 4, 4), seed=25)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve_prec(oracle.prec_config(kind), solver=solver, reduction=1e-10)
    assert st == 0 and rres.converged
    meth = pdg.CG if solver == "cg" else pdg.BICGSTAB
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=meth, preconditioner=kind)
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    r = ls.result()
    assert r.converged
    assert abs(r.iterations - rres.iterations) <= 1
    assert _rel(u, uref) <= 1e-8


def test_mixed_solve_with_sor(pdg, oracle):
    # FP32 block SOR inside the mixed-precision solve
    go, P, rng = _pair(pdg, oracle, 3, 2, (4, 4, 4), seed=27, conv=True)
    go.set_source(fc=np.ones(go.ncell))
    P.set(fc=np.ones(go.ncell))
    uref, rres, st = P.solve(solver="bicgstab", reduction=1e-12)
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                             preconditioner=pdg.PREC_SOR | pdg.PREC_BJ_DENSE,
                                             mixed=True, inner_reduction=1e-1)
    ls.opts.inner_maxit = 30
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    assert ls.result().converged
    assert _rel(u, uref) <= 1e-8


def test_adjoint_solve_with_sor(pdg, oracle):
    go, P, rng = _pair(pdg, oracle, 3, 2, (3, 3, 3), seed=29, conv=True)
    rhs = rng.uniform(-1, 1, go.ndof)
    o = pdg.default_options(method=pdg.BICGSTAB, preconditioner=pdg.PREC_SOR | pdg.PREC_BJ_DENSE,
                            reduction=1e-11)
    lam = np.zeros(go.ndof)
    assert go.adjoint_solve(rhs, lam, o).converged
    A = P.assemble_jacobian()
    assert _rel(P.blocks_apply(A, lam, transpose=True), rhs) <= 1e-9


def test_sor_graph_replay(pdg, oracle):
    # the first sweep of a generation runs eagerly and captures a CUDA graph;
    # later sweeps replay it; a coefficient change starts a new generation
    go, P, rng = _pair(pdg, oracle, 3, 2, (4, 3, 3), seed=31)
    prec = pdg.GridOperatorPreconditioner(go, kind=16 | 2)
    prec.pre()
    pc = oracle.prec_config(16 | 2)
    for rep in range(3):
        d = rng.uniform(-1, 1, go.ndof)
        v = np.zeros(go.ndof)
        prec.apply(v, d)
        vref, _ = P.prec_apply_cfg(pc, d)
        assert _rel(v, vref) <= 1e-9, rep
    K2 = np.exp(rng.standard_normal(go.ncell))
    go.set_permeability(K2)
    P.set(K=K2)
    prec = pdg.GridOperatorPreconditioner(go, kind=16 | 2)
    prec.pre()
    for rep in range(2):
        d = rng.uniform(-1, 1, go.ndof)
        v = np.zeros(go.ndof)
        prec.apply(v, d)
        vref, _ = P.prec_apply_cfg(pc, d)
        assert _rel(v, vref) <= 1e-9, rep


def test_prec_options_validation(pdg):
    go = pdg.GridOperator(3, 1, (2, 2, 2))
    with pytest.raises(pdg.PDGError):
        go.set_prec_options(omega=2.5)
    with pytest.raises(pdg.PDGError):
        go.set_prec_options(block_maxit=0)
    with pytest.raises(pdg.PDGError):
        pdg.GridOperatorPreconditioner(go, kind=4).pre()
