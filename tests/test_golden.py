"""Golden fixtures (tests/golden/*.npz, written by make_golden.py from the
pinned oracle): the oracle must keep reproducing them (CPU), and the CUDA
path must match them through the C ABI (GPU)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
APPLY = ["apply_q2_4.npz", "apply_q1_2d_8.npz", "apply_q4_2_nipg.npz"]


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def _problem(oracle, z):
    method = int(z["opt_method"]) if "opt_method" in z else oracle.SIPG
    dim, k, n = int(z["dim"]), int(z["k"]), int(z["n"])
    return oracle.Problem(dim, k, (n,) * dim, alpha=3.0, method=method, K=z["K"]), method


@pytest.mark.parametrize("name", APPLY)
def test_oracle_reproduces_apply_fixtures(oracle, name):
    z = _load(name)
    P, _ = _problem(oracle, z)
    assert _rel(P.jacobian_apply(z["x"]), z["y"]) <= 1e-13
    A = P.assemble_jacobian()
    assert _rel(P.blocks_apply(A, z["x"], transpose=True), z["yt"]) <= 1e-13
    lu, piv = P.lu(P.block_diagonal())
    assert _rel(P.lu_apply(lu, piv, z["d"]), z["v"]) <= 1e-12


def test_oracle_reproduces_solve_fixture(oracle):
    z = _load("mfl_q1_16.npz")
    P = oracle.Problem(2, 1, (16, 16), alpha=3.0, fq=z["f"], gq=z["g"])
    assert _rel(P.residual(np.zeros(P.ndof)), z["r0"]) <= 1e-13
    u, res, st = P.solve(solver="bicgstab", op=0, reduction=1e-12)
    assert res.iterations == int(z["iterations"])
    assert _rel(u, z["u"]) <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", APPLY)
def test_gpu_matches_apply_fixtures(oracle, name):
    import __graft_entry__
    __graft_entry__.build()
    import pdg
    z = _load(name)
    _, method = _problem(oracle, z)
    dim, k, n = int(z["dim"]), int(z["k"]), int(z["n"])
    go = pdg.GridOperator(dim, k, (n,) * dim, alpha=3.0, method=method)
    go.set_permeability(z["K"])
    y = np.zeros(go.ndof)
    go.jacobian_apply(z["x"], y)
    assert _rel(y, z["y"]) <= 1e-12
    yt = np.zeros(go.ndof)
    go.jacobian_apply_transpose(z["x"], yt)
    assert _rel(yt, z["yt"]) <= 1e-12
    prec = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE)
    prec.pre()
    v = np.zeros(go.ndof)
    prec.apply(v, z["d"])
    assert _rel(v, z["v"]) <= 1e-10


@pytest.mark.gpu
def test_gpu_matches_residual_and_solve_fixtures():
    import __graft_entry__
    __graft_entry__.build()
    import pdg
    z = _load("residual_q3_3.npz")
    go = pdg.GridOperator(3, 3, (3, 3, 3), alpha=3.0)
    go.set_permeability(z["K"])
    go.set_source(fq=z["fq"])
    go.set_boundary_data(g=z["g"])
    r = np.zeros(go.ndof)
    go.residual(z["x"], r)
    assert _rel(r, z["r"]) <= 1e-12
    z = _load("mfl_q1_16.npz")
    go = pdg.GridOperator(2, 1, (16, 16), alpha=3.0)
    go.set_source(fq=z["f"])
    go.set_boundary_data(g=z["g"])
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB)
    u = np.zeros(go.ndof)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-12).apply()
    assert ls.result().converged
    assert abs(ls.result().iterations - int(z["iterations"])) <= 1
    assert _rel(u, z["u"]) <= 1e-9
