"""The FP64 operator in float-pair arithmetic (pdg_set_f64_arithmetic with
PDG_F64_FLOAT_PAIR) against the oracle, through the C ABI.

Every FP64 value of the 3D operator kernel is carried as a sum of two floats
(48 significant bits) and the multiply-adds run on the FP32 pipe.  The bar is
the FP64 parity bar of the native operator: <= 1e-12 relative (max norm)
against the oracle's jacobian_apply, for the apply, the transposed apply and
the residual, at every degree; solves must match the native FP64 solves.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def pdg():
    import __graft_entry__
    __graft_entry__.build()
    import pdg as m
    return m


@pytest.mark.parametrize("k,n", [(1, 5), (2, 4), (3, 3), (4, 3)])
@pytest.mark.parametrize("method", [0, 1, 2])
def test_float_pair_apply_matches_oracle(pdg, oracle, k, n, method):
    rng = np.random.default_rng(100 + 10 * k + method)
    nc = (n, n + 1, n)
    ncell = int(np.prod(nc))
    K = np.exp(1.5 * rng.standard_normal(ncell))
    c = rng.uniform(0.5, 2.0, ncell)
    bct = [1, -1, 1, 1, -3, 1]
    go = pdg.GridOperator(3, k, nc, method=method, alpha=3.0, bctype=bct)
    go.set_permeability(K)
    go.set_reaction(c)
    go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    P = oracle.Problem(3, k, nc, method=method, alpha=3.0, bctype=bct, K=K, c=c)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x, y0.copy())) <= TOL64
    yt = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, yt)
    assert _rel(yt, P.jacobian_apply_transpose(x)) <= TOL64
    go.close()


def test_float_pair_residual_and_solves(pdg, oracle):
    rng = np.random.default_rng(7)
    n = 6
    K = np.exp(rng.standard_normal(n ** 3))
    go = pdg.GridOperator(3, 2, (n, n, n), alpha=3.0)
    go.set_permeability(K)
    P = oracle.Problem(3, 2, (n, n, n), alpha=3.0, K=K)
    f = rng.uniform(-1, 1, (go.ncell, P.nq_volume))
    g = rng.uniform(-1, 1, P.nbpts_total())
    go.set_source(fq=f)
    go.set_boundary_data(g=g)
    P.set(fq=f, gq=g)
    x = rng.uniform(-1, 1, go.ndof)
    go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64
    sols = {}
    for mode in (pdg.F64_NATIVE, pdg.F64_FLOAT_PAIR):
        go.set_f64_arithmetic(mode)
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG)
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        slp.apply()
        assert slp.result().converged
        sols[mode] = (u, slp.result().iterations)
    (u64, it64), (ufp, itfp) = sols[pdg.F64_NATIVE], sols[pdg.F64_FLOAT_PAIR]
    assert abs(it64 - itfp) <= 1
    assert _rel(ufp, u64) <= 1e-9
    go.close()


def test_float_pair_rejected_in_2d(pdg):
    go = pdg.GridOperator(2, 2, (4, 4))
    with pytest.raises(pdg.PDGError):
        go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    go.close()


def test_float_pair_host_buffers_match_device(pdg):
    """Host-vector applies run the float-pair kernel over slabs of grid planes
    (cell ranges) with copies overlapped: the same bits as one device apply."""
    import torch
    rng = np.random.default_rng(9)
    n = 32
    go = pdg.GridOperator(3, 2, (n, n, n), alpha=3.0)
    go.set_permeability(rng.standard_normal(go.ncell), is_log=True)
    go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    yd = torch.tensor(y0, device="cuda")
    go.jacobian_apply(torch.tensor(x, device="cuda"), yd)
    yh = y0.copy()
    go.jacobian_apply(x, yh)
    assert np.array_equal(yh, yd.cpu().numpy())
    go.close()


@pytest.mark.parametrize("nc", [(1, 1, 1), (2, 1, 3)])
def test_float_pair_small_grids(pdg, oracle, nc):
    rng = np.random.default_rng(sum(nc))
    K = np.exp(rng.standard_normal(int(np.prod(nc))))
    go = pdg.GridOperator(3, 3, nc, alpha=3.0)
    go.set_permeability(K)
    go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    P = oracle.Problem(3, 3, nc, alpha=3.0, K=K)
    x = rng.uniform(-1, 1, go.ndof)
    y = np.zeros(go.ndof)
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x)) <= TOL64
    go.close()
