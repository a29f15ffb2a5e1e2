"""Assembled Jacobian on the GPU (GridOperator::jacobian with the
jacobian_volume/_skeleton/_boundary methods) against the oracle's assembled
blocks, its block product against the matrix-free apply, and the
matrix-based solve against the matrix-free one (equal iteration counts, as
the reference's matrix-free test asserts)."""
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


def _pair(pdg, oracle, dim, k, nc, seed, method=1, conv=False, react=True, weights=0):
    rng = np.random.default_rng(seed)
    ncell = int(np.prod(nc))
    K = np.exp(rng.standard_normal(ncell))
    c = rng.uniform(0.5, 1.5, ncell) if react else None
    go = pdg.GridOperator(dim, k, nc, alpha=3.0, method=method, weights=weights)
    go.set_permeability(K)
    kw = dict(K=K)
    if react:
        go.set_reaction(c)
        kw["c"] = c
    if conv:
        modes = pdg.fourier_velocity_modes(seed)
        go.set_velocity_modes(modes)
        kw["modes"] = modes
    P = oracle.Problem(dim, k, nc, alpha=3.0, method=method, weights=weights, **kw)
    return go, P, rng


def _slots_from_bcrs(go, rowptr, colind, vals):
    """BCRS (ascending columns) -> [ncell][2d+1][n][n] with slot 0 = diagonal,
    1 + f = neighbour across face f (-x,+x,-y,+y,-z,+z)."""
    d, nb = go.dim, go.nbasis
    nx = go.cfg.cells[0]
    ny = go.cfg.cells[1] if d > 1 else 1
    strides = [1, nx, nx * ny]
    out = np.zeros((go.ncell, 2 * d + 1, nb, nb))
    for e in range(go.ncell):
        for k in range(rowptr[e], rowptr[e + 1]):
            c = colind[k]
            if c == e:
                s = 0
            else:
                delta = c - e
                f = None
                for dd in range(d):
                    if delta == strides[dd]:
                        f = 2 * dd + 1
                    elif delta == -strides[dd]:
                        f = 2 * dd
                assert f is not None
                s = 1 + f
            out[e, s] = vals[k]
    return out


CASES = [
    dict(dim=2, k=1, nc=(5, 4), method=1),
    dict(dim=2, k=3, nc=(3, 4), method=0),
    dict(dim=3, k=2, nc=(3, 4, 2), method=1),
    dict(dim=3, k=1, nc=(4, 3, 3), method=2, weights=1),   # IIPG, weights off
    dict(dim=3, k=2, nc=(3, 3, 3), method=1, conv=True),
]


@pytest.mark.parametrize("case", CASES)
def test_assembled_blocks_match_oracle(pdg, oracle, case):
    go, P, rng = _pair(pdg, oracle, seed=7, **case)
    go.jacobian_assemble()
    nnz = go.jacobian_pattern()
    rowptr, colind, vals = go.jacobian_export()
    assert rowptr[-1] == nnz and len(colind) == nnz
    assert all(np.all(np.diff(colind[rowptr[e]:rowptr[e + 1]]) > 0) for e in range(go.ncell))
    ours = _slots_from_bcrs(go, rowptr, colind, vals)
    ref = P.assemble_jacobian()
    assert _rel(ours, ref) <= 1e-12


@pytest.mark.parametrize("case", CASES[2:])
def test_matrix_apply_matches_matrix_free(pdg, oracle, case):
    go, P, rng = _pair(pdg, oracle, seed=8, **case)
    go.jacobian_assemble()
    x = rng.uniform(-1, 1, go.ndof)
    y_mb = go.matrix_apply(x, np.zeros(go.ndof))
    y_mf = go.jacobian_apply(x, np.zeros(go.ndof))
    assert _rel(y_mb, y_mf) <= 1e-12


def test_assembled_export_to_device(pdg, oracle):
    torch = pytest.importorskip("torch")
    go, P, rng = _pair(pdg, oracle, 3, 2, (3, 3, 3), seed=9)
    go.jacobian_assemble()
    nnz = go.jacobian_pattern()
    dev = torch.zeros((nnz, go.nbasis, go.nbasis), dtype=torch.float64, device="cuda")
    rowptr, colind, host = go.jacobian_export()
    pdg._check(pdg.load().pdg_jacobian_export(go.handle, None, None, dev.data_ptr()))
    assert np.array_equal(dev.cpu().numpy(), host)


@pytest.mark.parametrize("method,conv", [(0, False), (1, True)])
def test_matrix_based_solve_same_iterations(pdg, oracle, method, conv):
    go, P, rng = _pair(pdg, oracle, 3, 2, (4, 4, 4), seed=10, conv=conv)
    go.set_source(fc=np.ones(go.ncell))
    meth = pdg.CG if method == 0 else pdg.BICGSTAB
    prec = pdg.PREC_BJ_FDM if not conv else pdg.PREC_BJ_DENSE
    res = {}
    for assembled in (0, 1):
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=meth, preconditioner=prec)
        ls.opts.assembled = assembled
        u = np.zeros(go.ndof)
        pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
        assert ls.result().converged
        res[assembled] = (u, ls.result().iterations)
    assert res[0][1] == res[1][1]
    assert _rel(res[1][0], res[0][0]) <= 1e-10
    # the adjoint solve through the assembled transpose
    rhs = rng.uniform(-1, 1, go.ndof)
    lam = {}
    for assembled in (0, 1):
        o = pdg.default_options(method=pdg.BICGSTAB, preconditioner=pdg.PREC_BJ_DENSE,
                                reduction=1e-11, assembled=assembled)
        lam[assembled] = np.zeros(go.ndof)
        assert go.adjoint_solve(rhs, lam[assembled], o).converged
    assert _rel(lam[1], lam[0]) <= 1e-9
