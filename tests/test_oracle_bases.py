"""The oracle's Legendre and Gauss-Lobatto QkDG bases.

Pins:
  * dune/pdelab/test/testdglegendre.cc:146-194: the DG solution of the
    advection problem (:26-111) in the Legendre space equals the one in the
    Lagrange space, L2 difference squared < 1e-14 (:183-191);
  * the published Gauss-Lobatto rule (nodes 0, (1 -/+ sqrt(3/7))/2, 1/2, 1
    for five points; exact to degree 2m-3);
  * congruence of the local forms under the change of basis.
"""
import numpy as np
import pytest


def test_gauss_lobatto_rule(oracle):
    x, w = oracle.gauss_lobatto(5)
    ref = [0.0, (1 - np.sqrt(3 / 7)) / 2, 0.5, (1 + np.sqrt(3 / 7)) / 2, 1.0]
    assert np.allclose(x, ref, atol=1e-15, rtol=0)
    assert np.allclose(w, [1 / 20, 49 / 180, 16 / 45, 49 / 180, 1 / 20], atol=1e-15, rtol=0)
    for m in range(2, 9):
        x, w = oracle.gauss_lobatto(m)
        assert x[0] == 0.0 and x[-1] == 1.0 and np.all(np.diff(x) > 0)
        for p in range(2 * m - 2):
            assert abs(np.dot(w, x ** p) - 1.0 / (p + 1)) < 1e-14


def test_basis_values(oracle):
    L, LEG, LOB = oracle.LAGRANGE, oracle.LEGENDRE, oracle.LOBATTO
    for k in range(1, 6):
        xl, _ = oracle.gauss_lobatto(k + 1)
        for i in range(k + 1):
            # Legendre on [0,1]: P_i(0) = (-1)^i, P_i(1) = 1
            assert abs(oracle.basis1d(LEG, k, i, 0.0) - (-1) ** i) < 1e-14
            assert abs(oracle.basis1d(LEG, k, i, 1.0) - 1.0) < 1e-14
            for j in range(k + 1):
                assert abs(oracle.basis1d(LOB, k, i, xl[j]) - (i == j)) < 1e-13
                assert abs(oracle.basis1d(L, k, i, j / k) - (i == j)) < 1e-14


def _T1(oracle, basis, k):
    """1D matrix taking coefficients of `basis` to equidistant Lagrange ones."""
    n = k + 1
    return np.array([[oracle.basis1d(basis, k, i, j / k) for i in range(n)] for j in range(n)])


def _kron(T, dim):
    out = T
    for _ in range(dim - 1):
        out = np.kron(T, out)
    return out


def _cellwise(M, v, nb):
    return (v.reshape(-1, nb) @ M.T).ravel()


@pytest.mark.parametrize("dim,k,n", [(2, 2, (4, 3)), (3, 1, (3, 2, 2)), (3, 3, (2, 2, 2))])
@pytest.mark.parametrize("basis", ["legendre", "lobatto"])
def test_congruence(oracle, dim, k, n, basis):
    b = oracle.LEGENDRE if basis == "legendre" else oracle.LOBATTO
    rng = np.random.default_rng(k + dim)
    ncell = int(np.prod(n))
    K = np.exp(rng.standard_normal(ncell))
    Pl = oracle.Problem(dim, k, n, alpha=3.0, K=K)
    Pb = oracle.Problem(dim, k, n, alpha=3.0, K=K, basis=b)
    T = _kron(_T1(oracle, b, k), dim)
    nb = (k + 1) ** dim
    x = rng.uniform(-1, 1, Pb.ndof)
    y = Pb.jacobian_apply(x)
    yl = _cellwise(T.T, Pl.jacobian_apply(_cellwise(T, x, nb)), nb)
    assert np.max(np.abs(y - yl)) <= 1e-12 * np.max(np.abs(y))


def _advection_problem(oracle, basis, cells=10):
    # GenericAdvectionProblem of testdglegendre.cc:26-111: A = 0, b = (1, 1/3),
    # c = f = 0, Dirichlet on inflow sides (n.b < 0) with g = 0 below the line
    # y = x/3 + 1/4 and 1 above, outflow elsewhere; SIPG, weightsOn, alpha = 2
    # (:127-128), QkDG degree 1 on a cells x cells YaspGrid (:146-167)
    B, O = oracle.BC_DIRICHLET, oracle.BC_OUTFLOW
    modes = np.array([[0, 0, 0, np.pi / 2, 1.0, 1.0 / 3.0, 0.0]])
    P = oracle.Problem(2, 1, (cells, cells), alpha=2.0, bctype=[B, O, B, O],
                       K=np.zeros(cells * cells), modes=modes, basis=basis)
    bp = P.boundary_points()
    P.set(gq=np.where(bp[:, 1] < bp[:, 0] / 3.0 + 0.25, 0.0, 1.0))
    return P


def test_testdglegendre(oracle):
    sols = {}
    for name, b in (("lagrange", oracle.LAGRANGE), ("legendre", oracle.LEGENDRE),
                    ("lobatto", oracle.LOBATTO)):
        P = _advection_problem(oracle, b)
        u, res, st = P.solve(solver="bicgstab", op=0, reduction=1e-12)
        assert st == 0 and res.converged
        sols[name] = (P, u)
    Pl, ul = sols["lagrange"]
    _, _, vl = Pl.eval_points(ul, 6)        # integrateGridFunction order 10
    _, w, _ = Pl.eval_points(ul, 6)
    for name in ("legendre", "lobatto"):
        P, u = sols[name]
        _, _, v = P.eval_points(u, 6)
        l2 = float(np.sum(w * (v - vl) ** 2))
        assert l2 < 1e-14, name           # testdglegendre.cc:190
