"""The oracle reproduces the reference tests' own assertions.

The reference ships no golden vectors; these assertions are the pins:
  * dune/pdelab/test/matrixfree/matrix_free_linear.cc:387-393
  * dune/pdelab/test/testfastdgassembler.cc:160-175
  * dune/pdelab/test/testblocklocaloperatorwrapper.cc:200-276
  * dune/pdelab/test/testconvectiondiffusiondg.cc:160-168
  * dune/pdelab/test/testinstationaryfastdgassembler.cc:226-235
"""
import numpy as np
import pytest


def _mfl_problem(O, n=16, k=1, alpha=3.0):
    # PoissonProblem of matrix_free_linear.cc:28-60: g = exp(-|x-1/2|^2),
    # f = 4 (1 - c) g, SIPG, weightsOn, alpha = 3 (:104-108)
    P = O.Problem(2, k, (n, n), alpha=alpha)
    vp = P.volume_points()
    c = (0.5 - vp[..., 0]) ** 2 + (0.5 - vp[..., 1]) ** 2
    P.set(fq=4 * (1 - c) * np.exp(-c))
    bp = P.boundary_points()
    cb = (0.5 - bp[:, 0]) ** 2 + (0.5 - bp[:, 1]) ** 2
    P.set(gq=np.exp(-cb))
    return P


def _l2err2(P, u, exact, m=6):
    xyz, w, val = P.eval_points(u, m)
    return float(np.sum(w * (val - exact(xyz)) ** 2))


def test_gauss_legendre(oracle):
    for m in range(1, 9):
        x, w = oracle.gauss_legendre(m)
        assert abs(w.sum() - 1) < 1e-15
        # exact for polynomials of degree 2m-1 on [0,1]
        for p in range(2 * m):
            assert abs(np.dot(w, x ** p) - 1.0 / (p + 1)) < 1e-14


def test_lagrange_nodes(oracle):
    L = oracle.lib()
    for k in range(1, 6):
        for i in range(k + 1):
            for j in range(k + 1):
                assert abs(L.pdgo_lagrange(k, i, j / k) - (i == j)) < 1e-14


@pytest.mark.parametrize("solver", ["bicgstab", "cg"])
def test_matrix_free_linear(oracle, solver):
    P = _mfl_problem(oracle)
    u_mb, res_mb, st = P.solve(solver=solver, op=1, reduction=1e-12)
    assert st == 0
    u_mf, res_mf, st = P.solve(solver=solver, op=0, reduction=1e-12)
    assert st == 0
    assert res_mb.converged and res_mf.converged
    # equal Krylov iteration counts, matrix-based vs matrix-free (:392-393), at
    # the test's own size (matrix_free_linear.ini: cells = 16, refine = 0;
    # reduction 1e-12)
    print(f"{solver}: matrix-based {res_mb.iterations}, matrix-free {res_mf.iterations} iterations")
    assert res_mb.iterations == res_mf.iterations
    exact = lambda x: np.exp(-((0.5 - x[..., 0]) ** 2 + (0.5 - x[..., 1]) ** 2))
    err = _l2err2(P, u_mf, exact, 6)     # integrateGridFunction order 10
    assert err < 1e-6                    # (:387-391)


def test_fastdg_assembler(oracle):
    # ParameterA of testfastdgassembler.cc: g = exp(-|x|^2), f = (2d - 4|x|^2) g,
    # SIPG alpha = 2, 32x32 (refine 5), CG, reduction 1e-12
    P = oracle.Problem(2, 1, (32, 32), alpha=2.0)
    vp = P.volume_points()
    nrm = (vp ** 2).sum(-1)
    P.set(fq=(4 - 4 * nrm) * np.exp(-nrm))
    bp = P.boundary_points()
    P.set(gq=np.exp(-(bp ** 2).sum(-1)))
    u, res, st = P.solve(solver="cg", op=0, reduction=1e-12)
    assert st == 0 and res.converged
    err = _l2err2(P, u, lambda x: np.exp(-(x ** 2).sum(-1)), 7)   # order 12
    assert err < 1e-8


@pytest.mark.parametrize("dim,k,n", [(2, 1, 16), (2, 2, 6), (3, 1, 4), (3, 2, 3)])
def test_block_diagonal_identity(oracle, dim, k, n):
    # testblocklocaloperatorwrapper.cc:200-276: the wrapper's diagonal blocks
    # equal the assembled Jacobian's diagonal blocks to 1e-14
    rng = np.random.default_rng(1)
    P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0)
    P.set(K=np.exp(rng.standard_normal(P.ncell)))
    A = P.assemble_jacobian()
    D = P.block_diagonal()
    assert np.max(np.abs(A[:, 0] - D)) <= 1e-14 * np.max(np.abs(D))


@pytest.mark.parametrize("dim,k,n", [(2, 1, 8), (2, 3, 4), (3, 2, 3)])
def test_matrix_free_equals_assembled(oracle, dim, k, n):
    rng = np.random.default_rng(2)
    P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0)
    P.set(K=np.exp(rng.standard_normal(P.ncell)))
    x = rng.uniform(-1, 1, P.ndof)
    y = P.jacobian_apply(x)
    A = P.assemble_jacobian()
    y2 = P.blocks_apply(A, x)
    assert np.max(np.abs(y - y2)) <= 1e-13 * np.max(np.abs(y))
    # SIPG pure diffusion is symmetric: A^T x == A x
    y3 = P.blocks_apply(A, x, transpose=True)
    assert np.max(np.abs(y3 - y)) <= 1e-12 * np.max(np.abs(y))


@pytest.mark.parametrize("dim,k,n", [(2, 1, 5), (2, 4, 3), (3, 1, 3), (3, 2, 3), (3, 3, 2),
                                     (3, 4, 2)])
def test_matrix_free_transpose_equals_assembled(oracle, dim, k, n):
    # the checker of the GPU transposed applies: the oracle's matrix-free
    # transpose (NIPG, weights on, reaction, mixed boundary types) equals the
    # transpose of its assembled blocks, and the operator is not symmetric
    rng = np.random.default_rng(30 + dim * 10 + k)
    nc = (n,) * dim
    ncell = n ** dim
    P = oracle.Problem(dim, k, nc, method=0, weights=1, alpha=3.0,
                       bctype=[1, -1, -3, 1, -1, 1][:2 * dim],
                       K=np.exp(rng.standard_normal(ncell)), c=rng.uniform(0.5, 2.0, ncell))
    x = rng.uniform(-1, 1, P.ndof)
    A = P.assemble_jacobian()
    yt = P.jacobian_apply_transpose(x)
    assert np.max(np.abs(yt - P.blocks_apply(A, x, transpose=True))) <= 1e-13 * np.max(np.abs(yt))
    y = P.jacobian_apply(x)
    assert np.max(np.abs(yt - y)) > 1e-6 * np.max(np.abs(y))


@pytest.mark.parametrize("dim,k,ns", [
    (2, 1, (4, 8, 16)), (2, 2, (4, 8, 16)), (2, 3, (2, 4, 8)), (2, 4, (2, 4, 8)),
    (3, 1, (3, 6, 12)), (3, 2, (2, 4, 8)), (3, 3, (2, 4, 6)), (3, 4, (2, 3, 4))])
def test_convergence_order(oracle, dim, k, ns):
    # manufactured u = prod_i sin(pi x_i), K = 1, f = d pi^2 u, homogeneous
    # Dirichlet: the L2 error falls as O(h^{k+1}) over three grids
    exact = lambda x: np.prod(np.sin(np.pi * x), axis=-1)
    errs = []
    for n in ns:
        P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0)
        P.set(fq=dim * np.pi ** 2 * exact(P.volume_points()))
        u, res, st = P.solve(solver="cg", op=0, reduction=1e-13)
        assert st == 0 and res.converged
        errs.append(_l2err2(P, u, exact, k + 3) ** 0.5)
    rates = [np.log(errs[i] / errs[i + 1]) / np.log(ns[i + 1] / ns[i]) for i in range(len(ns) - 1)]
    print(f"d={dim} k={k} grids {ns}: L2 errors {errs}, orders {rates}")
    assert rates[-1] > k + 1 - 0.35, (errs, rates)
    assert rates[0] > k + 1 - 1.0, (errs, rates)


def test_convection_matrix_free_equals_assembled(oracle):
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "dune-pdelab_gb300"))
    import pdg
    rng = np.random.default_rng(4)
    m = pdg.fourier_velocity_modes(3)
    for method in (oracle.SIPG, oracle.NIPG):
        P = oracle.Problem(3, 2, (3, 3, 3), alpha=3.0, method=method,
                           K=np.exp(rng.standard_normal(27)), c=np.ones(27), modes=m)
        x = rng.uniform(-1, 1, P.ndof)
        y = P.jacobian_apply(x)
        A = P.assemble_jacobian()
        assert np.max(np.abs(y - P.blocks_apply(A, x))) <= 1e-13 * np.max(np.abs(y))


def test_block_sor_and_iterative_jacobi_oracle(oracle):
    """The oracle's block SOR sweep equals the explicit triangular solve
    omega (D + omega L)^{-1} d, and the iterative block Jacobi matches the
    exact block inverse to its block-solver reduction."""
    import numpy as np
    rng = np.random.default_rng(3)
    P = oracle.Problem(2, 2, (4, 3), alpha=3.0, K=np.exp(rng.standard_normal(12)))
    nb, nc = P.nb, P.ncell
    A = P.assemble_jacobian()
    dense = np.zeros((P.ndof, P.ndof))
    strides = [1, 4]
    for e in range(nc):
        ix = (e % 4, e // 4)
        for s in range(5):
            if s == 0:
                n = e
            else:
                f = s - 1
                dd, hi = f // 2, f % 2
                j = ix[dd] + (1 if hi else -1)
                if j < 0 or j >= (4, 3)[dd]:
                    continue
                n = e + (strides[dd] if hi else -strides[dd])
            dense[e * nb:(e + 1) * nb, n * nb:(n + 1) * nb] = A[e, s]
    d = rng.uniform(-1, 1, P.ndof)
    omega = 1.2
    Dm = np.zeros_like(dense)
    Lm = np.zeros_like(dense)
    for e in range(nc):
        sl = slice(e * nb, (e + 1) * nb)
        Dm[sl, sl] = dense[sl, sl]
        Lm[sl, :e * nb] = dense[sl, :e * nb]
    v, _ = P.prec_apply_cfg(oracle.prec_config(16 | 2, omega=omega), d)
    vref = omega * np.linalg.solve(Dm + omega * Lm, d)
    assert np.max(np.abs(v - vref)) <= 1e-12 * np.max(np.abs(vref))
    vt, _ = P.prec_apply_cfg(oracle.prec_config(16 | 2, omega=omega), d, transpose=True)
    vtref = omega * np.linalg.solve((Dm + omega * Lm).T, d)
    assert np.max(np.abs(vt - vtref)) <= 1e-12 * np.max(np.abs(vtref))
    vi, its = P.prec_apply_cfg(oracle.prec_config(3), d)
    vex = np.linalg.solve(Dm, d)
    assert np.max(np.abs(vi - vex)) <= 1e-4 * np.max(np.abs(vex))
    assert its.min() >= 1 and its.max() <= 100


@pytest.mark.parametrize("dim,k,method", [(2, 1, 1), (2, 3, 0), (3, 2, 2), (3, 1, 1)])
def test_residual_is_affine_with_jacobian(oracle, dim, k, method):
    # R(x) - R(0) = J x for the linear operator with source, Dirichlet, Neumann
    # and outflow data on mixed sides: the residual's data terms (lambda_*)
    # and the Jacobian's forms (alpha_* / jacobian_apply_*) are consistent
    rng = np.random.default_rng(90 + dim * 10 + k)
    nc = (3,) * dim
    ncell = 3 ** dim
    P = oracle.Problem(dim, k, nc, alpha=3.0, method=method, bctype=[1, -1, -2, 1, -1, 1][:2 * dim],
                       K=np.exp(rng.standard_normal(ncell)), c=rng.uniform(0.5, 1.5, ncell))
    nbp = P.nbpts_total()
    P.set(fq=rng.standard_normal(ncell * (k + 1) ** dim), gq=rng.standard_normal(nbp),
          jq=rng.standard_normal(nbp), oq=rng.standard_normal(nbp))
    x = rng.uniform(-1, 1, P.ndof)
    r0 = P.residual(np.zeros(P.ndof))
    assert np.max(np.abs(r0)) > 0.1
    lhs = P.residual(x) - r0
    jx = P.jacobian_apply(x)
    assert np.max(np.abs(lhs - jx)) <= 1e-13 * np.max(np.abs(jx))


@pytest.mark.parametrize("dim,k,nc", [(2, 2, (4, 3)), (3, 1, (3, 3, 2)), (3, 3, (2, 2, 2))])
def test_nonlinear_jacobian_central_differences(oracle, dim, k, nc):
    # the checker of the GPU jacobian_apply(x, z, y): the oracle's Jacobian of
    # the operator with the volume term int q(u) psi (NIPG, reaction) against
    # central differences of its own residual
    rng = np.random.default_rng(70 + dim * 10 + k)
    ncell = int(np.prod(nc))
    P = oracle.Problem(dim, k, nc, alpha=3.0, method=0, K=np.exp(rng.standard_normal(ncell)),
                       c=rng.uniform(0.5, 1.5, ncell))
    P.set_nonlinearity([0.3, -0.5, 2.0, 1.0])
    x = rng.uniform(-1, 1, P.ndof)
    z = rng.uniform(-1, 1, P.ndof)
    P.set_linearization_point(x)
    jz = P.jacobian_apply(z)
    h = 1e-5
    fd = (P.residual(x + h * z) - P.residual(x - h * z)) / (2 * h)
    assert np.max(np.abs(fd - jz)) <= 1e-7 * np.max(np.abs(jz))
    P.set_linearization_point(None)


def test_nonlinear_reference_problem_oracle(oracle):
    """matrix_free_nonlinear.cc:386-405: Newton on q(u) = 2 u^2, g = |x|^2
    (2D Q1 16^2, SIPG, weightsOn, alpha 3) reaches L2 error^2 < 1e-6; the
    oracle's nonlinear Jacobian matches central differences of its residual."""
    import numpy as np
    n = 16
    P = oracle.Problem(2, 1, (n, n), alpha=3.0)
    P.set_nonlinearity([0.0, 0.0, 2.0])
    xv = P.volume_points().reshape(-1, 2)
    g = (xv ** 2).sum(1)
    xb = P.boundary_points().reshape(-1, 2)
    P.set(fq=-4.0 + 2.0 * g * g, gq=(xb ** 2).sum(1))
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 1, P.ndof)
    z = rng.uniform(-1, 1, P.ndof)
    P.set_linearization_point(x)
    Jz = P.jacobian_apply(z)
    eps = 1e-6
    fd = (P.residual(x + eps * z) - P.residual(x - eps * z)) / (2 * eps)
    assert np.max(np.abs(Jz - fd)) <= 1e-8 * np.max(np.abs(fd))
    P.set_linearization_point(None)
    u, res, st = P.newton(oracle.prec_config(2), solver="bicgstab")
    assert st == 0 and res.converged and res.iterations <= 6
    xyz, w, val = P.eval_points(u, 6)
    assert float((w * (val - (xyz ** 2).sum(-1)) ** 2).sum()) < 1e-6


def test_onestep_orders_oracle(oracle):
    """The oracle's one-step methods (tables of instationary/onestepparameter.hh)
    converge to the exact semi-discrete solution exp(-M^{-1}J t) at their
    orders: implicit Euler 1, Crank-Nicolson 2, Alexander2 2, Heun 2, RK4 4."""
    import numpy as np
    scipy_linalg = __import__("pytest").importorskip("scipy.linalg")
    n = 4
    P = oracle.Problem(2, 1, (n, n), alpha=3.0)
    P.set(fc=np.ones(n * n))
    N = P.ndof
    E = np.eye(N)
    J = np.column_stack([P.jacobian_apply(E[i]) for i in range(N)])
    M = np.column_stack([P.mass_apply(E[i]) for i in range(N)])
    L = np.linalg.solve(M, J)
    ustar = np.linalg.solve(J, -P.residual(np.zeros(N)))
    u0 = np.sin(np.arange(N))
    al = 1 - 0.5 * np.sqrt(2)
    cases = {
        "IE": (np.array([[-1, 1.]]), np.array([[0, 1.]]), 1, 0.05, (8, 16, 32)),
        "CN": (np.array([[-1, 1.]]), np.array([[0.5, 0.5]]), 2, 0.05, (16, 32, 64)),
        "A2": (np.array([[-1, 1, 0], [-1, 0, 1.]]), np.array([[0, al, 0], [0, 1 - al, al]]), 2,
               0.05, (8, 16, 32)),
        "Heun": (np.array([[-1, 1, 0], [-0.5, -0.5, 1.]]), np.array([[1, 0, 0], [0, 0.5, 0.]]), 2,
                 0.01, (40, 80, 160)),
        "RK4": (np.array([[-1, 1, 0, 0, 0], [-1, 0, 1, 0, 0], [-1, 0, 0, 1, 0], [-1, 0, 0, 0, 1.]]),
                np.array([[.5, 0, 0, 0, 0], [0, .5, 0, 0, 0], [0, 0, 1, 0, 0],
                          [1 / 6, 1 / 3, 1 / 3, 1 / 6, 0]]), 4, 0.01, (40, 80, 160)),
    }
    for name, (A, B, order, T, steps) in cases.items():
        ue = ustar + scipy_linalg.expm(-L * T) @ (u0 - ustar)
        errs = []
        for m in steps:
            x = u0.copy()
            for _ in range(m):
                x, _ = P.onestep(A, B, T / m, x, oracle.prec_config(2), reduction=1e-13)
            errs.append(np.abs(x - ue).max())
        rate = np.log2(errs[-2] / errs[-1])
        assert abs(rate - order) < 0.25, (name, errs)


def test_convectiondiffusiondg_default_constructor(oracle):
    """testconvectiondiffusiondg.cc: the same Poisson problem with the local
    operator's default arguments (SIPG, weightsOn, alpha = 1,
    convectiondiffusiondg.hh:85-90) on 16x16 Q1, solved to reduction 1e-12
    (SuperLU there, an assembled Krylov solve here): L2 error squared < 1e-6
    (:160-168)."""
    P = _mfl_problem(oracle, alpha=1.0)
    u, res, st = P.solve(solver="bicgstab", op=1, reduction=1e-12)
    assert st == 0 and res.converged
    exact = lambda x: np.exp(-((0.5 - x[..., 0]) ** 2 + (0.5 - x[..., 1]) ** 2))
    assert _l2err2(P, u, exact, 6) < 1e-6


def test_instationary_fastdg_assembler(oracle):
    """testinstationaryfastdgassembler.cc: ParameterA (g = exp(-|x|^2),
    f = (2d - 4|x|^2) g, Dirichlet; :24-118) on the unit square refined to
    8x8, Q1, SIPG weightsOn alpha = 2 (:144), L2 mass (:152), initial value the
    nodal interpolant of g (:181), one Alexander2 step of dt = 0.1 to T = 0.1
    (:204-221), CG to 1e-10: L2 error squared < 5e-6 against g (integration
    order 12; :226-235)."""
    n, k = 8, 1
    P = oracle.Problem(2, k, (n, n), alpha=2.0)
    vp = P.volume_points()
    nrm = (vp ** 2).sum(-1)
    P.set(fq=(4 - 4 * nrm) * np.exp(-nrm))
    bp = P.boundary_points()
    P.set(gq=np.exp(-(bp ** 2).sum(-1)))
    h = 1.0 / n
    x0 = np.zeros(P.ndof)
    for cy in range(n):
        for cx in range(n):
            for j in range(k + 1):
                for i in range(k + 1):
                    X, Y = (cx + i / k) * h, (cy + j / k) * h
                    x0[(cx + n * cy) * (k + 1) ** 2 + i + (k + 1) * j] = np.exp(-(X * X + Y * Y))
    al = 1 - 0.5 * np.sqrt(2)          # Alexander2Parameter
    A = np.array([[-1, 1, 0], [-1, 0, 1.]])
    B = np.array([[0, al, 0], [0, 1 - al, al]])
    x1, its = P.onestep(A, B, 0.1, x0, oracle.prec_config(1), solver="cg", reduction=1e-10)
    assert its > 0
    exact = lambda x: np.exp(-(x ** 2).sum(-1))
    assert _l2err2(P, x1, exact, 7) < 5e-6
