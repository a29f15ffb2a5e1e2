"""The oracle's parameter interface beyond A = K I, checked on the CPU.

ConvectionDiffusionDG takes A(cell, x) as a d x d tensor, evaluated at the
cell centre (convectiondiffusiondg.hh:124-127, :305-309, :710-713) or at
every quadrature point when permeabilityIsConstantPerCell() is false
(:141-146, :365-382, :750-761), and b(cell, x) and c(cell, x) at every
quadrature point (:178-181, :426, :797).  These tests pin the oracle's
restatement of those paths:
  * consistency: a tensor K I equals the scalar K, per-point data equal to
    the per-cell data reproduce it, per-point b sampled from the Fourier
    field reproduces the modes (all to rounding);
  * structure: the matrix-free apply equals the assembled blocks, the
    matrix-free transpose equals the transposed blocks, and a symmetric
    tensor keeps SIPG diffusion symmetric;
  * the PDE: manufactured solutions for an anisotropic full tensor and for
    a tensor varying inside the cells converge at O(h^{k+1}) in L2.
"""
import numpy as np
import pytest


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _l2err(P, u, exact, m):
    xyz, w, val = P.eval_points(u, m)
    return float(np.sum(w * (val - exact(xyz)) ** 2)) ** 0.5


def _spd_tensors(rng, n, d, aniso=4.0):
    """n random SPD d x d tensors: rotated diagonals with eigenvalues in
    [1, aniso]."""
    out = np.zeros((n, d, d))
    for e in range(n):
        q, _ = np.linalg.qr(rng.standard_normal((d, d)))
        lam = rng.uniform(1.0, aniso, d)
        out[e] = (q * lam) @ q.T
    return out


def _pointwise_from_cell(P, Acell):
    nqv, nqf, d = P.nq_volume, P.nq_face, P.dim
    Av = np.repeat(Acell[:, None], nqv, axis=1)
    Af = np.repeat(np.repeat(Acell[:, None, None], 2 * d, axis=1), nqf, axis=2)
    return Av, Af


@pytest.mark.parametrize("dim,k,n", [(2, 2, 4), (3, 2, 3), (3, 1, 3)])
def test_tensor_consistency(oracle, dim, k, n):
    rng = np.random.default_rng(10 + dim + k)
    nc = n ** dim
    K = np.exp(rng.standard_normal(nc))
    P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0, K=K, bctype=[1, 1, -1, 1, 1, -1])
    x = rng.uniform(-1, 1, P.ndof)
    y_scalar = P.jacobian_apply(x)
    Acell = np.einsum("e,ij->eij", K, np.eye(dim))
    P.set(Acell=Acell)
    assert _rel(P.jacobian_apply(x), y_scalar) <= 1e-15
    Av, Af = _pointwise_from_cell(P, Acell)
    P.set(Aq_vol=Av, Aq_face=Af)
    assert _rel(P.jacobian_apply(x), y_scalar) <= 1e-15
    # a full tensor per cell, then the same tensor at every point
    At = _spd_tensors(rng, nc, dim)
    P.set(Aq_vol=None, Aq_face=None, Acell=At)
    y_full = P.jacobian_apply(x)
    Av, Af = _pointwise_from_cell(P, At)
    P.set(Aq_vol=Av, Aq_face=Af)
    assert _rel(P.jacobian_apply(x), y_full) <= 1e-14


@pytest.mark.parametrize("dim,k,n", [(2, 3, 3), (3, 2, 3)])
def test_pointwise_velocity_and_reaction(oracle, dim, k, n):
    import pdg
    rng = np.random.default_rng(3)
    nc = n ** dim
    modes = pdg.fourier_velocity_modes(2)
    c = rng.uniform(0.5, 2.0, nc)
    P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0, K=np.exp(rng.standard_normal(nc)),
                       c=c, modes=modes)
    x = rng.uniform(-1, 1, P.ndof)
    y_modes = P.jacobian_apply(x)
    # b sampled at the volume points and at the face-lattice points
    bv = _fourier_b(modes, P.volume_points(), dim)
    bf = _fourier_b(modes, P.face_lattice_points(), dim)
    P.set_modes(None)
    P.set(bq_vol=bv, bq_face=bf)
    assert _rel(P.jacobian_apply(x), y_modes) <= 1e-14
    # c split into a per-cell and a per-point part
    P.set(c=0.25 * c, cq=np.repeat(0.75 * c[:, None], P.nq_volume, axis=1))
    assert _rel(P.jacobian_apply(x), y_modes) <= 1e-14


def _fourier_b(modes, xyz, dim):
    """b(x) = sum_m coef_m sin(2 pi kv_m . x + phase_m) at the given points."""
    b = np.zeros(xyz.shape[:-1] + (dim,))
    for m in modes:
        arg = m[3] + 2 * np.pi * sum(m[j] * xyz[..., j] for j in range(dim))
        for j in range(dim):
            b[..., j] += m[4 + j] * np.sin(arg)
    return b


@pytest.mark.parametrize("dim,k,n,method,pointwise", [
    (2, 2, 4, 1, False), (3, 2, 3, 1, False), (3, 1, 3, 0, True), (2, 3, 3, 2, True)])
def test_tensor_structure(oracle, dim, k, n, method, pointwise):
    rng = np.random.default_rng(20 + dim * k)
    nc = n ** dim
    P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0, method=method,
                       bctype=[1, 1, -1, 1, 1, 1])
    At = _spd_tensors(rng, nc, dim)
    if pointwise:
        # a tensor that varies from point to point inside each cell
        Av = _spd_tensors(rng, nc * P.nq_volume, dim).reshape(nc, P.nq_volume, dim, dim)
        Af = _spd_tensors(rng, nc * 2 * dim * P.nq_face, dim).reshape(
            nc, 2 * dim, P.nq_face, dim, dim)
        P.set(Aq_vol=Av, Aq_face=Af)
    else:
        P.set(Acell=At)
    x = rng.uniform(-1, 1, P.ndof)
    A = P.assemble_jacobian()
    y = P.jacobian_apply(x)
    assert _rel(P.blocks_apply(A, x), y) <= 1e-13
    assert _rel(P.jacobian_apply_transpose(x), P.blocks_apply(A, x, transpose=True)) <= 1e-13
    if method == 1 and not pointwise:
        # SIPG with a symmetric tensor per cell is symmetric
        assert _rel(P.blocks_apply(A, x, transpose=True), y) <= 1e-12


def _orders(errs, ns):
    return [np.log(errs[i] / errs[i + 1]) / np.log(ns[i + 1] / ns[i]) for i in range(len(ns) - 1)]


@pytest.mark.parametrize("dim,k,ns", [(2, 1, (4, 8, 16)), (2, 2, (4, 8, 16)), (3, 1, (3, 6, 12)),
                                      (3, 2, (2, 4, 8))])
def test_convergence_anisotropic_tensor(oracle, dim, k, ns):
    """u = prod sin(pi x_i), constant SPD A with off-diagonal entries:
    f = -div(A grad u) = pi^2 sum_i A_ii u - pi^2 sum_{i != j} A_ij
    cos(pi x_i) cos(pi x_j) prod_{l != i,j} sin(pi x_l)."""
    A = np.array([[2.0, 0.6, 0.3], [0.6, 1.0, -0.4], [0.3, -0.4, 1.5]])[:dim, :dim]

    def f(x):
        s, c = np.sin(np.pi * x), np.cos(np.pi * x)
        out = np.pi ** 2 * np.trace(A) * np.prod(s, axis=-1)
        for i in range(dim):
            for j in range(dim):
                if i != j:
                    rest = np.prod([s[..., l] for l in range(dim) if l not in (i, j)], axis=0) \
                        if dim > 2 else 1.0
                    out -= np.pi ** 2 * A[i, j] * c[..., i] * c[..., j] * rest
        return out

    exact = lambda x: np.prod(np.sin(np.pi * x), axis=-1)
    errs = []
    for n in ns:
        P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0)
        P.set(Acell=np.repeat(A[None], P.ncell, axis=0), fq=f(P.volume_points()))
        u, res, st = P.solve(solver="cg", op=0, reduction=1e-12)
        assert st == 0 and res.converged
        errs.append(_l2err(P, u, exact, k + 3))
    rates = _orders(errs, ns)
    print(f"anisotropic tensor d={dim} k={k}: L2 errors {errs}, orders {rates}")
    assert min(rates[1:]) > k + 1 - 0.3, (errs, rates)


@pytest.mark.parametrize("dim,k,ns", [(2, 1, (4, 8, 16)), (2, 2, (4, 8, 16)), (3, 2, (2, 4, 8))])
def test_convergence_pointwise_tensor(oracle, dim, k, ns):
    """A(x) = (1 + x_0) I evaluated at every quadrature point
    (permeabilityIsConstantPerCell() == false), u = prod sin(pi x_i):
    f = (1 + x_0) d pi^2 u - pi cos(pi x_0) prod_{l>0} sin(pi x_l)."""
    exact = lambda x: np.prod(np.sin(np.pi * x), axis=-1)

    def f(x):
        s = np.sin(np.pi * x)
        return (1 + x[..., 0]) * dim * np.pi ** 2 * np.prod(s, axis=-1) \
            - np.pi * np.cos(np.pi * x[..., 0]) * np.prod(s[..., 1:], axis=-1)

    errs = []
    for n in ns:
        P = oracle.Problem(dim, k, (n,) * dim, alpha=3.0)
        I = np.eye(dim)
        Av = (1 + P.volume_points()[..., 0])[..., None, None] * I
        Af = (1 + P.cell_face_points()[..., 0])[..., None, None] * I
        P.set(Aq_vol=Av, Aq_face=Af, fq=f(P.volume_points()))
        u, res, st = P.solve(solver="cg", op=0, reduction=1e-12)
        assert st == 0 and res.converged
        errs.append(_l2err(P, u, exact, k + 3))
    rates = _orders(errs, ns)
    print(f"pointwise tensor d={dim} k={k}: L2 errors {errs}, orders {rates}")
    assert min(rates[1:]) > k + 1 - 0.3, (errs, rates)
