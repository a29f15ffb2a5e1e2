"""Convection on 2D grids through the C ABI, against the oracle.

In 2D the upwind convection terms of ConvectionDiffusionDG (volume -u b.grad
psi, the skeleton's upwind flux, Dirichlet inflow and outflow faces;
localoperator/convectiondiffusiondg.hh:175-186, 424-443, 796-849) run inside
the Gauss-point operator.  Checked: apply and transposed apply <= 1e-12 with
Fourier-mode and point-data velocities, the outflow-on-inflow error, and the
advection problem of dune/pdelab/test/testdglegendre.cc (:26-194) solved on the
GPU in the Lagrange, Legendre and Lobatto spaces against the oracle's solutions
and the reference's criterion (L2 difference squared < 1e-14 between the
spaces).
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


def _modes_2d(rng, n=4):
    m = np.zeros((n, 7))
    m[:, 0:2] = rng.integers(0, 3, (n, 2))
    m[:, 3] = rng.uniform(0, 2 * np.pi, n)
    m[:, 4:6] = rng.uniform(-2, 2, (n, 2))
    return m


@pytest.mark.parametrize("k,n", [(1, 6), (2, 5), (3, 4), (4, 3)])
@pytest.mark.parametrize("method", [0, 1, 2])
def test_convection_2d_apply_and_transpose(pdg, oracle, k, n, method):
    rng = np.random.default_rng(200 + 10 * k + method)
    nc = (n, n + 1)
    ncell = n * (n + 1)
    K = np.exp(rng.standard_normal(ncell))
    c = rng.uniform(0.5, 2.0, ncell)
    m = _modes_2d(rng)
    bct = [1, 1, -1, 1]
    go = pdg.GridOperator(2, k, nc, method=method, alpha=3.0, bctype=bct)
    go.set_permeability(K)
    go.set_reaction(c)
    go.set_velocity_modes(m)
    P = oracle.Problem(2, k, nc, method=method, alpha=3.0, bctype=bct, K=K, c=c, modes=m)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    y = y0.copy()
    go.jacobian_apply(x, y)
    assert _rel(y, P.jacobian_apply(x, y0.copy())) <= TOL64
    yt = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, yt)
    assert _rel(yt, P.jacobian_apply_transpose(x)) <= TOL64
    go.close()


def test_convection_2d_point_velocity_and_residual(pdg, oracle):
    rng = np.random.default_rng(77)
    nc = (5, 4)
    bct = [1, -2, 1, 1]      # outflow on +x
    go = pdg.GridOperator(2, 3, nc, alpha=3.0, bctype=bct)
    P = oracle.Problem(2, 3, nc, alpha=3.0, bctype=bct)
    K = np.exp(rng.standard_normal(go.ncell))
    go.set_permeability(K)

    def b_at(x):
        b = np.zeros(x.shape[:-1] + (3,))
        b[..., 0] = 1.5 + 0.5 * np.sin(2 * np.pi * x[..., 1])
        b[..., 1] = np.cos(2 * np.pi * x[..., 0])
        return b
    bv, bf = b_at(go.volume_points()), b_at(go.face_lattice_points())
    go.set_velocity_points(bv, bf)
    # the oracle holds dim components per point, the C ABI three
    P.set(K=K, bq_vol=bv[..., :2], bq_face=bf[..., :2])
    f = rng.uniform(-1, 1, (go.ncell, P.nq_volume))
    g = rng.uniform(-1, 1, P.nbpts_total())
    o = rng.uniform(-1, 1, P.nbpts_total())
    go.set_source(fq=f)
    go.set_boundary_data(g=g, o=o)
    P.set(fq=f, gq=g, oq=o)
    x = rng.uniform(-1, 1, go.ndof)
    r = np.zeros(go.ndof)
    go.residual(x, r)
    assert _rel(r, P.residual(x)) <= TOL64
    yt = np.zeros(go.ndof)
    go.jacobian_apply_transpose(x, yt)
    assert _rel(yt, P.jacobian_apply_transpose(x)) <= TOL64
    go.close()


def test_convection_2d_outflow_on_inflow_refused(pdg):
    go = pdg.GridOperator(2, 1, (3, 3), bctype=[-2, -2, -2, -2])
    m = np.array([[0, 0, 0, np.pi / 2, 1.0, 0.0, 0.0]])   # b = (1, 0): inflow at -x
    with pytest.raises(pdg.PDGError) as e:
        go.set_velocity_modes(m)
    assert e.value.status == pdg.PDG_EOUTFLOW
    go.close()


def _advection(pdg, oracle, basis, cells=10):
    # GenericAdvectionProblem of testdglegendre.cc:26-111 (b = (1, 1/3), A = 0,
    # Dirichlet inflow g = 0 below y = x/3 + 1/4 and 1 above, outflow elsewhere),
    # SIPG, alpha = 2, degree 1 on cells x cells
    B, O = pdg.BC_DIRICHLET, pdg.BC_OUTFLOW
    modes = np.array([[0, 0, 0, np.pi / 2, 1.0, 1.0 / 3.0, 0.0]])
    go = pdg.GridOperator(2, 1, (cells, cells), alpha=2.0, bctype=[B, O, B, O], basis=basis)
    go.set_permeability(np.zeros(go.ncell))
    go.set_velocity_modes(modes)
    bp = go.boundary_points()
    g = np.where(bp[:, 1] < bp[:, 0] / 3.0 + 0.25, 0.0, 1.0)
    go.set_boundary_data(g=g)
    P = oracle.Problem(2, 1, (cells, cells), alpha=2.0, bctype=[B, O, B, O],
                       K=np.zeros(cells * cells), modes=modes, gq=g, basis=basis)
    return go, P


def test_testdglegendre_on_gpu(pdg, oracle):
    sols = {}
    for name, b in (("lagrange", pdg.LAGRANGE), ("legendre", pdg.LEGENDRE),
                    ("lobatto", pdg.LOBATTO)):
        go, P = _advection(pdg, oracle, b)
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                                 preconditioner=pdg.PREC_BJ_DENSE)
        u = np.zeros(go.ndof)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-12)
        slp.apply()
        assert slp.result().converged
        uref, res, st = P.solve(solver="bicgstab", op=0, reduction=1e-12)
        assert st == 0 and res.converged
        assert _rel(u, uref) <= 1e-9
        sols[name] = (P, u)
        go.close()
    Pl, ul = sols["lagrange"]
    _, w, vl = Pl.eval_points(ul, 6)
    for name in ("legendre", "lobatto"):
        P, u = sols[name]
        _, _, v = P.eval_points(u, 6)
        assert float(np.sum(w * (v - vl) ** 2)) < 1e-14, name   # testdglegendre.cc:190
