"""Generate the golden fixtures in this directory from the CPU oracle.

The reference (PDELab) cannot be built here and ships no golden vectors, so
the fixtures come from the oracle, which is pinned to the reference tests'
assertions (tests/test_oracle_pins.py).  Inputs are seeded; run
``python tests/golden/make_golden.py`` to regenerate.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import pdg_oracle as O  # noqa: E402


def apply_case(name, dim, k, n, seed, **kw):
    rng = np.random.default_rng(seed)
    nc = (n,) * dim
    P = O.Problem(dim, k, nc, alpha=3.0, **kw)
    K = np.exp(rng.standard_normal(P.ncell))
    P.set(K=K)
    x = rng.uniform(-1, 1, P.ndof)
    y = P.jacobian_apply(x)
    A = P.assemble_jacobian()
    yt = P.blocks_apply(A, x, transpose=True)
    lu, piv = P.lu(P.block_diagonal())
    d = rng.uniform(-1, 1, P.ndof)
    v = P.lu_apply(lu, piv, d)
    np.savez_compressed(os.path.join(HERE, name), dim=dim, k=k, n=n, K=K, x=x, y=y, yt=yt,
                        d=d, v=v, **{f"opt_{a}": b for a, b in kw.items()})


def mfl_case():
    # matrix_free_linear.cc problem: 2D Q1 16x16 SIPG alpha=3, BiCGStab, 1e-12
    P = O.Problem(2, 1, (16, 16), alpha=3.0)
    vp = P.volume_points()
    c = (0.5 - vp[..., 0]) ** 2 + (0.5 - vp[..., 1]) ** 2
    bp = P.boundary_points()
    cb = (0.5 - bp[:, 0]) ** 2 + (0.5 - bp[:, 1]) ** 2
    f, g = 4 * (1 - c) * np.exp(-c), np.exp(-cb)
    P.set(fq=f, gq=g)
    u, res, st = P.solve(solver="bicgstab", op=0, reduction=1e-12)
    r = P.residual(np.zeros(P.ndof))
    np.savez_compressed(os.path.join(HERE, "mfl_q1_16.npz"), f=f, g=g, u=u, r0=r,
                        iterations=res.iterations)


def residual_case():
    rng = np.random.default_rng(11)
    P = O.Problem(3, 3, (3, 3, 3), alpha=3.0)
    K = np.exp(rng.standard_normal(P.ncell))
    fq = rng.standard_normal((P.ncell, P.nq_volume))
    g = rng.standard_normal(P.nbpts_total())
    P.set(K=K, fq=fq, gq=g)
    x = rng.uniform(-1, 1, P.ndof)
    r = P.residual(x)
    np.savez_compressed(os.path.join(HERE, "residual_q3_3.npz"), K=K, fq=fq, g=g, x=x, r=r)


if __name__ == "__main__":
    O.build()
    apply_case("apply_q2_4.npz", 3, 2, 4, seed=101)
    apply_case("apply_q1_2d_8.npz", 2, 1, 8, seed=102)
    apply_case("apply_q4_2_nipg.npz", 3, 4, 2, seed=103, method=O.NIPG)
    mfl_case()
    residual_case()
    print("fixtures written to", HERE)
