"""ctypes binding of the CPU oracle (oracle/pdg_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker.  The product library
never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpdg_oracle.so")

BC_DIRICHLET, BC_NEUMANN, BC_OUTFLOW, BC_NONE = 1, -1, -2, -3
NIPG, SIPG, IIPG = 0, 1, 2
WEIGHTS_ON, WEIGHTS_OFF = 0, 1
LAGRANGE, LEGENDRE, LOBATTO = 0, 1, 2     # QkDGBasisPolynomial

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Problem(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("k", C.c_int), ("nc", C.c_int * 3),
        ("L", C.c_double * 3), ("method", C.c_int), ("weights", C.c_int),
        ("alpha", C.c_double), ("bctype", C.c_int * 6),
        ("K", _dp), ("c", _dp), ("nmodes", C.c_int), ("modes", _dp),
        ("fq", _dp), ("fc", _dp), ("gq", _dp), ("jq", _dp), ("oq", _dp),
        ("nl_deg", C.c_int), ("nl_coef", C.c_double * 5), ("xlin", _dp),
        ("basis", C.c_int),
        ("Acell", _dp), ("Aq_vol", _dp), ("Aq_face", _dp), ("cq", _dp),
        ("bq_vol", _dp), ("bq_face", _dp),
    ]


class NewtonOpts(C.Structure):
    _fields_ = [
        ("reduction", C.c_double), ("absolute_limit", C.c_double),
        ("max_iterations", C.c_int), ("force_iteration", C.c_int),
        ("min_linear_reduction", C.c_double), ("fixed_linear_reduction", C.c_int),
        ("line_search", C.c_int), ("line_search_max_iterations", C.c_int),
        ("line_search_damping", C.c_double), ("line_search_accept_best", C.c_int),
        ("linear_maxit", C.c_int),
    ]


class NewtonResult(C.Structure):
    _fields_ = [
        ("converged", C.c_int), ("iterations", C.c_int),
        ("first_defect", C.c_double), ("defect", C.c_double),
        ("reduction", C.c_double), ("conv_rate", C.c_double),
        ("linear_iterations", C.c_int), ("status", C.c_int),
    ]


def newton_opts(**kw):
    """NewtonMethod defaults (solver/newton.hh:654-669, terminate.hh:74-75,
    linesearch.hh:206-208)."""
    o = NewtonOpts(1e-8, 1e-12, 40, 0, 1e-3, 0, 1, 10, 0.5, 0, 5000)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Result(C.Structure):
    _fields_ = [
        ("converged", C.c_int), ("iterations", C.c_int),
        ("reduction", C.c_double), ("conv_rate", C.c_double),
        ("first_defect", C.c_double), ("defect", C.c_double),
        ("status", C.c_int),
    ]


class PrecConfig(C.Structure):
    """Block preconditioner: kind 0 none, 1/2 LU block Jacobi, 3 iterative
    block Jacobi; + 16 for one block-SOR sweep."""
    _fields_ = [
        ("kind", C.c_int), ("omega", C.c_double), ("block_reduction", C.c_double),
        ("block_maxit", C.c_int), ("block_precondition", C.c_int),
        ("block_weight", C.c_double),
    ]


def prec_config(kind, omega=1.0, block_reduction=1e-5, block_maxit=100, block_precondition=1,
                block_weight=1.0):
    return PrecConfig(kind, omega, block_reduction, block_maxit, block_precondition,
                      block_weight)


def build():
    """Compile the oracle with its Makefile (plain gcc)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(_Problem)
        sigs = {
            "pdgo_ncell": (C.c_long, [P]),
            "pdgo_nbasis": (C.c_int, [P]),
            "pdgo_ndof": (C.c_long, [P]),
            "pdgo_nbpts_side": (C.c_long, [P, C.c_int]),
            "pdgo_bpts_offset": (C.c_long, [P, C.c_int]),
            "pdgo_nbpts_total": (C.c_long, [P]),
            "pdgo_gauss_legendre": (C.c_int, [C.c_int, _dp, _dp]),
            "pdgo_lagrange": (C.c_double, [C.c_int, C.c_int, C.c_double]),
            "pdgo_dlagrange": (C.c_double, [C.c_int, C.c_int, C.c_double]),
            "pdgo_basis1d": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_double]),
            "pdgo_dbasis1d": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_double]),
            "pdgo_gauss_lobatto": (C.c_int, [C.c_int, _dp, _dp]),
            "pdgo_volume_points": (C.c_int, [P, _dp]),
            "pdgo_boundary_points": (C.c_int, [P, _dp]),
            "pdgo_jacobian_apply": (C.c_int, [P, _dp, _dp]),
            "pdgo_residual": (C.c_int, [P, _dp, _dp]),
            "pdgo_jacobian_apply_range": (C.c_int, [P, _dp, _dp, C.c_long, C.c_long]),
            "pdgo_jacobian_apply_transpose": (C.c_int, [P, _dp, _dp]),
            "pdgo_jacobian_apply_transpose_range": (C.c_int, [P, _dp, _dp, C.c_long, C.c_long]),
            "pdgo_nface_lattice": (C.c_long, [P]),
            "pdgo_face_lattice_points": (C.c_int, [P, _dp]),
            "pdgo_cell_face_points": (C.c_int, [P, _dp]),
            "pdgo_assemble_jacobian": (C.c_int, [P, _dp]),
            "pdgo_blocks_apply": (C.c_int, [P, _dp, _dp, _dp]),
            "pdgo_blocks_apply_transpose": (C.c_int, [P, _dp, _dp, _dp]),
            "pdgo_block_diagonal": (C.c_int, [P, _dp]),
            "pdgo_lu_factor": (C.c_int, [C.c_int, C.c_long, _dp, _ip]),
            "pdgo_lu_apply": (None, [C.c_int, C.c_long, _dp, _ip, _dp, _dp]),
            "pdgo_cg": (C.c_int, [P, C.c_int, _dp, _dp, _ip, _dp, _dp, C.c_double, C.c_int, C.POINTER(Result)]),
            "pdgo_bicgstab": (C.c_int, [P, C.c_int, _dp, _dp, _ip, _dp, _dp, C.c_double, C.c_int, C.POINTER(Result)]),
            "pdgo_solve_linear_problem": (C.c_int, [P, C.c_int, C.c_int, _dp, C.c_double, C.c_double, C.c_int, C.POINTER(Result)]),
            "pdgo_eval_points": (C.c_int, [P, _dp, C.c_int, _dp, _dp, _dp]),
            "pdgo_grad_logK": (C.c_int, [P, _dp, _dp, _dp]),
            "pdgo_grad_fc": (C.c_int, [P, _dp, _dp]),
            "pdgo_block_bicgstab": (C.c_int, [C.c_int, _dp, C.c_int, _dp, _dp, C.c_double,
                                              C.c_int, C.c_int, C.c_double, _ip]),
            "pdgo_prec_apply_cfg": (C.c_int, [P, C.POINTER(PrecConfig), _dp, _dp, _ip, _dp,
                                              C.c_int, _dp, _dp, _ip]),
            "pdgo_mass_apply": (C.c_int, [P, _dp, _dp]),
            "pdgo_onestep": (C.c_int, [P, C.c_int, _dp, _dp, C.c_double, C.c_int,
                                       C.POINTER(PrecConfig), C.c_double, C.c_int, _dp, _dp,
                                       _ip]),
            "pdgo_newton": (C.c_int, [P, C.c_int, C.POINTER(PrecConfig), C.POINTER(NewtonOpts),
                                      _dp, C.POINTER(NewtonResult)]),
            "pdgo_solve_linear_problem_prec": (C.c_int, [P, C.c_int, C.c_int,
                                                         C.POINTER(PrecConfig), _dp, C.c_double,
                                                         C.c_double, C.c_int,
                                                         C.POINTER(Result)]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def gauss_legendre(m):
    x = np.zeros(m)
    w = np.zeros(m)
    lib().pdgo_gauss_legendre(m, _ptr(x), _ptr(w))
    return x, w


def gauss_lobatto(m):
    x = np.zeros(m)
    w = np.zeros(m)
    lib().pdgo_gauss_lobatto(m, _ptr(x), _ptr(w))
    return x, w


def basis1d(basis, k, i, x, derivative=False):
    f = lib().pdgo_dbasis1d if derivative else lib().pdgo_basis1d
    return f(basis, k, i, x)


class Problem:
    """SIPG/NIPG/IIPG ConvectionDiffusionDG problem on a structured grid.

    Arrays given here are kept alive by this object; all are float64.
    """

    def __init__(self, dim, k, nc, L=None, method=SIPG, weights=WEIGHTS_ON,
                 alpha=1.0, bctype=None, K=None, c=None, modes=None,
                 fq=None, fc=None, gq=None, jq=None, oq=None, basis=LAGRANGE):
        self.dim, self.k, self.basis = dim, k, basis
        self.nc = tuple(nc) + (1,) * (3 - len(nc))
        self.L = tuple(L) if L is not None else (1.0,) * dim
        self.L = self.L + (1.0,) * (3 - len(self.L))
        self.method, self.weights, self.alpha = method, weights, float(alpha)
        self.bctype = list(bctype) if bctype is not None else [BC_DIRICHLET] * 6
        self._arrays = {}
        self.s = _Problem()
        s = self.s
        s.dim, s.k = dim, k
        for j in range(3):
            s.nc[j] = self.nc[j]
            s.L[j] = self.L[j]
        s.method, s.weights, s.alpha = method, weights, self.alpha
        s.basis = basis
        for j in range(6):
            s.bctype[j] = self.bctype[j] if j < len(self.bctype) else BC_DIRICHLET
        self.set(K=K, c=c, fq=fq, fc=fc, gq=gq, jq=jq, oq=oq)
        self.set_modes(modes)

    def set(self, **arrays):
        for name, a in arrays.items():
            if a is None:
                self._arrays.pop(name, None)
                setattr(self.s, name, None)
                continue
            a = np.ascontiguousarray(a, dtype=np.float64).ravel()
            self._arrays[name] = a
            setattr(self.s, name, _ptr(a))

    def set_modes(self, modes):
        if modes is None or len(modes) == 0:
            self.s.nmodes = 0
            self.s.modes = None
            self._arrays.pop("modes", None)
            return
        m = np.ascontiguousarray(modes, dtype=np.float64).reshape(-1, 7)
        self._arrays["modes"] = m
        self.s.nmodes = m.shape[0]
        self.s.modes = _ptr(m)

    @property
    def ref(self):
        return C.byref(self.s)

    @property
    def ncell(self):
        return lib().pdgo_ncell(self.ref)

    @property
    def nb(self):
        return lib().pdgo_nbasis(self.ref)

    @property
    def ndof(self):
        return lib().pdgo_ndof(self.ref)

    @property
    def nq_volume(self):
        return (self.k + 1) ** self.dim

    def nbpts_total(self):
        return lib().pdgo_nbpts_total(self.ref)

    def volume_points(self):
        out = np.zeros((self.ncell, self.nq_volume, self.dim))
        _check(lib().pdgo_volume_points(self.ref, _ptr(out)))
        return out

    def boundary_points(self):
        out = np.zeros((self.nbpts_total(), self.dim))
        _check(lib().pdgo_boundary_points(self.ref, _ptr(out)))
        return out

    def jacobian_apply(self, z, y=None):
        z = np.ascontiguousarray(z, dtype=np.float64)
        y = np.zeros(self.ndof) if y is None else y
        _check(lib().pdgo_jacobian_apply(self.ref, _ptr(z), _ptr(y)))
        return y

    def jacobian_apply_transpose(self, z, y=None):
        """y += J^T z, matrix-free (the transposed local forms)."""
        z = np.ascontiguousarray(z, dtype=np.float64)
        y = np.zeros(self.ndof) if y is None else y
        _check(lib().pdgo_jacobian_apply_transpose(self.ref, _ptr(z), _ptr(y)))
        return y

    def jacobian_apply_transpose_range(self, z, y, e_begin, e_end):
        _check(lib().pdgo_jacobian_apply_transpose_range(self.ref, _ptr(z), _ptr(y), e_begin,
                                                         e_end))
        return y

    @property
    def nq_face(self):
        return (self.k + 1) ** (self.dim - 1)

    def nface_lattice(self):
        return lib().pdgo_nface_lattice(self.ref)

    def face_lattice_points(self):
        """[faces][nq_face][dim]: every face once (x-normal faces, then y, z)."""
        out = np.zeros((self.nface_lattice(), self.nq_face, self.dim))
        _check(lib().pdgo_face_lattice_points(self.ref, _ptr(out)))
        return out

    def cell_face_points(self):
        """[ncell][2 dim][nq_face][dim]: each cell's own points of its faces."""
        out = np.zeros((self.ncell, 2 * self.dim, self.nq_face, self.dim))
        _check(lib().pdgo_cell_face_points(self.ref, _ptr(out)))
        return out

    def jacobian_apply_range(self, z, y, e_begin, e_end):
        _check(lib().pdgo_jacobian_apply_range(self.ref, _ptr(z), _ptr(y), e_begin, e_end))
        return y

    def residual(self, x, r=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        r = np.zeros(self.ndof) if r is None else r
        _check(lib().pdgo_residual(self.ref, _ptr(x), _ptr(r)))
        return r

    def assemble_jacobian(self):
        nb = self.nb
        out = np.zeros((self.ncell, 2 * self.dim + 1, nb, nb))
        _check(lib().pdgo_assemble_jacobian(self.ref, _ptr(out)))
        return out

    def blocks_apply(self, blocks, x, transpose=False):
        y = np.zeros(self.ndof)
        fn = lib().pdgo_blocks_apply_transpose if transpose else lib().pdgo_blocks_apply
        _check(fn(self.ref, _ptr(blocks), _ptr(np.ascontiguousarray(x)), _ptr(y)))
        return y

    def block_diagonal(self):
        nb = self.nb
        out = np.zeros((self.ncell, nb, nb))
        _check(lib().pdgo_block_diagonal(self.ref, _ptr(out)))
        return out

    def lu(self, diag):
        a = np.ascontiguousarray(diag.copy())
        piv = np.zeros(a.shape[:-1], dtype=np.int32)
        _check(lib().pdgo_lu_factor(self.nb, self.ncell, _ptr(a), piv.ctypes.data_as(_ip)))
        return a, piv

    def lu_apply(self, lu, piv, d):
        v = np.zeros(self.ndof)
        lib().pdgo_lu_apply(self.nb, self.ncell, _ptr(lu), piv.ctypes.data_as(_ip),
                            _ptr(np.ascontiguousarray(d)), _ptr(v))
        return v

    def krylov(self, solver, x, b, reduction, maxit=5000, op=0, blocks=None,
               lu=None, piv=None):
        res = Result()
        fn = lib().pdgo_cg if solver == "cg" else lib().pdgo_bicgstab
        st = fn(self.ref, op, _ptr(blocks), _ptr(lu),
                None if piv is None else piv.ctypes.data_as(_ip),
                _ptr(x), _ptr(b), reduction, maxit, C.byref(res))
        return st, res

    def solve(self, x=None, solver="cg", op=0, reduction=1e-12, min_defect=1e-99,
              maxit=5000):
        x = np.zeros(self.ndof) if x is None else x
        res = Result()
        st = lib().pdgo_solve_linear_problem(self.ref, 0 if solver == "cg" else 1, op,
                                             _ptr(x), reduction, min_defect, maxit,
                                             C.byref(res))
        return x, res, st

    def mass_apply(self, x):
        y = np.zeros(self.ndof)
        _check(lib().pdgo_mass_apply(self.ref, _ptr(np.ascontiguousarray(x)), _ptr(y)))
        return y

    def onestep(self, A, B, dt, xold, pc, solver="cg", reduction=1e-12, maxit=5000):
        """One step of the one-step method with tables A, B [s][s+1]."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        xnew = np.zeros(self.ndof)
        its = np.zeros(1, dtype=np.int32)
        _check(lib().pdgo_onestep(self.ref, A.shape[0], _ptr(A), _ptr(B), dt,
                                  0 if solver == "cg" else 1, C.byref(pc), reduction, maxit,
                                  _ptr(np.ascontiguousarray(xold, dtype=np.float64)), _ptr(xnew),
                                  its.ctypes.data_as(_ip)))
        return xnew, int(its[0])

    def set_nonlinearity(self, coef):
        """q(u) = sum_m coef[m] u^m (coef None removes it)."""
        if coef is None:
            self.s.nl_deg = 0
            return
        self.s.nl_deg = len(coef) - 1
        for m in range(5):
            self.s.nl_coef[m] = coef[m] if m < len(coef) else 0.0

    def set_linearization_point(self, x):
        self._xlin = None if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        self.s.xlin = _ptr(self._xlin)

    def newton(self, pc, x=None, solver="bicgstab", **kw):
        x = np.zeros(self.ndof) if x is None else x
        res = NewtonResult()
        st = lib().pdgo_newton(self.ref, 0 if solver == "cg" else 1, C.byref(pc),
                               C.byref(newton_opts(**kw)), _ptr(x), C.byref(res))
        return x, res, st

    def prec_apply_cfg(self, pc, d, transpose=False):
        """v = M^{-1} d for a PrecConfig; returns (v, per-cell block iterations)."""
        nb, nc = self.nb, self.ncell
        diag = self.block_diagonal()
        lu = piv = None
        if pc.kind & 15 in (1, 2):
            src = np.ascontiguousarray(np.swapaxes(diag, 1, 2)) if transpose else diag
            lu, piv = self.lu(src)
        ab = self.assemble_jacobian() if pc.kind & 16 else None
        v = np.zeros(self.ndof)
        its = np.zeros(nc, dtype=np.int32)
        _check(lib().pdgo_prec_apply_cfg(self.ref, C.byref(pc), _ptr(diag), _ptr(lu),
                                         None if piv is None else piv.ctypes.data_as(_ip),
                                         _ptr(ab), int(transpose),
                                         _ptr(np.ascontiguousarray(d)), _ptr(v),
                                         its.ctypes.data_as(_ip)))
        return v, its

    def solve_prec(self, pc, x=None, solver="cg", op=0, reduction=1e-12, min_defect=1e-99,
                   maxit=5000):
        x = np.zeros(self.ndof) if x is None else x
        res = Result()
        st = lib().pdgo_solve_linear_problem_prec(self.ref, 0 if solver == "cg" else 1, op,
                                                  C.byref(pc), _ptr(x), reduction, min_defect,
                                                  maxit, C.byref(res))
        return x, res, st

    def eval_points(self, u, m):
        mq = m ** self.dim
        xyz = np.zeros((self.ncell, mq, self.dim))
        w = np.zeros((self.ncell, mq))
        val = np.zeros((self.ncell, mq))
        _check(lib().pdgo_eval_points(self.ref, _ptr(np.ascontiguousarray(u)), m,
                                      _ptr(xyz), _ptr(w), _ptr(val)))
        return xyz, w, val

    def grad_logK(self, u, lam):
        g = np.zeros(self.ncell)
        _check(lib().pdgo_grad_logK(self.ref, _ptr(np.ascontiguousarray(u)),
                                    _ptr(np.ascontiguousarray(lam)), _ptr(g)))
        return g

    def grad_fc(self, lam):
        g = np.zeros(self.ncell)
        _check(lib().pdgo_grad_fc(self.ref, _ptr(np.ascontiguousarray(lam)), _ptr(g)))
        return g


class OracleError(RuntimeError):
    pass


def _check(st):
    if st != 0:
        raise OracleError(f"oracle status {st}")


# --------------------------------------------------------------------------
# full-size applies over all host cores (test and baseline infrastructure)
# --------------------------------------------------------------------------
_POOL_STATE = {}


def _pool_init(spec, shm_x, ndof):
    from multiprocessing import shared_memory
    sx = shared_memory.SharedMemory(name=shm_x)
    _POOL_STATE.update(P=Problem(**spec), sx=sx,
                       x=np.ndarray((ndof,), dtype=np.float64, buffer=sx.buf))


def _pool_apply(args):
    from multiprocessing import shared_memory
    b, e, shm_y, ndof, transpose = args
    sy = shared_memory.SharedMemory(name=shm_y)
    y = np.ndarray((ndof,), dtype=np.float64, buffer=sy.buf)
    y[:] = 0.0
    P = _POOL_STATE["P"]
    if transpose:
        P.jacobian_apply_transpose_range(_POOL_STATE["x"], y, b, e)
    else:
        P.jacobian_apply_range(_POOL_STATE["x"], y, b, e)
    del y
    sy.close()
    return 0


def parallel_apply(spec, x, transpose=False, workers=None):
    """J x (or J^T x) of Problem(**spec), the cells split over `workers`
    spawned processes (default: all host cores, at most 32); the partial
    results of the cell ranges are summed.  Spawned, so it is safe after
    CUDA was initialised in the calling process."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from multiprocessing import shared_memory
    build()
    x = np.ascontiguousarray(x, dtype=np.float64)
    ndof = x.size
    probe = Problem(**spec)
    ncell = probe.ncell
    assert probe.ndof == ndof
    workers = workers or min(32, os.cpu_count() or 1)
    workers = max(1, min(workers, ncell))
    sx = shared_memory.SharedMemory(create=True, size=ndof * 8)
    sys_ = [shared_memory.SharedMemory(create=True, size=ndof * 8) for _ in range(workers)]
    try:
        np.ndarray((ndof,), dtype=np.float64, buffer=sx.buf)[:] = x
        bounds = np.linspace(0, ncell, workers + 1).astype(int)
        jobs = [(int(bounds[i]), int(bounds[i + 1]), sys_[i].name, ndof, bool(transpose))
                for i in range(workers)]
        # a process pool executor raises BrokenProcessPool when a worker
        # dies, where multiprocessing.Pool would wait for it forever
        with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn"),
                                    initializer=_pool_init,
                                    initargs=(spec, sx.name, ndof)) as pool:
            list(pool.map(_pool_apply, jobs))
        y = np.zeros(ndof)
        for s in sys_:
            y += np.ndarray((ndof,), dtype=np.float64, buffer=s.buf)
        return y
    finally:
        sx.close()
        sx.unlink()
        for s in sys_:
            s.close()
            s.unlink()
