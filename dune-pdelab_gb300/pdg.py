"""Python binding of libpdg.so (include/pdg.h) over ctypes.

The classes mirror the reference's interfaces for this path so that driver
code keeps its shape:

* ``GridOperator``      -- GridOperator::residual / jacobian_apply
  (dune/pdelab/gridoperator/gridoperator.hh:176-205) on one GPU context;
* ``OnTheFlyOperator``  -- ISTL LinearOperator apply / applyscaleadd
  (dune/pdelab/backend/istl/seqistlsolverbackend.hh:45-100);
* ``GridOperatorPreconditioner`` -- pre / apply
  (dune/pdelab/backend/istl/matrixfree/gridoperatorpreconditioner.hh:45-84);
* ``ISTLBackend_SEQ_MatrixFree_Base`` -- apply(z, r, reduction), norm, result
  (dune/pdelab/backend/istl/matrixfree/backends.hh:62-143);
* ``StationaryLinearProblemSolver`` -- apply / result
  (dune/pdelab/stationary/linearproblem.hh:59-338).

Vectors are numpy float64 arrays (host) or torch tensors on the GPU (device
pointers are passed straight through).  Unless a stream is bound with
``GridOperator.set_stream``, every call that can touch device buffers is
ordered after the work already queued on torch's current stream, and torch's
current stream waits for the call's work (events, no host synchronisation),
so tensors made or read by torch around a call need no explicit
``torch.cuda.synchronize()``.  Every failure raises ``PDGError``
with the library's message, as the reference raises Dune exceptions.
There is no CPU fallback: without the CUDA library nothing here works.
"""
from __future__ import annotations

import ctypes as C
import functools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpdg.so")

PDG_OK, PDG_EINVAL, PDG_ECUDA, PDG_ENOTCONVERGED, PDG_EBREAKDOWN = 0, 1, 2, 3, 4
PDG_ESTATE, PDG_EUNSUPPORTED, PDG_EOUTFLOW, PDG_ENONFINITE, PDG_ETIMEOUT = 5, 6, 7, 8, 9
PDG_ELINESEARCH = 10
(ONESTEP_THETA, IMPLICIT_EULER, EXPLICIT_EULER, ALEXANDER2, ALEXANDER3, FRACTIONAL_STEP, HEUN,
 SHU3, RK4) = range(9)
NIPG, SIPG, IIPG = 0, 1, 2
WEIGHTS_ON, WEIGHTS_OFF = 0, 1
BC_DIRICHLET, BC_NEUMANN, BC_OUTFLOW, BC_NONE = 1, -1, -2, -3
CG, BICGSTAB, GMRES = 0, 1, 2
PREC_NONE, PREC_BJ_FDM, PREC_BJ_DENSE, PREC_BJ_ITERATIVE = 0, 1, 2, 3
PREC_SOR = 16          # OR-ed with a block kind: one block-SOR sweep
F64, F32 = 0, 1
F64_NATIVE, F64_FLOAT_PAIR = 0, 1          # arithmetic of the FP64 operator applies
LAGRANGE, LEGENDRE, LOBATTO = 0, 1, 2     # QkDGBasisPolynomial


class PDGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"pdg status {status}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("cells", C.c_int * 3),
                ("extent", C.c_double * 3), ("method", C.c_int), ("weights", C.c_int),
                ("alpha", C.c_double), ("bctype", C.c_int * 6), ("device", C.c_int),
                ("basis", C.c_int)]


class SolverOptions(C.Structure):
    _fields_ = [("method", C.c_int), ("preconditioner", C.c_int),
                ("reduction", C.c_double), ("min_defect", C.c_double), ("maxit", C.c_int),
                ("mixed", C.c_int), ("inner_reduction", C.c_double),
                ("inner_maxit", C.c_int), ("max_outer", C.c_int), ("verbose", C.c_int),
                ("inner_breakdown", C.c_double), ("inner_method", C.c_int),
                ("restart", C.c_int), ("inner_replace", C.c_int), ("inner_vectors", C.c_int),
                ("assembled", C.c_int)]


class PrecOptions(C.Structure):
    """BlockSORPreconditionerLocalOperator omega + BlockSolverOptions."""
    _fields_ = [("omega", C.c_double), ("block_reduction", C.c_double),
                ("block_maxit", C.c_int), ("block_precondition", C.c_int),
                ("block_weight", C.c_double), ("dense_fp16", C.c_int)]


class NewtonOptions(C.Structure):
    """NewtonMethod parameters (solver/newton.hh), reference defaults."""
    _fields_ = [("reduction", C.c_double), ("absolute_limit", C.c_double),
                ("max_iterations", C.c_int), ("force_iteration", C.c_int),
                ("min_linear_reduction", C.c_double), ("fixed_linear_reduction", C.c_int),
                ("line_search", C.c_int), ("line_search_max_iterations", C.c_int),
                ("line_search_damping", C.c_double), ("line_search_accept_best", C.c_int),
                ("verbose", C.c_int)]


class NewtonResult(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int),
                ("first_defect", C.c_double), ("defect", C.c_double),
                ("reduction", C.c_double), ("conv_rate", C.c_double),
                ("linear_solver_iterations", C.c_int), ("elapsed", C.c_double),
                ("status", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class OneStepResult(C.Structure):
    _fields_ = [("stages", C.c_int), ("linear_solver_iterations", C.c_int),
                ("elapsed", C.c_double), ("status", C.c_int)]


class SolverResult(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int), ("elapsed", C.c_double),
                ("reduction", C.c_double), ("conv_rate", C.c_double),
                ("first_defect", C.c_double), ("defect", C.c_double),
                ("outer_iterations", C.c_int), ("status", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# exported symbols and their signatures (every declaration of include/pdg.h)
_vp = C.c_void_p
_SIGS = {
    "pdg_create": (C.c_int, [C.POINTER(Config), C.POINTER(_vp)]),
    "pdg_destroy": (C.c_int, [_vp]),
    "pdg_last_error": (C.c_char_p, []),
    "pdg_default_solver_options": (None, [C.POINTER(SolverOptions)]),
    "pdg_set_stream": (C.c_int, [_vp, _vp]),
    "pdg_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "pdg_sizes": (C.c_int, [_vp, C.POINTER(C.c_long), C.POINTER(C.c_int), C.POINTER(C.c_long),
                            C.POINTER(C.c_int), C.POINTER(C.c_long)]),
    "pdg_volume_points": (C.c_int, [_vp, _vp]),
    "pdg_boundary_points": (C.c_int, [_vp, _vp]),
    "pdg_set_permeability": (C.c_int, [_vp, _vp, C.c_int]),
    "pdg_set_reaction": (C.c_int, [_vp, _vp]),
    "pdg_set_velocity_modes": (C.c_int, [_vp, C.c_int, _vp]),
    "pdg_set_source": (C.c_int, [_vp, _vp, _vp]),
    "pdg_set_boundary_data": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pdg_residual": (C.c_int, [_vp, _vp, _vp]),
    "pdg_jacobian_apply": (C.c_int, [_vp, _vp, _vp]),
    "pdg_jacobian_apply_f32": (C.c_int, [_vp, _vp, _vp]),
    "pdg_jacobian_apply_transpose_f32": (C.c_int, [_vp, _vp, _vp]),
    "pdg_apply_f32": (C.c_int, [_vp, _vp, _vp]),
    "pdg_jacobian_apply_transpose": (C.c_int, [_vp, _vp, _vp]),
    "pdg_apply": (C.c_int, [_vp, _vp, _vp]),
    "pdg_applyscaleadd": (C.c_int, [_vp, C.c_double, _vp, _vp]),
    "pdg_prec_setup": (C.c_int, [_vp, C.c_int, C.c_int]),
    "pdg_prec_apply": (C.c_int, [_vp, _vp, _vp]),
    "pdg_prec_apply_f32": (C.c_int, [_vp, _vp, _vp]),
    "pdg_prec_apply_transpose": (C.c_int, [_vp, _vp, _vp]),
    "pdg_norm": (C.c_int, [_vp, _vp, C.POINTER(C.c_double)]),
    "pdg_dot": (C.c_int, [_vp, _vp, _vp, C.POINTER(C.c_double)]),
    "pdg_dot_noalloc": (C.c_int, [C.c_long, _vp, _vp, _vp, _vp]),
    "pdg_krylov_solve": (C.c_int, [_vp, C.POINTER(SolverOptions), _vp, _vp,
                                   C.POINTER(SolverResult)]),
    "pdg_solve_linear_problem": (C.c_int, [_vp, C.POINTER(SolverOptions), _vp,
                                           C.POINTER(SolverResult)]),
    "pdg_adjoint_solve": (C.c_int, [_vp, C.POINTER(SolverOptions), _vp, _vp,
                                    C.POINTER(SolverResult)]),
    "pdg_grad_logK": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pdg_grad_source": (C.c_int, [_vp, _vp, _vp]),
    "pdg_default_prec_options": (None, [C.POINTER(PrecOptions)]),
    "pdg_set_prec_options": (C.c_int, [_vp, C.POINTER(PrecOptions)]),
    "pdg_prec_block_iterations": (C.c_int, [_vp, C.c_int, _vp]),
    "pdg_set_nonlinearity": (C.c_int, [_vp, C.c_int, _vp]),
    "pdg_set_linearization_point": (C.c_int, [_vp, _vp]),
    "pdg_jacobian_apply_nonlinear": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pdg_default_newton_options": (None, [C.POINTER(NewtonOptions)]),
    "pdg_newton_solve": (C.c_int, [_vp, C.POINTER(NewtonOptions), C.POINTER(SolverOptions), _vp,
                                   C.POINTER(NewtonResult)]),
    "pdg_mass_apply": (C.c_int, [_vp, _vp, _vp]),
    "pdg_onestep_table": (C.c_int, [C.c_int, C.c_double, C.POINTER(C.c_int), _vp, _vp, _vp]),
    "pdg_onestep_apply": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, C.c_double,
                                    C.POINTER(SolverOptions), _vp, _vp,
                                    C.POINTER(OneStepResult)]),
    "pdg_jacobian_assemble": (C.c_int, [_vp]),
    "pdg_jacobian_pattern": (C.c_int, [_vp, C.POINTER(C.c_long)]),
    "pdg_jacobian_export": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pdg_matrix_apply": (C.c_int, [_vp, _vp, _vp]),
    "pdg_set_f64_arithmetic": (C.c_int, [_vp, C.c_int]),
    "pdg_set_permeability_tensor": (C.c_int, [_vp, _vp]),
    "pdg_set_permeability_points": (C.c_int, [_vp, _vp, _vp]),
    "pdg_set_reaction_points": (C.c_int, [_vp, _vp]),
    "pdg_set_velocity_points": (C.c_int, [_vp, _vp, _vp]),
    "pdg_face_lattice_size": (C.c_int, [_vp, C.POINTER(C.c_long)]),
    "pdg_face_lattice_points": (C.c_int, [_vp, _vp]),
    "pdg_cell_face_points": (C.c_int, [_vp, _vp]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libpdg.so; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise PDGError(PDG_EUNSUPPORTED,
                           f"{path} missing: build it with __graft_entry__.build()")
        lib = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(st, allow=()):
    if st != PDG_OK and st not in allow:
        msg = load().pdg_last_error()
        raise PDGError(st, msg.decode() if msg else "")
    return st


def _torch_streams(go):
    """(torch's current stream, the context's stream as a torch stream) when
    torch has initialised CUDA and no stream was bound explicitly, else None."""
    torch = sys.modules.get("torch")
    if torch is None or go._explicit_stream or not go._h or not torch.cuda.is_initialized():
        return None
    p = _vp()
    _check(load().pdg_get_stream(go._h, C.byref(p)))
    dev = torch.device("cuda", go.cfg.device)
    if go._lib_stream is None or go._lib_stream[0] != p.value:
        go._lib_stream = (p.value, torch.cuda.ExternalStream(p.value, device=dev))
    return torch.cuda.current_stream(dev), go._lib_stream[1]


def _stream_ordered(method):
    """Order a call's work between torch's current stream and the context's."""
    @functools.wraps(method)
    def wrapper(self, *args, **kw):
        s = _torch_streams(self if isinstance(self, GridOperator) else self.go)
        if s is None:
            return method(self, *args, **kw)
        cur, lib = s
        lib.wait_stream(cur)
        try:
            return method(self, *args, **kw)
        finally:
            cur.wait_stream(lib)
    return wrapper


def _ptr(v, dtype=np.float64):
    """Raw address of a numpy array or torch tensor (contiguous, right dtype)."""
    if v is None:
        return None
    if isinstance(v, np.ndarray):
        if v.dtype != dtype or not v.flags["C_CONTIGUOUS"]:
            raise TypeError(f"expected contiguous {dtype} array")
        return v.ctypes.data
    if hasattr(v, "data_ptr"):
        if not v.is_contiguous():
            raise TypeError("expected a contiguous tensor")
        return v.data_ptr()
    raise TypeError(f"unsupported vector type {type(v)}")


def fourier_velocity_modes(seed, nmodes=8, bmax=10.0, kmax=2):
    """Divergence-free velocity b = curl A of a seeded Fourier vector potential
    A(x) = sum_m a_m cos(2 pi k_m.x + phi_m):
    b(x) = sum_m c_m sin(2 pi k_m.x + phi_m) with c_m = -2 pi k_m x a_m
    (so k_m . c_m = 0 and div b = 0), scaled so that sum_m |c_m| = bmax,
    which bounds |b| <= bmax everywhere.  Rows: kx ky kz phase cx cy cz."""
    rng = np.random.default_rng(seed)
    modes = np.zeros((nmodes, 7))
    for m in range(nmodes):
        k = np.zeros(3)
        while not k.any():
            k = rng.integers(-kmax, kmax + 1, 3).astype(float)
        a = rng.standard_normal(3)
        modes[m, :3] = k
        modes[m, 3] = rng.uniform(0, 2 * np.pi)
        modes[m, 4:] = -2 * np.pi * np.cross(k, a)
    s = np.linalg.norm(modes[:, 4:], axis=1).sum()
    modes[:, 4:] *= bmax / s
    return modes


def newton_options(**kw):
    o = NewtonOptions()
    load().pdg_default_newton_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def prec_options(**kw):
    o = PrecOptions()
    load().pdg_default_prec_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def default_options(**kw):
    o = SolverOptions()
    load().pdg_default_solver_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class GridOperator:
    """One DG problem on the GPU: YaspGrid + QkDG space + ConvectionDiffusionDG
    + GridOperator of the reference, as a single context."""

    def __init__(self, dim, degree, cells, extent=None, method=SIPG, weights=WEIGHTS_ON,
                 alpha=1.0, bctype=None, device=0, basis=LAGRANGE):
        cfg = Config()
        cfg.dim, cfg.degree = dim, degree
        cells = list(cells) + [1] * (3 - len(cells))
        extent = list(extent) if extent is not None else [1.0] * dim
        extent = extent + [1.0] * (3 - len(extent))
        for j in range(3):
            cfg.cells[j] = cells[j]
            cfg.extent[j] = extent[j]
        cfg.method, cfg.weights, cfg.alpha = method, weights, alpha
        bct = list(bctype) if bctype is not None else [BC_DIRICHLET] * 6
        for j in range(6):
            cfg.bctype[j] = bct[j] if j < len(bct) else BC_DIRICHLET
        cfg.device = device
        cfg.basis = basis
        self.cfg = cfg
        self.dim, self.degree, self.basis = dim, degree, basis
        self._explicit_stream = False
        self._lib_stream = None
        self._h = _vp()
        _check(load().pdg_create(C.byref(cfg), C.byref(self._h)))
        nc, nb, nd, nq, nbp = C.c_long(), C.c_int(), C.c_long(), C.c_int(), C.c_long()
        _check(load().pdg_sizes(self._h, C.byref(nc), C.byref(nb), C.byref(nd),
                                C.byref(nq), C.byref(nbp)))
        self.ncell, self.nbasis, self.ndof = nc.value, nb.value, nd.value
        self.nq_volume, self.nq_boundary = nq.value, nbp.value

    def close(self):
        if self._h:
            load().pdg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream):
        """Bind the context to a CUDA stream (a torch stream or a raw
        cudaStream_t address; None: the context's own stream again).  While a
        stream is bound, the caller orders its work against it."""
        ptr = getattr(stream, "cuda_stream", stream)
        _check(load().pdg_set_stream(self._h, _vp(ptr) if ptr else None))
        # torch's default stream (address 0) is followed through events instead
        self._explicit_stream = bool(ptr)

    # -- geometry ---------------------------------------------------------
    def volume_points(self):
        out = np.zeros((self.ncell, self.nq_volume, self.dim))
        _check(load().pdg_volume_points(self._h, out.ctypes.data))
        return out

    def boundary_points(self):
        out = np.zeros((self.nq_boundary, self.dim))
        _check(load().pdg_boundary_points(self._h, out.ctypes.data))
        return out

    @property
    def nq_face(self):
        return (self.degree + 1) ** (self.dim - 1)

    def face_lattice_size(self):
        n = C.c_long()
        _check(load().pdg_face_lattice_size(self._h, C.byref(n)))
        return n.value

    def face_lattice_points(self):
        """[faces][nq_face][dim]: every face once (x-normal faces, then y, z)."""
        out = np.zeros((self.face_lattice_size(), self.nq_face, self.dim))
        _check(load().pdg_face_lattice_points(self._h, out.ctypes.data))
        return out

    def cell_face_points(self):
        """[ncell][2 dim][nq_face][dim]: each cell's own points of its faces."""
        out = np.zeros((self.ncell, 2 * self.dim, self.nq_face, self.dim))
        _check(load().pdg_cell_face_points(self._h, out.ctypes.data))
        return out

    # -- parameters -------------------------------------------------------
    @_stream_ordered
    def set_permeability(self, K, is_log=False):
        K = np.ascontiguousarray(K, dtype=np.float64) if isinstance(K, (list, np.ndarray)) else K
        _check(load().pdg_set_permeability(self._h, _ptr(K), int(is_log)))

    def set_f64_arithmetic(self, mode):
        """F64_NATIVE or F64_FLOAT_PAIR (the 3D operator's FP64 applies on the
        FP32 pipe in float pairs)."""
        _check(load().pdg_set_f64_arithmetic(self._h, int(mode)))

    def set_permeability_tensor(self, A):
        """A(cell) as a dim x dim tensor per cell ([ncell][dim][dim]); None
        returns to A = K I."""
        A = None if A is None else np.ascontiguousarray(A, dtype=np.float64)
        _check(load().pdg_set_permeability_tensor(self._h, _ptr(A)))

    def set_permeability_points(self, Avol, Aface):
        """A per quadrature point: [ncell][nq_volume][dim][dim] and
        [ncell][2 dim][nq_face][dim][dim] (permeabilityIsConstantPerCell()
        false); both None return to A = K I."""
        Av = None if Avol is None else np.ascontiguousarray(Avol, dtype=np.float64)
        Af = None if Aface is None else np.ascontiguousarray(Aface, dtype=np.float64)
        _check(load().pdg_set_permeability_points(self._h, _ptr(Av), _ptr(Af)))

    def set_reaction_points(self, cq):
        """c per volume quadrature point [ncell][nq_volume], added to the per-cell c."""
        cq = None if cq is None else np.ascontiguousarray(cq, dtype=np.float64)
        _check(load().pdg_set_reaction_points(self._h, _ptr(cq)))

    def set_velocity_points(self, bvol, bface):
        """b at the volume points [ncell][nq_volume][3] and at the face-lattice
        points [faces][nq_face][3] (3D); both None remove the velocity."""
        bv = None if bvol is None else np.ascontiguousarray(bvol, dtype=np.float64)
        bf = None if bface is None else np.ascontiguousarray(bface, dtype=np.float64)
        _check(load().pdg_set_velocity_points(self._h, _ptr(bv), _ptr(bf)))

    def set_reaction(self, c):
        c = None if c is None else np.ascontiguousarray(c, dtype=np.float64)
        _check(load().pdg_set_reaction(self._h, _ptr(c)))

    def set_velocity_modes(self, modes):
        m = None if modes is None else np.ascontiguousarray(modes, dtype=np.float64).reshape(-1, 7)
        n = 0 if m is None else m.shape[0]
        _check(load().pdg_set_velocity_modes(self._h, n, _ptr(m)))

    def set_source(self, fq=None, fc=None):
        fq = None if fq is None else np.ascontiguousarray(fq, dtype=np.float64)
        fc = None if fc is None else np.ascontiguousarray(fc, dtype=np.float64)
        _check(load().pdg_set_source(self._h, _ptr(fq), _ptr(fc)))

    def set_boundary_data(self, g=None, j=None, o=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (g, j, o)]
        _check(load().pdg_set_boundary_data(self._h, *[_ptr(a) for a in arrs]))

    # -- GridOperator -----------------------------------------------------
    @_stream_ordered
    def residual(self, x, r):
        """r += R(x)"""
        _check(load().pdg_residual(self._h, _ptr(x), _ptr(r)))
        return r

    @_stream_ordered
    def jacobian_apply(self, z, y):
        """y += J z"""
        _check(load().pdg_jacobian_apply(self._h, _ptr(z), _ptr(y)))
        return y

    @_stream_ordered
    def jacobian_apply_f32(self, z, y):
        """y += J z in FP32 (device tensors)"""
        _check(load().pdg_jacobian_apply_f32(self._h, _ptr(z, np.float32), _ptr(y, np.float32)))
        return y

    @_stream_ordered
    def apply_f32(self, x, y):
        """y = J x in FP32 (device tensors)"""
        _check(load().pdg_apply_f32(self._h, _ptr(x, np.float32), _ptr(y, np.float32)))
        return y

    @_stream_ordered
    def jacobian_apply_transpose_f32(self, z, y):
        """y += J^T z in FP32 (device tensors)"""
        _check(load().pdg_jacobian_apply_transpose_f32(self._h, _ptr(z, np.float32),
                                                       _ptr(y, np.float32)))
        return y

    @_stream_ordered
    def jacobian_apply_transpose(self, z, y):
        """y += J^T z"""
        _check(load().pdg_jacobian_apply_transpose(self._h, _ptr(z), _ptr(y)))
        return y

    @_stream_ordered
    def norm(self, v):
        out = C.c_double()
        _check(load().pdg_norm(self._h, _ptr(v), C.byref(out)))
        return out.value

    @_stream_ordered
    def dot(self, a, b):
        out = C.c_double()
        _check(load().pdg_dot(self._h, _ptr(a), _ptr(b), C.byref(out)))
        return out.value

    @_stream_ordered
    def grad_logK(self, u, lam, g):
        _check(load().pdg_grad_logK(self._h, _ptr(u), _ptr(lam), _ptr(g)))
        return g

    def set_nonlinearity(self, coef):
        """Volume term int q(u) psi, q(u) = sum_m coef[m] u^m (None removes it)."""
        if coef is None:
            _check(load().pdg_set_nonlinearity(self._h, 0, None))
            return
        c = np.ascontiguousarray(coef, dtype=np.float64)
        _check(load().pdg_set_nonlinearity(self._h, len(c) - 1, c.ctypes.data))

    @_stream_ordered
    def set_linearization_point(self, x):
        _check(load().pdg_set_linearization_point(self._h, _ptr(x)))

    @_stream_ordered
    def jacobian_apply_nonlinear(self, x, z, y):
        """y += J(x) z"""
        _check(load().pdg_jacobian_apply_nonlinear(self._h, _ptr(x), _ptr(z), _ptr(y)))
        return y

    def set_prec_options(self, options=None, **kw):
        """Options of the block preconditioners (SOR omega, block solver)."""
        o = options if options is not None else prec_options(**kw)
        _check(load().pdg_set_prec_options(self._h, C.byref(o)))

    def prec_block_iterations(self, precision=F64):
        """Iteration count of every block solve of the last iterative
        block-Jacobi application (SolverStatistics)."""
        out = np.zeros(self.ncell, dtype=np.int32)
        _check(load().pdg_prec_block_iterations(self._h, precision, out.ctypes.data))
        return out

    def jacobian_assemble(self):
        """Assemble the Jacobian on the device (GridOperator::jacobian)."""
        _check(load().pdg_jacobian_assemble(self._h))

    def jacobian_pattern(self):
        nnz = C.c_long()
        _check(load().pdg_jacobian_pattern(self._h, C.byref(nnz)))
        return nnz.value

    @_stream_ordered
    def jacobian_export(self, values=True):
        """(rowptr, colind, blocks[nnz, n, n]) in BCRS order; blocks row-major."""
        nnz = self.jacobian_pattern()
        rowptr = np.zeros(self.ncell + 1, dtype=np.int64)
        colind = np.zeros(nnz, dtype=np.int64)
        vals = np.zeros((nnz, self.nbasis, self.nbasis)) if values else None
        _check(load().pdg_jacobian_export(self._h, rowptr.ctypes.data, colind.ctypes.data,
                                          _ptr(vals) if values else None))
        return rowptr, colind, vals

    @_stream_ordered
    def matrix_apply(self, x, y):
        """y = A x with the assembled Jacobian"""
        _check(load().pdg_matrix_apply(self._h, _ptr(x), _ptr(y)))
        return y

    @_stream_ordered
    def mass_apply(self, x, y):
        """y = M x (DG mass matrix)"""
        _check(load().pdg_mass_apply(self._h, _ptr(x), _ptr(y)))
        return y

    @_stream_ordered
    def grad_source(self, lam, g):
        _check(load().pdg_grad_source(self._h, _ptr(lam), _ptr(g)))
        return g

    @_stream_ordered
    def adjoint_solve(self, rhs, lam, options=None):
        o = options or default_options()
        res = SolverResult()
        _check(load().pdg_adjoint_solve(self._h, C.byref(o), _ptr(rhs), _ptr(lam),
                                        C.byref(res)), allow=(PDG_ENOTCONVERGED,))
        return res

    def zeros(self):
        return np.zeros(self.ndof)


class OnTheFlyOperator:
    """ISTL LinearOperator over GridOperator::jacobian_apply."""

    def __init__(self, go: GridOperator):
        self.go = go

    @_stream_ordered
    def apply(self, x, y):
        """y = J x"""
        _check(load().pdg_apply(self.go.handle, _ptr(x), _ptr(y)))

    @_stream_ordered
    def applyscaleadd(self, alpha, x, y):
        """y += alpha J x"""
        _check(load().pdg_applyscaleadd(self.go.handle, float(alpha), _ptr(x), _ptr(y)))

    def category(self):
        return "sequential"


class GridOperatorPreconditioner:
    """ISTL Preconditioner: pre() sets up the cell-block Jacobi, apply(v, d)
    computes v = D^{-1} d."""

    def __init__(self, go: GridOperator, kind=PREC_BJ_FDM, precision=F64):
        self.go, self.kind, self.precision = go, kind, precision
        self._ready = False

    @_stream_ordered
    def pre(self, v=None, d=None):
        if not self._ready:
            _check(load().pdg_prec_setup(self.go.handle, self.kind, self.precision))
            self._ready = True

    @_stream_ordered
    def apply(self, v, d):
        if self.precision == F64:
            _check(load().pdg_prec_apply(self.go.handle, _ptr(d), _ptr(v)))
        else:
            _check(load().pdg_prec_apply_f32(self.go.handle, _ptr(d, np.float32),
                                             _ptr(v, np.float32)))

    def post(self, v=None):
        pass


class ISTLBackend_SEQ_MatrixFree_Base:
    """Matrix-free Krylov backend: apply(z, r, reduction) solves J z = r."""

    isMatrixFree = True

    def __init__(self, go: GridOperator, method=CG, preconditioner=PREC_BJ_FDM,
                 maxiter=5000, verbose=0, mixed=False, inner_reduction=1e-3):
        self.go = go
        self.opts = default_options(method=method, preconditioner=preconditioner,
                                    maxit=maxiter, verbose=verbose, mixed=int(mixed),
                                    inner_reduction=inner_reduction)
        self.res = SolverResult()

    @_stream_ordered
    def apply(self, z, r, reduction):
        self.opts.reduction = reduction
        _check(load().pdg_krylov_solve(self.go.handle, C.byref(self.opts), _ptr(z), _ptr(r),
                                       C.byref(self.res)), allow=(PDG_ENOTCONVERGED,))

    @_stream_ordered
    def norm(self, v):
        return self.go.norm(v)

    def result(self):
        return self.res


def onestep_table(method, theta=1.0):
    """(A, B, D) of a TimeSteppingParameterInterface scheme: A, B [s][s+1], D [s+1]."""
    st = C.c_int()
    A = np.zeros(20)
    B = np.zeros(20)
    D = np.zeros(5)
    _check(load().pdg_onestep_table(method, float(theta), C.byref(st), A.ctypes.data,
                                    B.ctypes.data, D.ctypes.data))
    s = st.value
    return A[:s * (s + 1)].reshape(s, s + 1).copy(), B[:s * (s + 1)].reshape(s, s + 1).copy(), \
        D[:s + 1].copy()


class OneStepMethod:
    """OneStepMethod(method, igos, pdesolver) (instationary/implicitonestep.hh):
    apply(time, dt, xold, xnew) advances one step and returns the step size
    taken (implicitonestep.hh:144); `method` is a scheme id (IMPLICIT_EULER,
    ALEXANDER2, ...) or explicit (A, B, D) tables."""

    def __init__(self, method, go: GridOperator, ls: "ISTLBackend_SEQ_MatrixFree_Base",
                 theta=1.0):
        self.go, self.ls = go, ls
        self.A, self.B, self.D = (onestep_table(method, theta) if np.isscalar(method)
                                  else [np.ascontiguousarray(t, dtype=np.float64) for t in method])
        self.res = OneStepResult()

    @_stream_ordered
    def apply(self, time, dt, xold, xnew):
        s = self.A.shape[0]
        A = np.ascontiguousarray(self.A, dtype=np.float64)
        B = np.ascontiguousarray(self.B, dtype=np.float64)
        D = np.ascontiguousarray(self.D, dtype=np.float64)
        _check(load().pdg_onestep_apply(self.go.handle, s, A.ctypes.data, B.ctypes.data,
                                        D.ctypes.data, float(dt), C.byref(self.ls.opts),
                                        _ptr(xold), _ptr(xnew), C.byref(self.res)))
        return dt

    def result(self):
        return self.res


class NewtonMethod:
    """NewtonMethod<GridOperator, LinearSolver> (solver/newton.hh): apply(u)
    solves R(u) = 0 from the initial guess u with the backend's Krylov
    method and preconditioner for the linear steps."""

    def __init__(self, go: GridOperator, ls: "ISTLBackend_SEQ_MatrixFree_Base", **kw):
        self.go, self.ls = go, ls
        self.opts = newton_options(**kw)
        self.res = NewtonResult()

    @_stream_ordered
    def apply(self, u):
        st = load().pdg_newton_solve(self.go.handle, C.byref(self.opts), C.byref(self.ls.opts),
                                     _ptr(u), C.byref(self.res))
        _check(st)
        return u

    def result(self):
        return self.res


class StationaryLinearProblemSolver:
    """r = R(x); J z = r; x -= z   (linearproblem.hh:188-302)."""

    def __init__(self, go: GridOperator, ls: ISTLBackend_SEQ_MatrixFree_Base, x, reduction,
                 min_defect=1e-99, verbose=0):
        self.go, self.ls, self.x = go, ls, x
        self.reduction, self.min_defect = reduction, min_defect
        self.res = SolverResult()

    @_stream_ordered
    def apply(self, x=None):
        if x is not None:
            self.x = x
        o = SolverOptions()
        C.memmove(C.byref(o), C.byref(self.ls.opts), C.sizeof(SolverOptions))
        o.reduction, o.min_defect = self.reduction, self.min_defect
        _check(load().pdg_solve_linear_problem(self.go.handle, C.byref(o), _ptr(self.x),
                                               C.byref(self.res)), allow=(PDG_ENOTCONVERGED,))
        self.ls.res = self.res
        return self.x

    def result(self):
        return self.res
