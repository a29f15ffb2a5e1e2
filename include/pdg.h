/*
 * pdg.h -- C ABI of the GB300-native matrix-free SIPG DG operator.
 *
 * One context holds one structured grid, one Q_k DG space and one
 * ConvectionDiffusionDG operator (SIPG/NIPG/IIPG), all resident on one
 * GPU.  Every entry point returns an int status (PDG_OK = 0); no C++
 * exception crosses this boundary.  pdg_last_error() returns a message for
 * the last failure on the calling thread.
 *
 * Vectors are Blocking::fixed DG vectors: DOF index = cell * (k+1)^d +
 * local basis index, cells numbered lexicographically with x fastest
 * (YaspGrid leaf order), local index x fastest (QkDG multiindex).
 *
 * Pointer convention: vector arguments may be device pointers (the fast
 * path) or host pointers; host pointers are detected and staged through
 * device buffers on the context's stream.  Nothing is allocated or freed
 * on behalf of the caller: ownership of every buffer stays with the caller.
 *
 * Streams: every call is ordered on the context's stream (pdg_set_stream);
 * calls that return host values (solves, norms, dots) synchronise it.
 */
#ifndef PDG_H
#define PDG_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- */
/* status codes                                                      */
/* ---------------------------------------------------------------- */
enum {
  PDG_OK = 0,
  PDG_EINVAL = 1,          /* bad argument (null pointer, bad size, bad enum) */
  PDG_ECUDA = 2,           /* a CUDA runtime call failed */
  PDG_ENOTCONVERGED = 3,   /* solver reached maxit without the reduction */
  PDG_EBREAKDOWN = 4,      /* Krylov breakdown (BiCGStab rho/omega/h tiny) */
  PDG_ESTATE = 5,          /* call order violated (e.g. prec not set up) */
  PDG_EUNSUPPORTED = 6,    /* configuration not compiled in / not supported */
  PDG_EOUTFLOW = 7,        /* outflow boundary on inflow (convectiondiffusiondg.hh:802-806) */
  PDG_ENONFINITE = 8,      /* NaN/Inf defect */
  PDG_ETIMEOUT = 9,        /* a bounded device wait ran out */
  PDG_ELINESEARCH = 10     /* Newton line search failed (LineSearchError,
                              solver/linesearch.hh:134-154) */
};

/* ConvectionDiffusionDGMethod::Type  (convectiondiffusiondg.hh:29-32) */
enum { PDG_NIPG = 0, PDG_SIPG = 1, PDG_IIPG = 2 };
/* ConvectionDiffusionDGWeights::Type (convectiondiffusiondg.hh:34-37) */
enum { PDG_WEIGHTS_ON = 0, PDG_WEIGHTS_OFF = 1 };
/* ConvectionDiffusionBoundaryConditions::Type
   (convectiondiffusionparameter.hh:111-115) */
enum { PDG_BC_DIRICHLET = 1, PDG_BC_NEUMANN = -1, PDG_BC_OUTFLOW = -2,
       PDG_BC_NONE = -3 };

/* Krylov methods (dune-istl CGSolver / BiCGSTABSolver as used by
   ISTLBackend_SEQ_MatrixFree_Base, backend/istl/matrixfree/backends.hh:62-143) */
enum { PDG_CG = 0, PDG_BICGSTAB = 1,
       PDG_GMRES = 2 /* restarted right-preconditioned GMRES(m); no
                        reference counterpart, the inner solver of the
                        mixed-precision solve for non-symmetric operators */ };
/* preconditioners */
enum {
  PDG_PREC_NONE = 0,
  PDG_PREC_BJ_FDM = 1,     /* cell-block Jacobi, inverse applied by fast
                              diagonalisation of the Kronecker-sum block
                              (exact for symmetric separable blocks) */
  PDG_PREC_BJ_DENSE = 2,   /* cell-block Jacobi, explicit per-cell inverse
                              (exact for every block, n^2 values per cell) */
  PDG_PREC_BJ_ITERATIVE = 3,/* fully matrix-free-style block Jacobi: each
                              block system solved by a local BiCGStab with
                              point-Jacobi preconditioner
                              (IterativeBlockJacobiPreconditionerLocalOperator,
                              matrixfree/iterativeblockjacobipreconditioner.hh:
                              262-452); options in pdg_prec_options */
  PDG_PREC_SOR = 16,       /* OR-ed with a block kind above: one forward
                              block-SOR sweep over the cells in grid order,
                              each block inverted by that kind
                              (BlockSORPreconditionerLocalOperator,
                              matrixfree/blocksorpreconditioner.hh:37-296);
                              the transposed preconditioner is the backward
                              sweep with transposed blocks */
  PDG_PREC_BLOCK_MASK = 15
};

/* Options of the block solvers: BlockSORPreconditionerLocalOperator's omega
   (blocksorpreconditioner.hh:59-63) and BlockSolverOptions
   (iterativeblockjacobipreconditioner.hh:202-233). */
typedef struct pdg_prec_options {
  double omega;            /* SOR relaxation factor (1.0) */
  double block_reduction;  /* residual reduction of each block solve (1e-5) */
  int block_maxit;         /* iteration cap of each block solve (100) */
  int block_precondition;  /* point-Jacobi inside the block solve (1) */
  double block_weight;     /* weight of that point Jacobi (1.0) */
  int dense_fp16;          /* PDG_PREC_BJ_DENSE in PDG_F32 precision: store each
                              block inverse in FP16 with one FP32 scale per block
                              (half the bytes per apply); no counterpart in the
                              reference, for the inner solves of mixed precision
                              (0) */
} pdg_prec_options;
/* precisions */
enum { PDG_F64 = 0, PDG_F32 = 1 };
/* local DG bases: QkDGBasisPolynomial (finiteelementmap/qkdg.hh:18).
   LAGRANGE: equidistant nodes j/k (qkdglagrange.hh:55-79); LEGENDRE:
   Legendre polynomials on [0,1] (qkdglegendre.hh:76-113), vectors hold
   modal coefficients; LOBATTO: Lagrange polynomials on the Gauss-Lobatto
   points, ascending (qkdglobatto.hh:21-117).  With LEGENDRE the nonlinear
   volume term, block SOR and explicit one-step stages are not available
   (PDG_EUNSUPPORTED). */
enum { PDG_BASIS_LAGRANGE = 0, PDG_BASIS_LEGENDRE = 1, PDG_BASIS_LOBATTO = 2 };

typedef struct pdg_context pdg_context;

/* Grid, space and operator configuration.  Mirrors the constructor
   arguments of YaspGrid (unit-cube extent), QkDGLocalFiniteElementMap
   (degree, dim) and ConvectionDiffusionDG (convectiondiffusiondg.hh:87-101:
   method, weights, alpha; intorderadd = 0). */
typedef struct pdg_config {
  int dim;                 /* 2 or 3 */
  int degree;              /* 1..4 */
  int cells[3];            /* cells per direction (cells[2] ignored in 2D) */
  double extent[3];        /* domain [0,extent[0]] x ... */
  int method;              /* PDG_SIPG, PDG_NIPG, PDG_IIPG */
  int weights;             /* PDG_WEIGHTS_ON / PDG_WEIGHTS_OFF */
  double alpha;            /* penalty factor */
  int bctype[6];           /* boundary type per side -x,+x,-y,+y,-z,+z */
  int device;              /* CUDA device ordinal */
  int basis;               /* PDG_BASIS_*: the QkDGBasisPolynomial of the
                              QkDGLocalFiniteElementMap */
} pdg_config;

/* Solver options: ISTLBackend_SEQ_MatrixFree_Base(go, precgo, maxiter,
   verbose) (backends.hh:71-72) plus StationaryLinearProblemSolver's
   reduction / min_defect (stationary/linearproblem.hh:111-120). */
typedef struct pdg_solver_options {
  int method;              /* PDG_CG / PDG_BICGSTAB */
  int preconditioner;      /* PDG_PREC_* */
  double reduction;        /* defect reduction relative to the first defect */
  double min_defect;       /* StationaryLinearProblemSolver min_defect */
  int maxit;
  int mixed;               /* 0: FP64 Krylov.  1: FP32 operator + FP32 block
                              Jacobi inside an FP64 outer loop: defect
                              correction for CG, flexible GMRES (outer
                              restart min(restart, max_outer)) for BiCGStab /
                              GMRES.  2: always defect correction.  3: always
                              flexible GMRES. */
  double inner_reduction;  /* mixed: reduction of each FP32 inner solve */
  int inner_maxit;         /* mixed: iteration cap of each inner solve */
  int max_outer;           /* mixed: cap on outer steps (defect corrections
                              or flexible-GMRES steps) */
  int verbose;
  double inner_breakdown;  /* mixed: relative breakdown test of the FP32
                              BiCGStab (|<rt,v>| < tol |rt||v|, likewise rho);
                              0 keeps only dune-istl's absolute tests */
  int inner_method;        /* mixed: Krylov method of the FP32 inner solves;
                              -1 = the outer method (CG or BiCGStab) */
  int restart;             /* GMRES restart length m (1..64) */
  int inner_replace;       /* mixed, BiCGStab: replace the recursive residual
                              by b - A x every this many iterations (0 = never) */
  int inner_vectors;       /* mixed: precision of the inner Krylov vectors and
                              recurrences: PDG_F32, or PDG_F64 with the operator
                              and the block Jacobi still applied in FP32;
                              -1 = FP32, except FP64 for BiCGStab / GMRES
                              under plain defect correction (mixed = 2) */
  int assembled;           /* 1: the Krylov operator is the assembled Jacobian
                              (pdg_jacobian_assemble; assembled on first use),
                              the matrix-based path of the reference's
                              matrix-free tests; FP64 only */
} pdg_solver_options;

/* LinearSolverResult (backend/solver.hh:29-51) +
   StationaryLinearProblemSolverResult (stationary/linearproblem.hh:27-44) */
typedef struct pdg_solver_result {
  int converged;
  int iterations;          /* Krylov iterations (sum of inner ones if mixed) */
  double elapsed;          /* seconds, device clock */
  double reduction;
  double conv_rate;
  double first_defect;
  double defect;
  int outer_iterations;    /* mixed: outer steps */
  int status;
} pdg_solver_result;

/* ---------------------------------------------------------------- */
/* context                                                           */
/* ---------------------------------------------------------------- */

/* Replaces building YaspGrid + GridFunctionSpace + ConvectionDiffusionDG +
   GridOperator (test/matrixfree/matrix_free_linear.cc:73-151). */
int pdg_create(const pdg_config *cfg, pdg_context **out);
/* Ends the objects pdg_create replaces (their destructors). */
int pdg_destroy(pdg_context *ctx);
/* Message of the last failure on the calling thread: the text the reference
   puts in the Dune::Exception it throws (DUNE_THROW); no exception crosses
   this boundary. */
const char *pdg_last_error(void);
/* Defaults of the solver options: maxiter 5000 as in the
   ISTLBackend_SEQ_MatrixFree_Base constructor
   (backend/istl/matrixfree/backends.hh:74-78). */
void pdg_default_solver_options(pdg_solver_options *opt);

/* Stream for all subsequent work (cudaStream_t passed as void*; NULL =
   the context's own non-blocking stream).  No reference counterpart (the
   reference runs on the host). */
int pdg_set_stream(pdg_context *ctx, void *stream);

/* The stream the context currently works on (the one set by pdg_set_stream,
   else its own).  No reference counterpart: a caller on another stream
   (a framework's current stream) orders its own work against this one with
   events before and after passing device buffers. */
int pdg_get_stream(const pdg_context *ctx, void **stream);

/* sizes: cells, basis functions per cell, DOFs, volume quadrature points
   per cell ((k+1)^d) and boundary quadrature points in total (the sizes of
   GridFunctionSpace::size() and of the Blocking::fixed blocks,
   backend/istl/descriptors.hh:26-47) */
int pdg_sizes(const pdg_context *ctx, long *ncell, int *nbasis, long *ndof,
              int *nq_volume, long *nq_boundary);

/* Quadrature-point coordinates (host output) so that callers evaluate
   their parameter functions where the operator integrates them:
   volume [ncell][(k+1)^d][dim]; boundary points grouped by side, faces
   lexicographic over the remaining directions, (k+1)^(d-1) points each.
   No reference counterpart: the reference evaluates f, g, j, o inside the
   local operator at the same Gauss points of order 2k
   (convectiondiffusiondg.hh:1060-1061, :745-746). */
int pdg_volume_points(const pdg_context *ctx, double *xyz);
int pdg_boundary_points(const pdg_context *ctx, double *xyz);

/* ---------------------------------------------------------------- */
/* parameters (ConvectionDiffusionModelProblem, convectiondiffusion-   */
/* parameter.hh:134-209; permeabilityIsConstantPerCell() == true)     */
/* ---------------------------------------------------------------- */

/* A(cell) = K_e I per cell; is_log != 0 means the array holds log K.  Drops
   a tensor of pdg_set_permeability_tensor / _points. */
int pdg_set_permeability(pdg_context *ctx, const double *K, int is_log);
/* c(cell) per cell (NULL = 0) */
int pdg_set_reaction(pdg_context *ctx, const double *c);
/* b(x) = sum_m coef_m sin(2 pi kv_m . x + phase_m); modes [n][7] =
   kx ky kz phase cx cy cz (n = 0 clears the velocity; in 2D the z entries are
   ignored).  PDG_EOUTFLOW if an outflow side sees inflow. */
int pdg_set_velocity_modes(pdg_context *ctx, int nmodes, const double *modes);
/* f at volume quadrature points [ncell][(k+1)^d] (NULL = 0) plus a per-cell
   constant fc [ncell] (NULL = 0).  Used by lambda_volume
   (convectiondiffusiondg.hh:1047-1075). */
int pdg_set_source(pdg_context *ctx, const double *fq, const double *fc);
/* Boundary data at boundary quadrature points (NULL = 0): Dirichlet g,
   Neumann j, outflow o (convectiondiffusiondg.hh:770-879). */
int pdg_set_boundary_data(pdg_context *ctx, const double *g, const double *j,
                          const double *o);

/* Parameter fields beyond A = K I, as ConvectionDiffusionDG evaluates them
   (convectiondiffusionparameter.hh:143-183: A(cell, x) a d x d tensor,
   b(cell, x), c(cell, x) per point).  With any of these set the diffusion
   and reaction terms are evaluated at the operator's Gauss points (order
   2k) instead of in Kronecker form; the FDM block Jacobi (which needs
   separable blocks) and the log-K gradient are then unavailable
   (PDG_EUNSUPPORTED): use PDG_PREC_BJ_DENSE or PDG_PREC_BJ_ITERATIVE.
   pdg_set_permeability drops a tensor set before. */

/* A(cell) per cell [ncell][dim][dim], row-major (A[i][j] multiplies
   d u/d x_j in row i), taken at the cell centre as the reference does
   (convectiondiffusiondg.hh:124-127, 305-309, 710-713).  NULL returns to
   A = K I. */
int pdg_set_permeability_tensor(pdg_context *ctx, const double *A);
/* permeabilityIsConstantPerCell() == false: A at every volume quadrature
   point [ncell][(k+1)^d][dim][dim] (order of pdg_volume_points) and at
   every cell's own points of its 2d faces [ncell][2d][(k+1)^(d-1)][dim][dim]
   (sides -x,+x,-y,+y,-z,+z; points of pdg_cell_face_points), where
   alpha_volume, alpha_skeleton and the boundary integral re-evaluate it
   (convectiondiffusiondg.hh:141-146, 365-382, 750-761); weights and
   penalty are then formed per point.  Both NULL returns to A = K I. */
int pdg_set_permeability_points(pdg_context *ctx, const double *Avol, const double *Aface);
/* c(cell, x) at the volume quadrature points [ncell][(k+1)^d], added to the
   per-cell c of pdg_set_reaction (convectiondiffusiondg.hh:181).  NULL
   removes it. */
int pdg_set_reaction_points(pdg_context *ctx, const double *cq);
/* b(cell, x) at the volume quadrature points [ncell][(k+1)^3][3] and at
   the face-lattice points [nfaces][(k+1)^2][3] (pdg_face_lattice_points):
   one value per face point serves both sides, as the reference upwinds
   with the inside cell's b and assumes an H(div) field
   (convectiondiffusiondg.hh:425-426, 796-797); in 2D the third component
   is ignored.  Replaces Fourier modes.  Both NULL removes the velocity. */
int pdg_set_velocity_points(pdg_context *ctx, const double *bvol, const double *bface);
/* The face lattice: every face of the grid once.  Faces normal to x come
   first, then y, then z; per direction the planes 0..cells[dir] in order;
   in a plane the faces are lexicographic over the other directions (x
   fastest); (k+1)^(d-1) points per face, lexicographic over the other
   directions.  No reference counterpart (the reference calls b(cell, x)
   at these points). */
int pdg_face_lattice_size(const pdg_context *ctx, long *nfaces);
/* coordinates of the face-lattice points [nfaces][(k+1)^(d-1)][dim] and of
   every cell's own face points [ncell][2d][(k+1)^(d-1)][dim] (host
   outputs), for evaluating b and A where the operator integrates them */
int pdg_face_lattice_points(const pdg_context *ctx, double *xyz);
int pdg_cell_face_points(const pdg_context *ctx, double *xyz);

/* ---------------------------------------------------------------- */
/* operator (GridOperator, gridoperator/gridoperator.hh:176-205)      */
/* ---------------------------------------------------------------- */

/* GridOperator::residual(x, r): r += R(x)  (gridoperator.hh:176-181) */
int pdg_residual(pdg_context *ctx, const double *x, double *r);
/* GridOperator::jacobian_apply(z, y): y += J z  (gridoperator.hh:192-197) */
int pdg_jacobian_apply(pdg_context *ctx, const double *z, double *y);
/* Same in FP32 (the inner operator of the mixed-precision solve).  No
   reference counterpart: the reference computes in RF = double
   (test/matrixfree/matrix_free_linear.cc:89). */
int pdg_jacobian_apply_f32(pdg_context *ctx, const float *z, float *y);
/* Transposed apply y += J^T z (adjoint; no reference counterpart, derived
   from jacobian_skeleton's sn/ns blocks, convectiondiffusiondg.hh:483-669) */
int pdg_jacobian_apply_transpose(pdg_context *ctx, const double *z, double *y);
/* Same in FP32, device pointers (the transposed inner operator of the
   mixed-precision adjoint solve) */
int pdg_jacobian_apply_transpose_f32(pdg_context *ctx, const float *z, float *y);
/* y = J x in FP32, device pointers: the operator apply of the inner CG of the
   mixed-precision solve (OnTheFlyOperator::apply in FP32) */
int pdg_apply_f32(pdg_context *ctx, const float *x, float *y);
/* OnTheFlyOperator::apply(x, y): y = J x
   (backend/istl/seqistlsolverbackend.hh:66-76) */
int pdg_apply(pdg_context *ctx, const double *x, double *y);
/* OnTheFlyOperator::applyscaleadd(alpha, x, y): y += alpha J x
   (seqistlsolverbackend.hh:78-90), without the full-vector temporary */
int pdg_applyscaleadd(pdg_context *ctx, double alpha, const double *x, double *y);

/* Arithmetic of the FP64 operator applies.  No reference counterpart (the
   reference computes in RF = double).  PDG_F64_FLOAT_PAIR carries every FP64
   value of the 3D operator kernel (scalar or diagonal-tensor K per cell) as
   an unevaluated sum of two floats and runs the multiply-adds on the FP32
   pipe (exact two-product and two-sum, 48 significant bits): results agree
   with PDG_F64_NATIVE to about 1e-14 relative; every other kernel (convection,
   tensor fields, preconditioners, vector updates) stays FP64.  3D only. */
enum { PDG_F64_NATIVE = 0, PDG_F64_FLOAT_PAIR = 1 };
int pdg_set_f64_arithmetic(pdg_context *ctx, int mode);

/* ---------------------------------------------------------------- */
/* preconditioner (GridOperatorPreconditioner over                    */
/* AssembledBlockJacobiPreconditionerLocalOperator,                   */
/* backend/istl/matrixfree/gridoperatorpreconditioner.hh:45-84,       */
/* assembledblockjacobipreconditioner.hh:162-233)                     */
/* ---------------------------------------------------------------- */

/* GridOperatorPreconditioner::pre: set up cell-block Jacobi of the given
   kind in the given precision (PDG_F64 or PDG_F32). */
int pdg_prec_setup(pdg_context *ctx, int kind, int precision);
/* GridOperatorPreconditioner::apply(v, d): v = D^{-1} d */
int pdg_prec_apply(pdg_context *ctx, const double *d, double *v);
int pdg_prec_apply_f32(pdg_context *ctx, const float *d, float *v);
/* v = D^{-T} d (adjoint solve preconditioner) */
int pdg_prec_apply_transpose(pdg_context *ctx, const double *d, double *v);

/* ---------------------------------------------------------------- */
/* vector helpers (SequentialNorm, backend/solver.hh:16-25)           */
/* ---------------------------------------------------------------- */
int pdg_norm(pdg_context *ctx, const double *v, double *out);
int pdg_dot(pdg_context *ctx, const double *a, const double *b, double *out);

/* Dot product *result = sum_i a[i] b[i] of two device vectors that
   allocates nothing.  No counterpart in the reference.  For callers that
   cannot allocate device memory when they call: host solvers that own every
   buffer and forbid library allocations after set-up (a dune-istl Krylov
   loop over device vectors asks for a dot product in every iteration), and
   embeddings that budget device memory and must not see the hidden
   allocations, or the synchronisation, of cudaMalloc and cudaFree.  No
   context is needed.  a, b and result are device pointers on the current
   device (others are rejected with PDG_EINVAL); the result is written on
   `stream` (cudaStream_t as void*, NULL = legacy default stream).  The
   reduction scratch is a file-scope device array of 1024 partial sums that
   every GPU loading the library holds until exit; n <= PDG_DOT_NOALLOC_MAX_N
   (1024 chunks of 65,536 elements) and larger n is rejected with PDG_EINVAL.
   The first call on a device (and the first call after cudaDeviceReset gave
   the device a new context) looks up the array's device address with that
   device current; make that first call before any stream capture.  All
   calls share the one array: calls that overlap on the GPU (other streams,
   other threads) race and must be serialised by the caller. */
#define PDG_DOT_NOALLOC_MAX_N 67108864L
int pdg_dot_noalloc(long n, const double *a, const double *b, double *result,
                    void *stream);

/* ---------------------------------------------------------------- */
/* solvers                                                           */
/* ---------------------------------------------------------------- */

/* ISTLBackend_SEQ_MatrixFree_Base::apply(z, r, reduction)
   (backends.hh:116-126): Krylov solve J z = r from the initial guess in z;
   r is overwritten with the final defect. */
int pdg_krylov_solve(pdg_context *ctx, const pdg_solver_options *opt,
                     double *z, double *r, pdg_solver_result *res);

/* StationaryLinearProblemSolver::apply (stationary/linearproblem.hh:
   188-302): r = R(x); solve J z = r to max(reduction, min_defect/|r|);
   x -= z.  With opt->mixed the correction is computed by FP32 Krylov
   solves inside an FP64 defect-correction loop that stops on the true
   FP64 defect. */
int pdg_solve_linear_problem(pdg_context *ctx, const pdg_solver_options *opt,
                             double *x, pdg_solver_result *res);

/* Defaults of pdg_prec_options: the reference's (the iterative block
   Jacobi's and block SOR's constructor arguments,
   backend/istl/matrixfree/iterativeblockjacobipreconditioner.hh:302-310,
   blocksorpreconditioner.hh:38-296). */
void pdg_default_prec_options(pdg_prec_options *o);
/* Options used by the next pdg_prec_setup (and every apply after it). */
int pdg_set_prec_options(pdg_context *ctx, const pdg_prec_options *o);
/* SolverStatistics (matrixfree/solverstatistics.hh:17-146): iteration count
   of every block solve of the last application of the PDG_PREC_BJ_ITERATIVE
   preconditioner in `precision`, one per cell (ncell ints, host array). */
int pdg_prec_block_iterations(pdg_context *ctx, int precision, int *iterations);

/* ---------------------------------------------------------------- */
/* nonlinear operator and Newton                                     */
/* ---------------------------------------------------------------- */

/* NonlinearConvectionDiffusionDG (test/localoperator/
   nonlinearconvectiondiffusiondg.hh:28-307): the operator plus the volume
   term int q(u) psi with q(u) = sum_{m<=degree} coef[m] u^m (degree 1..4);
   coef = NULL removes it.  The residual includes the term; Jacobian applies
   add int q'(u(x)) z psi at the linearization point x. */
int pdg_set_nonlinearity(pdg_context *ctx, int degree, const double *coef);
/* OnTheFlyOperator / GridOperatorPreconditioner::setLinearizationPoint
   (backends.hh:129-135, gridoperatorpreconditioner.hh:38-42): the point x
   of every following Jacobian apply and Krylov solve. */
int pdg_set_linearization_point(pdg_context *ctx, const double *x);
/* GridOperator::jacobian_apply(x, z, y) (gridoperator.hh:200-205):
   y += J(x) z (sets x as the linearization point). */
int pdg_jacobian_apply_nonlinear(pdg_context *ctx, const double *x, const double *z,
                                 double *y);

/* NewtonMethod (solver/newton.hh:63-669) with DefaultTerminate
   (solver/terminate.hh:20-76) and the Hackbusch-Reusken line search
   (solver/linesearch.hh:71-209); defaults are the reference's. */
typedef struct pdg_newton_options {
  double reduction;              /* 1e-8 */
  double absolute_limit;         /* 1e-12 */
  int max_iterations;            /* 40 */
  int force_iteration;           /* 0 */
  double min_linear_reduction;   /* 1e-3 */
  int fixed_linear_reduction;    /* 0 */
  int line_search;               /* 1: Hackbusch-Reusken, 0: none (full steps) */
  int line_search_max_iterations;/* 10 */
  double line_search_damping;    /* 0.5 */
  int line_search_accept_best;   /* 0 */
  int verbose;
} pdg_newton_options;
/* NewtonResult (newton.hh) */
typedef struct pdg_newton_result {
  int converged;
  int iterations;
  double first_defect, defect, reduction, conv_rate;
  int linear_solver_iterations;
  double elapsed;
  int status;
} pdg_newton_result;
void pdg_default_newton_options(pdg_newton_options *o);
/* NewtonMethod::apply(u): u is the initial guess and the result; the
   linear solves use `lin` (its reduction is replaced by Newton's linear
   reduction; the preconditioner is set up at the first linearization point
   and kept, as GridOperatorPreconditioner::pre does). */
int pdg_newton_solve(pdg_context *ctx, const pdg_newton_options *opt,
                     const pdg_solver_options *lin, double *u, pdg_newton_result *res);

/* ---------------------------------------------------------------- */
/* instationary one-step methods                                     */
/* ---------------------------------------------------------------- */

/* y = M x with the DG mass matrix: the temporal operator L2
   (localoperator/l2.hh:45-89, 149-152) of the one-step grid operator. */
int pdg_mass_apply(pdg_context *ctx, const double *x, double *y);

/* TimeSteppingParameterInterface implementations
   (instationary/onestepparameter.hh: theta :89, explicit / implicit Euler
   :164 / :189, Heun :214, Shu3 :287, RK4 :364, Alexander2 :445,
   fractional step :522, Alexander3 :605): */
enum {
  PDG_ONESTEP_THETA = 0,          /* OneStepThetaParameter(theta) */
  PDG_ONESTEP_IMPLICIT_EULER = 1, /* theta = 1 */
  PDG_ONESTEP_EXPLICIT_EULER = 2, /* theta = 0 */
  PDG_ONESTEP_ALEXANDER2 = 3,
  PDG_ONESTEP_ALEXANDER3 = 4,
  PDG_ONESTEP_FRACTIONAL_STEP = 5,
  PDG_ONESTEP_HEUN = 6,
  PDG_ONESTEP_SHU3 = 7,
  PDG_ONESTEP_RK4 = 8
};
/* The method's tables: *stages = s, A and B [s][s+1] (row r-1 holds
   a(r, 0..s), b(r, 0..s)), D [s+1]; arrays of at least 4*5 and 5 values. */
int pdg_onestep_table(int method, double theta, int *stages, double *A, double *B,
                      double *D);
typedef struct pdg_onestep_result {
  int stages;
  int linear_solver_iterations;
  double elapsed;
  int status;
} pdg_onestep_result;
/* OneStepMethod::apply(time, dt, xold, xnew) (instationary/implicitonestep.hh:
   144-275): stage r solves
     sum_{j<r} [a_rj M x_j + b_rj dt R(x_j)] + a_rr M x_r + b_rr dt R(x_r) = 0
   (residual weights of the one-step local assembler with
   MultiplyOperator0ByDT, gridoperator/onestep/prestageengine.hh:181-227);
   implicit stages by the Krylov solver `lin` on the operator J + a_rr/(b_rr dt) M,
   explicit stages (b_rr = 0) by the exact block-diagonal mass inverse.  The
   spatial data (f, g, j, o) are time-independent. */
int pdg_onestep_apply(pdg_context *ctx, int stages, const double *A, const double *B,
                      const double *D, double dt, const pdg_solver_options *lin,
                      const double *xold, double *xnew, pdg_onestep_result *res);

/* ---------------------------------------------------------------- */
/* assembled Jacobian                                                */
/* ---------------------------------------------------------------- */

/* GridOperator::jacobian(x, A) (gridoperator/gridoperator.hh:184-189) with
   ConvectionDiffusionDG::jacobian_volume / _skeleton / _boundary
   (convectiondiffusiondg.hh:198-266, 483-669, 901-1044): assembles every
   block of the Jacobian on the device (kept in the context; invalidated
   when a coefficient changes). */
int pdg_jacobian_assemble(pdg_context *ctx);
/* Number of nonzero blocks of the BCRS pattern (ncell + 2 * interior faces;
   PDELab's pattern: the cell and its face neighbours, assembled by
   GridOperator::jacobian, gridoperator/gridoperator.hh:184-189). */
int pdg_jacobian_pattern(const pdg_context *ctx, long *nnz_blocks);
/* Export in ISTL BCRSMatrix<FieldMatrix<double,n,n>> layout: rowptr
   [ncell+1] and colind [nnz_blocks] (host arrays; either may be NULL),
   values [nnz_blocks * n * n] (host or device; NULL skips), block rows in
   cell order, column blocks ascending, each block row-major (test function
   i, trial function j). */
int pdg_jacobian_export(pdg_context *ctx, long *rowptr, long *colind, double *values);
/* y = A x with the assembled Jacobian (dune-istl MatrixAdapter::apply, the
   operator of the matrix-based backends,
   backend/istl/seqistlsolverbackend.hh:138). */
int pdg_matrix_apply(pdg_context *ctx, const double *x, double *y);

/* ---------------------------------------------------------------- */
/* adjoint (no reference counterpart)                                */
/* ---------------------------------------------------------------- */

/* Solve J^T lambda = rhs (lambda: initial guess in, solution out). */
int pdg_adjoint_solve(pdg_context *ctx, const pdg_solver_options *opt,
                      const double *rhs, double *lambda,
                      pdg_solver_result *res);
/* Fused per-cell gradient g_e = -lambda^T dR(u)/d(log K_e), the sum of the
   volume, interior-face and Dirichlet-face contributions. */
int pdg_grad_logK(pdg_context *ctx, const double *u, const double *lambda,
                  double *g);
/* g_e = -lambda^T dR/d(fc_e) = sum_i lambda_{e,i} int_e psi_i */
int pdg_grad_source(pdg_context *ctx, const double *lambda, double *g);

#ifdef __cplusplus
}
#endif
#endif
