/*
 * pdg_oracle.h -- CPU restatement of PDELab's matrix-free SIPG DG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA
 * implementation is checked against.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  The product library
 * (libpdg.so) never links or calls it.
 *
 * Parity status: the reference publishes no golden vectors or stored
 * outputs for this path and cannot be built here (it needs the DUNE core
 * modules and Eigen).  The restatement is pinned against the reference
 * tests' own assertions instead:
 *   - dune/pdelab/test/matrixfree/matrix_free_linear.cc:387-393
 *     (2D Q1 16x16 SIPG alpha=3: L2 err^2 < 1e-6 and equal Krylov
 *     iteration counts matrix-based vs matrix-free),
 *   - dune/pdelab/test/testfastdgassembler.cc:160-175 (2D Q1 32x32 SIPG
 *     alpha=2: L2 err^2 < 1e-8),
 *   - dune/pdelab/test/testblocklocaloperatorwrapper.cc:200-276 (block
 *     diagonal of the assembled Jacobian equals the block-diagonal
 *     wrapper's blocks to 1e-14),
 *   - dune/pdelab/test/testconvectiondiffusiondg.cc:160-168 (the operator's
 *     default arguments, alpha = 1: L2 err^2 < 1e-6),
 *   - dune/pdelab/test/testinstationaryfastdgassembler.cc:226-235 (one
 *     Alexander2 step on 8x8 Q1: L2 err^2 < 5e-6),
 *   - dune/pdelab/test/matrixfree/matrix_free_nonlinear.cc:386-405 (Newton
 *     on the nonlinear test problem),
 *   - dune/pdelab/test/testdglegendre.cc:146-194 (Legendre, Lobatto and
 *     Lagrange spaces give the same advection solution, L2 diff^2 < 1e-14).
 *
 * Everything follows the loop structure of the reference: per-point basis
 * evaluation, dense O(q*n) loops, one-sided face visits (inside = larger
 * cell index), assembled local blocks, per-cell partial-pivot LU.
 *
 * Geometry: structured axis-parallel grid on [0,L0]x[0,L1](x[0,L2]),
 * cells numbered lexicographically with x fastest (YaspGrid leaf order),
 * DOF index = cell * (k+1)^d + local basis index (Blocking::fixed).
 */
#ifndef PDG_ORACLE_H
#define PDG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ConvectionDiffusionBoundaryConditions::Type
   (convectiondiffusionparameter.hh:111-115) */
enum { PDGO_BC_DIRICHLET = 1, PDGO_BC_NEUMANN = -1, PDGO_BC_OUTFLOW = -2,
       PDGO_BC_NONE = -3 };

/* ConvectionDiffusionDGMethod::Type (convectiondiffusiondg.hh:29-32) */
enum { PDGO_NIPG = 0, PDGO_SIPG = 1, PDGO_IIPG = 2 };
/* ConvectionDiffusionDGWeights::Type (convectiondiffusiondg.hh:34-37) */
enum { PDGO_WEIGHTS_ON = 0, PDGO_WEIGHTS_OFF = 1 };
/* QkDGBasisPolynomial (finiteelementmap/qkdg.hh:18) */
enum { PDGO_LAGRANGE = 0, PDGO_LEGENDRE = 1, PDGO_LOBATTO = 2 };

/* status codes */
enum { PDGO_OK = 0, PDGO_EARG = 1, PDGO_EOUTFLOW_ON_INFLOW = 2,
       PDGO_EBREAKDOWN = 3, PDGO_ESINGULAR = 4,
       PDGO_ENOTCONV = 5 /* Newton: iteration cap, line search or non-finite defect */ };

typedef struct pdgo_problem {
  int dim;            /* 2 or 3 */
  int k;              /* polynomial degree, 1..6 */
  int nc[3];          /* cells per direction */
  double L[3];        /* domain extent, lower-left corner at 0 */
  int method;         /* PDGO_NIPG / PDGO_SIPG / PDGO_IIPG */
  int weights;        /* PDGO_WEIGHTS_ON / PDGO_WEIGHTS_OFF */
  double alpha;       /* penalty factor */
  int bctype[6];      /* per boundary side: -x,+x,-y,+y,-z,+z */
  /* coefficients (NULL = default) */
  const double *K;    /* [ncell] scalar diffusion A = K I, default 1 */
  const double *c;    /* [ncell] reaction, default 0 */
  int nmodes;         /* velocity b(x) = sum_m coef_m sin(2 pi kv_m.x + ph_m) */
  const double *modes;/* [nmodes][7] = kx ky kz phase cx cy cz */
  const double *fq;   /* [ncell][nq^d] source at volume quadrature points */
  const double *fc;   /* [ncell] source constant per cell (added to fq) */
  const double *gq;   /* Dirichlet g at boundary quadrature points */
  const double *jq;   /* Neumann flux j at boundary quadrature points */
  const double *oq;   /* outflow flux o at boundary quadrature points */
  /* NonlinearConvectionDiffusionDG (test/localoperator/
     nonlinearconvectiondiffusiondg.hh): volume term int q(u) psi,
     q(u) = sum_m nl_coef[m] u^m (nl_deg 0 = none); Jacobian applies and
     assembled blocks are taken at the linearization point xlin. */
  int nl_deg;
  double nl_coef[5];
  const double *xlin;
  /* local basis of the QkDG space (QkDGBasisPolynomial,
     finiteelementmap/qkdg.hh:18): PDGO_LAGRANGE (default), PDGO_LEGENDRE,
     PDGO_LOBATTO */
  int basis;
  /* Diffusion tensor beyond A = K I (ConvectionDiffusionModelProblem::A,
     convectiondiffusionparameter.hh:148-157): Acell [ncell][d][d] row-major
     is A(cell, centre) and replaces K.  With Aq_vol and Aq_face both set,
     permeabilityIsConstantPerCell() is false and A is taken at every
     quadrature point (convectiondiffusiondg.hh:141-146, 365-382, 750-761):
     Aq_vol [ncell][nq^d][d][d] at the volume points, Aq_face
     [ncell][2d][nq^(d-1)][d][d] at each cell's own points of its faces
     -x,+x,-y,+y(,-z,+z), in the face-point order of the boundary points. */
  const double *Acell;
  const double *Aq_vol;
  const double *Aq_face;
  /* reaction c(cell, x) per volume quadrature point [ncell][nq^d] (added to
     the per-cell c) */
  const double *cq;
  /* velocity b(cell, x) per point; both set replaces the Fourier modes.
     bq_vol [ncell][nq^d][d]; bq_face [face lattice][nq^(d-1)][d], one value
     per face point shared by both sides (the reference upwinds with b from
     the inside cell and assumes an H(div) field, :425-426): see
     pdgo_face_lattice_index for the face numbering. */
  const double *bq_vol;
  const double *bq_face;
} pdgo_problem;

typedef struct pdgo_result {
  int converged;
  int iterations;
  double reduction;
  double conv_rate;
  double first_defect;
  double defect;
  int status;
} pdgo_result;

/* sizes */
long pdgo_ncell(const pdgo_problem *p);
int  pdgo_nbasis(const pdgo_problem *p);
long pdgo_ndof(const pdgo_problem *p);
/* number of quadrature points per boundary side (faces * nq^(d-1)) */
long pdgo_nbpts_side(const pdgo_problem *p, int side);
/* offset of a side's block inside a boundary-point array */
long pdgo_bpts_offset(const pdgo_problem *p, int side);
long pdgo_nbpts_total(const pdgo_problem *p);

/* 1D tables: Gauss-Legendre points/weights on [0,1] with m points */
int pdgo_gauss_legendre(int m, double *x, double *w);
/* Lagrange basis p_i(x) / dp_i(x) of degree k at equidistant nodes */
double pdgo_lagrange(int k, int i, double x);
double pdgo_dlagrange(int k, int i, double x);
/* 1D basis function i of degree k of the given kind and its derivative */
double pdgo_basis1d(int basis, int k, int i, double x);
double pdgo_dbasis1d(int basis, int k, int i, double x);
/* Gauss-Lobatto points and weights on [0,1], m >= 2, ascending */
int pdgo_gauss_lobatto(int m, double *x, double *w);

/* coordinates of every volume quadrature point, [ncell][nq^d][dim] */
int pdgo_volume_points(const pdgo_problem *p, double *xyz);
/* coordinates of every boundary quadrature point, [side blocks][dim] */
int pdgo_boundary_points(const pdgo_problem *p, double *xyz);

/* GridOperator::jacobian_apply(z, y): y += J z  (gridoperator.hh:192-197) */
int pdgo_jacobian_apply(const pdgo_problem *p, const double *z, double *y);
/* Same, restricted to the element loop over cells [e_begin, e_end) (the
   faces those cells visit included); partial results over a partition of
   the cells sum to the full apply. */
int pdgo_jacobian_apply_range(const pdgo_problem *p, const double *z, double *y,
                              long e_begin, long e_end);
/* y += J^T z, matrix-free: the transposed local forms of jacobian_apply
   over the same one-sided traversal (no reference counterpart; checked
   against the transposed assembled blocks). */
int pdgo_jacobian_apply_transpose(const pdgo_problem *p, const double *z, double *y);
int pdgo_jacobian_apply_transpose_range(const pdgo_problem *p, const double *z, double *y,
                                        long e_begin, long e_end);
/* The face lattice of the grid: every face once.  Faces normal to x come
   first, then y, then z; per direction the planes 0..nc[dir] in order, and
   in a plane the faces lexicographic over the other directions (x
   fastest).  Face (dir, cell ix, upper side hi) has index
   pdgo_face_lattice_index(p, dir, ix[dir] + hi, ix). */
long pdgo_nface_lattice(const pdgo_problem *p);
long pdgo_face_lattice_index(const pdgo_problem *p, int dir, int plane, const int *ix);
/* coordinates of every face-lattice point [faces][nq^(d-1)][dim] and of
   every cell's own face points [ncell][2d][nq^(d-1)][dim] */
int pdgo_face_lattice_points(const pdgo_problem *p, double *xyz);
int pdgo_cell_face_points(const pdgo_problem *p, double *xyz);
/* GridOperator::residual(x, r): r += R(x)  (gridoperator.hh:176-181) */
int pdgo_residual(const pdgo_problem *p, const double *x, double *r);

/* Assembled Jacobian, block rows: [ncell][2d+1][nb][nb].
   slot 0 = diagonal block, slot 1+f = coupling across face f=2*dir+hi. */
int pdgo_assemble_jacobian(const pdgo_problem *p, double *blocks);
int pdgo_blocks_apply(const pdgo_problem *p, const double *blocks,
                      const double *x, double *y);   /* y = A x */
/* Jacobian with the transposed blocks: y = A^T x */
int pdgo_blocks_apply_transpose(const pdgo_problem *p, const double *blocks,
                                const double *x, double *y);

/* Block-diagonal (assembleLocalDiagonalBlock, blockdiagonalwrapper.hh:
   225-257) per cell [ncell][nb][nb] */
int pdgo_block_diagonal(const pdgo_problem *p, double *diag);
/* In-place partial-pivot LU of every block; piv [ncell][nb] */
int pdgo_lu_factor(int nb, long nblocks, double *a, int *piv);
/* v = D^{-1} d using the factors */
void pdgo_lu_apply(int nb, long nblocks, const double *lu, const int *piv,
                   const double *d, double *v);

/* Krylov solvers (restatement of dune-istl CGSolver / BiCGSTABSolver):
   op: 0 = matrix-free jacobian_apply, 1 = assembled blocks (A),
       2 = assembled blocks transposed (A^T).
   prec: 0 = none, 1 = block Jacobi from lu/piv.
   x is the initial guess and the result, b is overwritten by the defect. */
int pdgo_cg(const pdgo_problem *p, int op, const double *blocks,
            const double *lu, const int *piv, double *x, double *b,
            double reduction, int maxit, pdgo_result *res);
int pdgo_bicgstab(const pdgo_problem *p, int op, const double *blocks,
                  const double *lu, const int *piv, double *x, double *b,
                  double reduction, int maxit, pdgo_result *res);

/* StationaryLinearProblemSolver::apply (linearproblem.hh:188-302):
   r = R(x); z = J^{-1} r (Krylov to max(reduction, min_defect/|r|));
   x -= z.  solver: 0 = CG, 1 = BiCGStab.  op as above. */
int pdgo_solve_linear_problem(const pdgo_problem *p, int solver, int op,
                              double *x, double reduction, double min_defect,
                              int maxit, pdgo_result *res);

/* Matrix-free block preconditioners beyond block Jacobi:
   BlockSORPreconditionerLocalOperator (matrixfree/blocksorpreconditioner.hh)
   and IterativeBlockJacobiPreconditionerLocalOperator
   (matrixfree/iterativeblockjacobipreconditioner.hh). */
typedef struct pdgo_prec_config {
  int kind;                /* block kind: 0 none, 1/2 LU, 3 iterative; | 16 SOR */
  double omega;
  double block_reduction;
  int block_maxit;
  int block_precondition;
  double block_weight;
} pdgo_prec_config;
/* Local dune-istl BiCGStab with point Jacobi on one dense block (row-major);
   returns PDGO_EBREAKDOWN after a breakdown (x holds the last iterate). */
int pdgo_block_bicgstab(int nb, const double *D, int transpose, const double *d, double *x,
                        double red, int maxit, int precond, double weight, int *iterations);
/* v = M^{-1} d; diag: diagonal blocks (row-major), lu/piv: their LU (of the
   transposed blocks when transpose), ablocks: assembled blocks (SOR).
   iters (optional, ncell): block-solve iteration counts. */
int pdgo_prec_apply_cfg(const pdgo_problem *p, const pdgo_prec_config *pc, const double *diag,
                        const double *lu, const int *piv, const double *ablocks, int transpose,
                        const double *d, double *v, int *iters);
int pdgo_solve_linear_problem_prec(const pdgo_problem *p, int solver, int op,
                                   const pdgo_prec_config *pc, double *x, double reduction,
                                   double min_defect, int maxit, pdgo_result *res);

/* NewtonMethod (solver/newton.hh) with DefaultTerminate and the
   Hackbusch-Reusken line search; linear solves by CG (solver 0) or BiCGStab
   (1) with the configured preconditioner, set up at the first
   linearization point and kept.  p->xlin is set during the solve. */
typedef struct pdgo_newton_opts {
  double reduction, absolute_limit;
  int max_iterations, force_iteration;
  double min_linear_reduction;
  int fixed_linear_reduction;
  int line_search, line_search_max_iterations;
  double line_search_damping;
  int line_search_accept_best;
  int linear_maxit;
} pdgo_newton_opts;
typedef struct pdgo_newton_result {
  int converged, iterations;
  double first_defect, defect, reduction, conv_rate;
  int linear_iterations;
  int status;
} pdgo_newton_result;
int pdgo_newton(pdgo_problem *p, int solver, const pdgo_prec_config *pc,
                const pdgo_newton_opts *o, double *x, pdgo_newton_result *res);

/* y = M x: the DG mass matrix int u psi (L2 temporal operator), per cell
   at the volume quadrature points. */
int pdgo_mass_apply(const pdgo_problem *p, const double *x, double *y);
/* OneStepMethod::apply (instationary/implicitonestep.hh:144-275) with the
   one-step residual weights (gridoperator/onestep/prestageengine.hh):
   stage r solves sum_{j<=r} [a_rj M x_j + b_rj dt R(x_j)] = 0; implicit
   stages by residual-form Krylov (CG 0 / BiCGStab 1) with the configured
   preconditioner on J + a_rr/(b_rr dt) M, explicit stages by the per-cell
   mass inverse.  A, B [s][s+1] row-major. */
int pdgo_onestep(pdgo_problem *p, int s, const double *A, const double *B, double dt,
                 int solver, const pdgo_prec_config *pc, double reduction, int maxit,
                 const double *xold, double *xnew, int *linear_iterations);

/* Evaluate u_h at an m-point tensor Gauss rule in every cell:
   xyz [ncell][m^d][dim], w [ncell][m^d] (weights times |J|),
   val [ncell][m^d]. */
int pdgo_eval_points(const pdgo_problem *p, const double *u, int m,
                     double *xyz, double *w, double *val);

/* Gradient of J(u) w.r.t. log K per cell, given primal u and adjoint
   lambda (A^T lambda = dJ/du):  g_e = -lambda^T dR/d(log K_e).
   Built from the assembled local Jacobian blocks with unit coefficients. */
int pdgo_grad_logK(const pdgo_problem *p, const double *u,
                   const double *lam, double *g);
/* Gradient w.r.t. the per-cell constant source fc: g_e = -lambda^T dR/dfc_e */
int pdgo_grad_fc(const pdgo_problem *p, const double *lam, double *g);

#ifdef __cplusplus
}
#endif
#endif
