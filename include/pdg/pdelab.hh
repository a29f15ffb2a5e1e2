// pdg/pdelab.hh -- C++ adapters over the C ABI (include/pdg.h) with the
// names and method signatures of the PDELab / dune-istl interfaces they
// replace, so driver code written against PDELab keeps its shape.
//
//   pdg::GridOperator                    GridOperator::residual / jacobian_apply
//                                        (dune/pdelab/gridoperator/gridoperator.hh:176-205)
//   pdg::OnTheFlyOperator                LinearOperator::apply / applyscaleadd
//                                        (dune/pdelab/backend/istl/seqistlsolverbackend.hh:45-100)
//   pdg::GridOperatorPreconditioner      Preconditioner::pre / apply / post
//                                        (dune/pdelab/backend/istl/matrixfree/gridoperatorpreconditioner.hh:18-91)
//   pdg::ISTLBackend_SEQ_MatrixFree_Base apply(z, r, reduction), norm, result
//                                        (dune/pdelab/backend/istl/matrixfree/backends.hh:62-143)
//   pdg::StationaryLinearProblemSolver   apply, result
//                                        (dune/pdelab/stationary/linearproblem.hh:59-338)
//   pdg::NewtonMethod                    apply, result, set* of the method, its
//                                        DefaultTerminate and line search
//                                        (dune/pdelab/solver/newton.hh:63-669,
//                                        terminate.hh:20-76, linesearch.hh:71-209)
//   pdg::OneStepMethod                   apply(time, dt, xold, xnew), setMethod, result
//                                        (dune/pdelab/instationary/implicitonestep.hh:56-275)
//   pdg::Adjoint                         adjoint solve and gradients (no reference
//                                        counterpart)
//
// Vectors are any contiguous double container with data()/size() (for a
// PDELab ISTL BlockVector of FieldVector<double,n>, pass
// Dune::PDELab::Backend::native(v) through pdg::span(&v[0][0], v.dim())).
// Failures throw pdg::Error (the reference throws Dune::Exception); solver
// non-convergence is reported through result(), as LinearSolverResult does.
// Header-only; link with libpdg.so.
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "../pdg.h"

namespace pdg {

struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string &m) : std::runtime_error(m), status(st) {}
};

inline void check(int st, bool allow_not_converged = false) {
  if (st == PDG_OK) return;
  if (allow_not_converged && st == PDG_ENOTCONVERGED) return;
  throw Error(st, std::string("pdg: ") + pdg_last_error());
}

// non-owning view of contiguous doubles (host or device memory): span for
// vectors a call writes, cspan for vectors it only reads (PDELab's
// `const Domain&` arguments)
struct span {
  double *p;
  std::size_t n;
  span(double *ptr, std::size_t size) : p(ptr), n(size) {}
  template <class V>
  span(V &v) : p(v.data()), n(v.size()) {}
  double *data() const { return p; }
  std::size_t size() const { return n; }
};

struct cspan {
  const double *p;
  std::size_t n;
  cspan(const double *ptr, std::size_t size) : p(ptr), n(size) {}
  template <class V>
  cspan(const V &v) : p(v.data()), n(v.size()) {}
  const double *data() const { return p; }
  std::size_t size() const { return n; }
};

struct Config : pdg_config {
  Config(int dim, int degree, int nx, int ny, int nz = 1) : pdg_config() {
    this->dim = dim;
    this->degree = degree;
    cells[0] = nx;
    cells[1] = ny;
    cells[2] = nz;
    extent[0] = extent[1] = extent[2] = 1.0;
    method = PDG_SIPG;
    weights = PDG_WEIGHTS_ON;
    alpha = 1.0;   // ConvectionDiffusionDG default (convectiondiffusiondg.hh:87-91)
    for (int &b : bctype) b = PDG_BC_DIRICHLET;
    device = 0;
    basis = PDG_BASIS_LAGRANGE;
  }
};

// GridFunctionSpace + ConvectionDiffusionDG + GridOperator on one GPU.
class GridOperator {
 public:
  explicit GridOperator(const pdg_config &cfg) { check(pdg_create(&cfg, &ctx_)); }
  ~GridOperator() { pdg_destroy(ctx_); }
  GridOperator(const GridOperator &) = delete;
  GridOperator &operator=(const GridOperator &) = delete;

  pdg_context *handle() const { return ctx_; }
  long size() const {
    long nd = 0;
    check(pdg_sizes(ctx_, nullptr, nullptr, &nd, nullptr, nullptr));
    return nd;
  }
  long cells() const {
    long nc = 0;
    check(pdg_sizes(ctx_, &nc, nullptr, nullptr, nullptr, nullptr));
    return nc;
  }

  // r += R(x)
  void residual(cspan x, span r) const { check(pdg_residual(ctx_, x.data(), r.data())); }
  // y += J z  (linear problem: the linearization point is not needed)
  void jacobian_apply(cspan z, span y) const {
    check(pdg_jacobian_apply(ctx_, z.data(), y.data()));
  }
  // y += J(x) z  (gridoperator.hh:200-205; sets x as the linearization point)
  void jacobian_apply(cspan x, cspan z, span y) const {
    check(pdg_jacobian_apply_nonlinear(ctx_, x.data(), z.data(), y.data()));
  }
  // y += J^T z  (the adjoint's operator; no reference counterpart)
  void jacobian_apply_transpose(cspan z, span y) const {
    check(pdg_jacobian_apply_transpose(ctx_, z.data(), y.data()));
  }
  // y = M x with the DG mass matrix (the L2 temporal operator, localoperator/l2.hh)
  void mass_apply(cspan x, span y) const { check(pdg_mass_apply(ctx_, x.data(), y.data())); }

  // GridOperator::jacobian(x, A) (gridoperator.hh:184-189) into an ISTL-shaped
  // BCRS matrix: block rows in cell order, column blocks ascending, each
  // block block x block, row-major
  struct BCRSMatrix {
    long rows = 0;
    int block = 0;
    std::vector<long> rowptr, colind;
    std::vector<double> values;
  };
  void jacobian(BCRSMatrix &A) const {
    long nc = 0, nnz = 0;
    int nb = 0;
    check(pdg_sizes(ctx_, &nc, &nb, nullptr, nullptr, nullptr));
    check(pdg_jacobian_assemble(ctx_));
    check(pdg_jacobian_pattern(ctx_, &nnz));
    A.rows = nc;
    A.block = nb;
    A.rowptr.assign(nc + 1, 0);
    A.colind.assign(nnz, 0);
    A.values.assign((std::size_t)nnz * nb * nb, 0.0);
    check(pdg_jacobian_export(ctx_, A.rowptr.data(), A.colind.data(), A.values.data()));
  }

  void setPermeability(const std::vector<double> &K, bool is_log = false) {
    check(pdg_set_permeability(ctx_, K.data(), is_log ? 1 : 0));
  }
  // c per cell (an empty vector: c = 0)
  void setReaction(const std::vector<double> &c) {
    check(pdg_set_reaction(ctx_, c.empty() ? nullptr : c.data()));
  }
  // b(x) as Fourier modes [n][7] = kx ky kz phase cx cy cz (empty: b = 0)
  void setVelocityModes(const std::vector<double> &modes) {
    check(pdg_set_velocity_modes(ctx_, (int)(modes.size() / 7),
                                 modes.empty() ? nullptr : modes.data()));
  }
  // the nonlinear volume term q(u) = sum_m coef[m] u^m of
  // NonlinearConvectionDiffusionDG (coef.size() - 1 = degree, 1..4; empty
  // removes it)
  void setNonlinearity(const std::vector<double> &coef) {
    check(pdg_set_nonlinearity(ctx_, coef.empty() ? 0 : (int)coef.size() - 1,
                               coef.empty() ? nullptr : coef.data()));
  }
  // A(cell, x) beyond K I: a dim x dim tensor per cell (row-major), or per
  // quadrature point when the parameter class's permeabilityIsConstantPerCell()
  // is false (convectiondiffusionparameter.hh:143-157)
  void setPermeabilityTensor(const std::vector<double> &A) {
    check(pdg_set_permeability_tensor(ctx_, A.data()));
  }
  void setPermeabilityPoints(const std::vector<double> &Avol, const std::vector<double> &Aface) {
    check(pdg_set_permeability_points(ctx_, Avol.data(), Aface.data()));
  }
  // c(cell, x) at the volume points, b(cell, x) at the volume and face-lattice points
  void setReactionPoints(const std::vector<double> &cq) {
    check(pdg_set_reaction_points(ctx_, cq.data()));
  }
  void setVelocityPoints(const std::vector<double> &bvol, const std::vector<double> &bface) {
    check(pdg_set_velocity_points(ctx_, bvol.data(), bface.data()));
  }
  // PDG_F64_NATIVE or PDG_F64_FLOAT_PAIR (no reference counterpart)
  void setF64Arithmetic(int mode) { check(pdg_set_f64_arithmetic(ctx_, mode)); }
  void setSource(const double *fq, const double *fc) { check(pdg_set_source(ctx_, fq, fc)); }
  void setBoundaryData(const double *g, const double *j = nullptr, const double *o = nullptr) {
    check(pdg_set_boundary_data(ctx_, g, j, o));
  }

 private:
  pdg_context *ctx_ = nullptr;
};

// Dune::LinearOperator over GridOperator::jacobian_apply
class OnTheFlyOperator {
 public:
  explicit OnTheFlyOperator(const GridOperator &go) : go_(go) {}
  void apply(cspan x, span y) const { check(pdg_apply(go_.handle(), x.data(), y.data())); }
  void applyscaleadd(double alpha, cspan x, span y) const {
    check(pdg_applyscaleadd(go_.handle(), alpha, x.data(), y.data()));
  }
  // backends.hh:129-135
  void setLinearizationPoint(cspan x) {
    check(pdg_set_linearization_point(go_.handle(), x.data()));
  }

 private:
  const GridOperator &go_;
};

// Dune::Preconditioner over the cell-block Jacobi of the operator
class GridOperatorPreconditioner {
 public:
  explicit GridOperatorPreconditioner(const GridOperator &go, int kind = PDG_PREC_BJ_FDM,
                                      int precision = PDG_F64)
      : go_(go), kind_(kind), precision_(precision) {}
  void pre(span, span) {
    if (!ready_) {
      check(pdg_prec_setup(go_.handle(), kind_, precision_));
      ready_ = true;
    }
  }
  void apply(span v, cspan d) { check(pdg_prec_apply(go_.handle(), d.data(), v.data())); }
  void post(span) {}
  // gridoperatorpreconditioner.hh:38-42: the blocks are rebuilt at the new point
  void setLinearizationPoint(cspan x) {
    check(pdg_set_linearization_point(go_.handle(), x.data()));
    ready_ = false;
  }

 private:
  const GridOperator &go_;
  int kind_, precision_;
  bool ready_ = false;
};

// Sequential matrix-free Krylov backend: apply(z, r, reduction) solves J z = r
class ISTLBackend_SEQ_MatrixFree_Base {
 public:
  static constexpr bool isMatrixFree = true;
  ISTLBackend_SEQ_MatrixFree_Base(const GridOperator &go, int method = PDG_CG,
                                  int preconditioner = PDG_PREC_BJ_FDM, unsigned maxiter = 5000,
                                  int verbose = 0)
      : go_(go) {
    pdg_default_solver_options(&opt_);
    opt_.method = method;
    opt_.preconditioner = preconditioner;
    opt_.maxit = (int)maxiter;
    opt_.verbose = verbose;
  }
  void setMixedPrecision(bool on, double inner_reduction = 1e-3) {
    // inner FP32 Krylov solves inside FP64 defect correction
    opt_.mixed = on ? 1 : 0;
    opt_.inner_reduction = inner_reduction;
  }
  void apply(span z, span r, double reduction) {
    opt_.reduction = reduction;
    check(pdg_krylov_solve(go_.handle(), &opt_, z.data(), r.data(), &res_), true);
  }
  double norm(cspan v) const {
    double out = 0.0;
    check(pdg_norm(go_.handle(), v.data(), &out));
    return out;
  }
  const pdg_solver_result &result() const { return res_; }
  pdg_solver_options &options() { return opt_; }

 private:
  const GridOperator &go_;
  pdg_solver_options opt_;
  pdg_solver_result res_{};
};

// r = R(x); J z = r; x -= z
class StationaryLinearProblemSolver {
 public:
  StationaryLinearProblemSolver(const GridOperator &go, ISTLBackend_SEQ_MatrixFree_Base &ls,
                                span x, double reduction, double min_defect = 1e-99)
      : go_(go), ls_(ls), x_(x), reduction_(reduction), min_defect_(min_defect) {}
  void apply() {
    pdg_solver_options o = ls_.options();
    o.reduction = reduction_;
    o.min_defect = min_defect_;
    check(pdg_solve_linear_problem(go_.handle(), &o, x_.data(), &res_), true);
  }
  const pdg_solver_result &result() const { return res_; }

 private:
  const GridOperator &go_;
  ISTLBackend_SEQ_MatrixFree_Base &ls_;
  span x_;
  double reduction_, min_defect_;
  pdg_solver_result res_{};
};

// NewtonMethod<GridOperator, LinearSolver>: apply(u) solves R(u) = 0 from the
// initial guess in u.  Reaching the iteration limit throws, as the reference's
// DefaultTerminate does (TerminateError); a failed line search throws with
// PDG_ELINESEARCH (LineSearchError).
class NewtonMethod {
 public:
  NewtonMethod(const GridOperator &go, ISTLBackend_SEQ_MatrixFree_Base &ls) : go_(go), ls_(ls) {
    pdg_default_newton_options(&opt_);
  }
  void apply(span u) {
    check(pdg_newton_solve(go_.handle(), &opt_, &ls_.options(), u.data(), &res_));
  }
  const pdg_newton_result &result() const { return res_; }

  void setVerbosityLevel(unsigned v) { opt_.verbose = (int)v; }
  void setReduction(double r) { opt_.reduction = r; }
  void setAbsoluteLimit(double a) { opt_.absolute_limit = a; }
  void setMinLinearReduction(double r) { opt_.min_linear_reduction = r; }
  void setFixedLinearReduction(bool b) { opt_.fixed_linear_reduction = b ? 1 : 0; }
  // DefaultTerminate (terminate.hh:20-76)
  void setMaxIterations(unsigned n) { opt_.max_iterations = (int)n; }
  void setForceIteration(bool b) { opt_.force_iteration = b ? 1 : 0; }
  // line search: Hackbusch-Reusken (true) or full Newton steps (false),
  // HackbuschReuskenLineSearch's settings (linesearch.hh:71-209)
  void setLineSearch(bool hackbusch_reusken) { opt_.line_search = hackbusch_reusken ? 1 : 0; }
  void setLineSearchMaxIterations(unsigned n) { opt_.line_search_max_iterations = (int)n; }
  void setLineSearchDampingFactor(double d) { opt_.line_search_damping = d; }
  void setLineSearchAcceptBest(bool b) { opt_.line_search_accept_best = b ? 1 : 0; }
  pdg_newton_options &options() { return opt_; }

 private:
  const GridOperator &go_;
  ISTLBackend_SEQ_MatrixFree_Base &ls_;
  pdg_newton_options opt_;
  pdg_newton_result res_{};
};

// OneStepMethod with one of the TimeSteppingParameterInterface methods
// (PDG_ONESTEP_*, instationary/onestepparameter.hh); the spatial data are
// time-independent, so `time` only labels the step
class OneStepMethod {
 public:
  OneStepMethod(const GridOperator &go, ISTLBackend_SEQ_MatrixFree_Base &ls, int method,
                double theta = 1.0)
      : go_(go), ls_(ls) {
    setMethod(method, theta);
  }
  void setMethod(int method, double theta = 1.0) {
    check(pdg_onestep_table(method, theta, &stages_, A_, B_, D_));
  }
  // implicitonestep.hh:144: xnew holds the initial guess on entry; returns dt
  double apply(double /*time*/, double dt, cspan xold, span xnew) {
    check(pdg_onestep_apply(go_.handle(), stages_, A_, B_, D_, dt, &ls_.options(), xold.data(),
                            xnew.data(), &res_));
    return dt;
  }
  const pdg_onestep_result &result() const { return res_; }

 private:
  const GridOperator &go_;
  ISTLBackend_SEQ_MatrixFree_Base &ls_;
  int stages_ = 0;
  double A_[20] = {}, B_[20] = {}, D_[5] = {};
  pdg_onestep_result res_{};
};

// Adjoint solve J^T lambda = rhs and the fused gradients dJ/dlog K and
// dJ/d(per-cell source) from the primal u and the adjoint lambda (no
// reference counterpart).  Non-convergence is reported through result().
class Adjoint {
 public:
  Adjoint(const GridOperator &go, ISTLBackend_SEQ_MatrixFree_Base &ls) : go_(go), ls_(ls) {}
  void solve(cspan rhs, span lambda, double reduction) {
    pdg_solver_options o = ls_.options();
    o.reduction = reduction;
    check(pdg_adjoint_solve(go_.handle(), &o, rhs.data(), lambda.data(), &res_), true);
  }
  void gradLogK(cspan u, cspan lambda, span g) const {
    check(pdg_grad_logK(go_.handle(), u.data(), lambda.data(), g.data()));
  }
  void gradSource(cspan lambda, span g) const {
    check(pdg_grad_source(go_.handle(), lambda.data(), g.data()));
  }
  const pdg_solver_result &result() const { return res_; }

 private:
  const GridOperator &go_;
  ISTLBackend_SEQ_MatrixFree_Base &ls_;
  pdg_solver_result res_{};
};

}  // namespace pdg
