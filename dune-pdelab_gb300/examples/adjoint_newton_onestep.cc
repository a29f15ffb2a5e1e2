// adjoint_newton_onestep.cc -- the adjoint, assembled-matrix, Newton and
// one-step adapters of include/pdg/pdelab.hh driven from C++ on the GPU
// (host vectors; the library stages them), each checked against an identity
// that needs no reference data:
//
//   adjoint   3D Q2 6^3, J = 1/2 |u - u_obs|^2 with u the SIPG solution:
//             g . d from Adjoint::gradLogK / gradSource against central
//             differences of J along a seeded direction (h = 1e-6)
//   jacobian  3D Q2 4^3, NIPG with reaction: the exported BCRS matrix times x
//             against jacobian_apply, its transpose against
//             jacobian_apply_transpose (the operator is not symmetric)
//   newton    3D Q1 6^3, q(u) = u + u^3, f = 5: NewtonMethod to 1e-10, then
//             |R(u)| against the first defect
//   onestep   3D Q2 4^3, implicit Euler: |M (x1 - x0) + dt R(x1)| against
//             |M x1|
//
// Prints one JSON line; exit code 0 when every check holds.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "pdg/pdelab.hh"

namespace {

// seeded uniform numbers in [-1, 1) (64-bit LCG, top 53 bits)
struct Rng {
  std::uint64_t s;
  explicit Rng(std::uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 1) {}
  double operator()() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(s >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
  std::vector<double> vec(long n) {
    std::vector<double> v(n);
    for (double &x : v) x = (*this)();
    return v;
  }
};

double dot(const std::vector<double> &a, const std::vector<double> &b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}

double maxabs(const std::vector<double> &a) {
  double m = 0.0;
  for (double x : a) m = std::fmax(m, std::fabs(x));
  return m;
}

double maxdiff(const std::vector<double> &a, const std::vector<double> &b) {
  double m = 0.0;
  for (size_t i = 0; i < a.size(); i++) m = std::fmax(m, std::fabs(a[i] - b[i]));
  return m;
}

// relative error of the adjoint directional derivative against central
// differences, for log K and for the per-cell source
void adjoint_check(double *err_logK, double *err_source) {
  pdg::Config cfg(3, 2, 6, 6, 6);
  cfg.alpha = 3.0;
  pdg::GridOperator go(cfg);
  const long nd = go.size(), nc = go.cells();
  Rng rng(7);
  std::vector<double> fc(nc, 1.0);
  go.setSource(nullptr, fc.data());
  pdg::ISTLBackend_SEQ_MatrixFree_Base ls(go, PDG_CG, PDG_PREC_BJ_FDM, 5000, 0);
  auto solve = [&](const std::vector<double> &logK, const std::vector<double> &f) {
    go.setPermeability(logK, true);
    go.setSource(nullptr, f.data());
    std::vector<double> u(nd, 0.0);
    pdg::StationaryLinearProblemSolver slp(go, ls, pdg::span(u), 1e-13);
    slp.apply();
    if (!slp.result().converged) throw pdg::Error(PDG_ENOTCONVERGED, "forward solve");
    return u;
  };
  std::vector<double> u_obs = solve(rng.vec(nc), fc);
  for (double &v : u_obs) v *= 1.0 + 0.01 * rng();
  auto loss = [&](const std::vector<double> &logK, const std::vector<double> &f) {
    const std::vector<double> u = solve(logK, f);
    double s = 0.0;
    for (long i = 0; i < nd; i++) s += 0.5 * (u[i] - u_obs[i]) * (u[i] - u_obs[i]);
    return s;
  };
  const std::vector<double> logK = rng.vec(nc);
  std::vector<double> u = solve(logK, fc);
  std::vector<double> rhs(nd), lambda(nd, 0.0), g(nc, 0.0), gf(nc, 0.0);
  for (long i = 0; i < nd; i++) rhs[i] = u[i] - u_obs[i];
  pdg::Adjoint adj(go, ls);
  adj.solve(rhs, lambda, 1e-13);
  if (!adj.result().converged) throw pdg::Error(PDG_ENOTCONVERGED, "adjoint solve");
  adj.gradLogK(u, lambda, g);
  adj.gradSource(lambda, gf);
  const double h = 1e-6;
  const std::vector<double> d = rng.vec(nc);
  std::vector<double> kp(logK), km(logK), fp(fc), fm(fc);
  for (long e = 0; e < nc; e++) {
    kp[e] += h * d[e];
    km[e] -= h * d[e];
    fp[e] += h * d[e];
    fm[e] -= h * d[e];
  }
  const double fd = (loss(kp, fc) - loss(km, fc)) / (2 * h);
  const double fdf = (loss(logK, fp) - loss(logK, fm)) / (2 * h);
  *err_logK = std::fabs(fd - dot(g, d)) / std::fabs(dot(g, d));
  *err_source = std::fabs(fdf - dot(gf, d)) / std::fabs(dot(gf, d));
}

// relative errors of A x and A^T x from the exported matrix, and the relative
// difference between J x and J^T x (nonzero: NIPG is not symmetric)
void jacobian_check(double *err, double *err_t, double *asym) {
  pdg::Config cfg(3, 2, 4, 4, 4);
  cfg.alpha = 3.0;
  cfg.method = PDG_NIPG;
  pdg::GridOperator go(cfg);
  const long nd = go.size(), nc = go.cells();
  Rng rng(11);
  go.setPermeability(rng.vec(nc), true);
  std::vector<double> c = rng.vec(nc);
  for (double &v : c) v = 1.0 + 0.5 * v;
  go.setReaction(c);
  pdg::GridOperator::BCRSMatrix A;
  go.jacobian(A);
  std::vector<double> x = rng.vec(nd);
  std::vector<double> y(nd, 0.0), yt(nd, 0.0), ya(nd, 0.0), yat(nd, 0.0);
  go.jacobian_apply(x, y);
  go.jacobian_apply_transpose(x, yt);
  const int b = A.block;
  for (long r = 0; r < A.rows; r++)
    for (long p = A.rowptr[r]; p < A.rowptr[r + 1]; p++) {
      const long cb = A.colind[p];
      const double *v = A.values.data() + (size_t)p * b * b;
      for (int i = 0; i < b; i++)
        for (int j = 0; j < b; j++) {
          ya[r * b + i] += v[i * b + j] * x[cb * b + j];
          yat[cb * b + j] += v[i * b + j] * x[r * b + i];
        }
    }
  *err = maxdiff(y, ya) / maxabs(y);
  *err_t = maxdiff(yt, yat) / maxabs(yt);
  *asym = maxdiff(y, yt) / maxabs(y);
}

// Newton on -div(K grad u) + u + u^3 = 5; returns |R(u)| / first defect
double newton_check(int *iterations, int *converged) {
  pdg::Config cfg(3, 1, 6, 6, 6);
  cfg.alpha = 3.0;
  pdg::GridOperator go(cfg);
  const long nd = go.size(), nc = go.cells();
  Rng rng(13);
  std::vector<double> logK = rng.vec(nc);
  for (double &v : logK) v *= 0.5;
  go.setPermeability(logK, true);
  go.setNonlinearity({0.0, 1.0, 0.0, 1.0});
  std::vector<double> f(nc, 5.0);
  go.setSource(nullptr, f.data());
  pdg::ISTLBackend_SEQ_MatrixFree_Base ls(go, PDG_BICGSTAB, PDG_PREC_BJ_DENSE, 5000, 0);
  pdg::NewtonMethod newton(go, ls);
  newton.setReduction(1e-10);
  std::vector<double> u(nd, 0.0);
  newton.apply(u);
  *iterations = newton.result().iterations;
  *converged = newton.result().converged;
  std::vector<double> r(nd, 0.0);
  go.residual(u, r);
  return ls.norm(r) / newton.result().first_defect;
}

// implicit Euler step: |M (x1 - x0) + dt R(x1)| / |M x1|
double onestep_check() {
  pdg::Config cfg(3, 2, 4, 4, 4);
  cfg.alpha = 3.0;
  pdg::GridOperator go(cfg);
  const long nd = go.size(), nc = go.cells();
  Rng rng(17);
  go.setPermeability(rng.vec(nc), true);
  std::vector<double> f(nc, 1.0);
  go.setSource(nullptr, f.data());
  pdg::ISTLBackend_SEQ_MatrixFree_Base ls(go, PDG_CG, PDG_PREC_BJ_FDM, 5000, 0);
  ls.options().reduction = 1e-13;
  pdg::OneStepMethod osm(go, ls, PDG_ONESTEP_IMPLICIT_EULER);
  const double dt = 1e-2;
  std::vector<double> x0 = rng.vec(nd);
  std::vector<double> x1(nd, 0.0), dx(nd), m(nd, 0.0), mx1(nd, 0.0), r(nd, 0.0);
  osm.apply(0.0, dt, x0, x1);
  for (long i = 0; i < nd; i++) dx[i] = x1[i] - x0[i];
  go.mass_apply(dx, m);
  go.mass_apply(x1, mx1);
  go.residual(x1, r);
  for (long i = 0; i < nd; i++) m[i] += dt * r[i];
  return maxabs(m) / maxabs(mx1);
}

}  // namespace

int main() {
  try {
    double e_k = 0, e_f = 0, e_a = 0, e_at = 0, asym = 0;
    adjoint_check(&e_k, &e_f);
    jacobian_check(&e_a, &e_at, &asym);
    int nit = 0, nconv = 0;
    const double nres = newton_check(&nit, &nconv);
    const double ores = onestep_check();
    std::printf("{\"adjoint_fd_rel_logK\": %.3e, \"adjoint_fd_rel_source\": %.3e, "
                "\"bcrs_rel\": %.3e, \"bcrs_transpose_rel\": %.3e, \"nipg_asymmetry\": %.3e, "
                "\"newton_converged\": %d, \"newton_iterations\": %d, "
                "\"newton_residual_rel\": %.3e, \"implicit_euler_rel\": %.3e}\n",
                e_k, e_f, e_a, e_at, asym, nconv, nit, nres, ores);
    const bool ok = e_k < 1e-5 && e_f < 1e-5 && e_a < 1e-12 && e_at < 1e-12 && asym > 1e-6 &&
                    nconv && nres < 1e-9 && ores < 1e-10;
    return ok ? 0 : 1;
  } catch (const pdg::Error &e) {
    std::fprintf(stderr, "pdg error %d: %s\n", e.status, e.what());
    return 2;
  }
}
