// matrix_free_linear.cc -- the driver of PDELab's
// dune/pdelab/test/matrixfree/matrix_free_linear.cc (2D Poisson, QkDG degree
// 1 on a 16x16 YaspGrid, SIPG, weightsOn, alpha = 3, Dirichlet data
// g = exp(-|x - 1/2|^2) which is also the exact solution, matrix-free
// BiCGStab with cell-block Jacobi, reduction 1e-12) written against the C++
// adapters of include/pdg/pdelab.hh, running on the GPU.
//
// Prints one JSON line; exit code 0 when the test's own criterion holds
// (L2 error^2 < 1e-6, matrix_free_linear.cc:387-391).
#include <cmath>
#include <cstdio>
#include <vector>

#include "pdg/pdelab.hh"

namespace {

// Lagrange basis of degree k at equidistant nodes, as qkdglagrange.hh:55-62
double lagrange(int k, int i, double x) {
  double r = 1.0;
  for (int j = 0; j <= k; j++)
    if (j != i) r *= (k * x - j) / (i - j);
  return r;
}

double exact(double x, double y) {
  const double c = (0.5 - x) * (0.5 - x) + (0.5 - y) * (0.5 - y);
  return std::exp(-c);
}

}  // namespace

int main(int argc, char **argv) {
  const int cells = argc > 1 ? std::atoi(argv[1]) : 16;
  const int degree = 1;
  pdg::Config cfg(2, degree, cells, cells);
  cfg.alpha = 3.0;   // ConvectionDiffusionDG(problem, SIPG, weightsOn, 3.0)
  try {
    pdg::GridOperator go(cfg);
    long ncell = 0, nbp = 0, ndof = 0;
    int nb = 0, nqv = 0;
    pdg::check(pdg_sizes(go.handle(), &ncell, &nb, &ndof, &nqv, &nbp));
    // source f = 4 (1 - c) g at the operator's volume quadrature points
    std::vector<double> vp((size_t)ncell * nqv * 2), bp((size_t)nbp * 2);
    pdg::check(pdg_volume_points(go.handle(), vp.data()));
    pdg::check(pdg_boundary_points(go.handle(), bp.data()));
    std::vector<double> f((size_t)ncell * nqv), g(nbp);
    for (size_t q = 0; q < f.size(); q++) {
      const double x = vp[2 * q], y = vp[2 * q + 1];
      const double c = (0.5 - x) * (0.5 - x) + (0.5 - y) * (0.5 - y);
      f[q] = 4.0 * (1.0 - c) * std::exp(-c);
    }
    for (long q = 0; q < nbp; q++) g[q] = exact(bp[2 * q], bp[2 * q + 1]);
    go.setSource(f.data(), nullptr);
    go.setBoundaryData(g.data());

    std::vector<double> x(ndof, 0.0);
    pdg::ISTLBackend_SEQ_MatrixFree_Base ls(go, PDG_BICGSTAB, PDG_PREC_BJ_FDM, 5000, 0);
    pdg::StationaryLinearProblemSolver slp(go, ls, pdg::span(x), 1e-12);
    slp.apply();
    const pdg_solver_result &res = slp.result();

    // L2 error^2 with a 6-point Gauss rule per direction (integration order 10)
    const int m = 6;
    const double gx[m] = {0.03376524289842399, 0.16939530676686773, 0.38069040695840156,
                          0.6193095930415985, 0.8306046932331322, 0.966234757101576};
    const double gw[m] = {0.08566224618958518, 0.1803807865240693, 0.23395696728634552,
                          0.23395696728634552, 0.1803807865240693, 0.08566224618958518};
    const double h = 1.0 / cells;
    double err2 = 0.0;
    for (long e = 0; e < ncell; e++) {
      const int ix = (int)(e % cells), iy = (int)(e / cells);
      for (int qy = 0; qy < m; qy++)
        for (int qx = 0; qx < m; qx++) {
          double uh = 0.0;
          for (int i = 0; i < nb; i++)
            uh += x[e * nb + i] * lagrange(degree, i % (degree + 1), gx[qx]) *
                  lagrange(degree, i / (degree + 1), gx[qy]);
          const double d = uh - exact((ix + gx[qx]) * h, (iy + gx[qy]) * h);
          err2 += gw[qx] * gw[qy] * h * h * d * d;
        }
    }
    std::printf("{\"converged\": %d, \"iterations\": %d, \"reduction\": %.3e, "
                "\"l2errorsquared\": %.6e}\n",
                res.converged, res.iterations, res.reduction, err2);
    return (res.converged && err2 < 1e-6) ? 0 : 1;
  } catch (const pdg::Error &e) {
    std::fprintf(stderr, "pdg error %d: %s\n", e.status, e.what());
    return 2;
  }
}
