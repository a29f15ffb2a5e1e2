/*
 * pdg_oracle.c -- CPU restatement of PDELab's ConvectionDiffusionDG
 * matrix-free path.  TEST INFRASTRUCTURE ONLY (see pdg_oracle.h).
 *
 * Each routine cites the reference file:line it restates.  Paths are
 * relative to the dune-pdelab source tree (dune/pdelab/...).
 *
 * Third-party arithmetic that is not part of dune-pdelab and is restated
 * here from its published algorithm:
 *   - dune-geometry (>= 2.10) QuadratureRules, Gauss-Legendre: nodes are
 *     the roots of P_m found by Newton iteration, weights 2/((1-x^2)P'_m^2)
 *     (Abramowitz & Stegun 25.4.29), mapped to [0,1].  Order 2k selects
 *     m = k+1 points per direction.
 *   - dune-istl (>= 2.10) CGSolver / BiCGSTABSolver: preconditioned CG
 *     (Hestenes & Stiefel 1952) and BiCGStab (van der Vorst 1992) in the
 *     form dune-istl uses (defect-based, reduction relative to the
 *     initial defect two-norm, half-step iteration count for BiCGStab).
 *   - Eigen PartialPivLU: LU with row partial pivoting (max |a_ij| in
 *     the column).
 *   - dune-grid YaspGrid: axis-parallel cells, lexicographic leaf index
 *     with x fastest, intersections ordered -x,+x,-y,+y,-z,+z.
 */
#include "pdg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXD 3
#define MAXK 6
#define MAXN1 (MAXK + 1)
#define MAXNB (MAXN1 * MAXN1 * MAXN1)

/* ------------------------------------------------------------------ */
/* 1D building blocks                                                  */
/* ------------------------------------------------------------------ */

/* QkStuff::p  (finiteelement/qkdglagrange.hh:55-62) */
double pdgo_lagrange(int k, int i, double x) {
  double result = 1.0;
  for (int j = 0; j <= k; j++)
    if (j != i) result *= (k * x - j) / (i - j);
  return result;
}

/* QkStuff::dp  (finiteelement/qkdglagrange.hh:65-79) */
double pdgo_dlagrange(int k, int i, double x) {
  double result = 0.0;
  for (int j = 0; j <= k; j++)
    if (j != i) {
      double prod = (k * 1.0) / (i - j);
      for (int l = 0; l <= k; l++)
        if (l != i && l != j) prod *= (k * x - l) / (i - l);
      result += prod;
    }
  return result;
}

/* Gauss-Lobatto rule with m >= 2 points on [0,1], ascending (the rule the
   Lobatto basis takes its nodes from, qkdglobatto.hh:27-67; dune-geometry's
   QuadratureType::GaussLobatto, restated): the end points and the roots of
   P'_{m-1}, found by Newton iteration on P'_n with P''_n from Legendre's
   equation (1-z^2) P''_n = 2 z P'_n - n(n+1) P_n, started at the
   Chebyshev-Gauss-Lobatto points cos(pi j/n); weights 2/(n(n+1) P_n(z)^2)
   on [-1,1] (Abramowitz & Stegun 25.4.32), halved on [0,1]. */
static void legendre_pn(int n, long double z, long double *pn, long double *pn1) {
  long double p0 = 1.0L, p1 = 0.0L;
  for (int j = 1; j <= n; j++) {
    long double p2 = p1;
    p1 = p0;
    p0 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p2) / j;
  }
  *pn = p0;
  *pn1 = p1;
}

int pdgo_gauss_lobatto(int m, double *x, double *w) {
  if (m < 2 || m > 32) return PDGO_EARG;
  const int n = m - 1;
  const long double pi = 3.14159265358979323846264338327950288L;
  for (int j = 0; j <= n; j++) {
    long double z = cosl(pi * j / n);
    if (j > 0 && j < n) {
      for (int it = 0; it < 100; it++) {
        long double pn, pn1;
        legendre_pn(n, z, &pn, &pn1);
        const long double dp = n * (pn1 - z * pn) / (1.0L - z * z);
        const long double d2 = (2.0L * z * dp - n * (n + 1.0L) * pn) / (1.0L - z * z);
        const long double dz = dp / d2;
        z -= dz;
        if (fabsl(dz) < 1e-19L) break;
      }
    }
    long double pn, pn1;
    legendre_pn(n, z, &pn, &pn1);
    x[j] = (double)((1.0L - z) * 0.5L);
    w[j] = (double)(1.0L / (n * (n + 1.0L) * pn * pn));
  }
  return PDGO_OK;
}

/* DGLegendreLocalBasis 1D factor (qkdglegendre.hh:80-113): Legendre
   polynomials on [0,1], P_0 = 1, P_1 = 2x-1,
   P_n = ((2n-1)(2x-1) P_{n-1} - (n-1) P_{n-2}) / n,
   P'_n = (2x-1) P'_{n-1} + 2n P_{n-1}. */
static void legendre01(int k, double x, double *v, double *dv) {
  v[0] = 1.0;
  dv[0] = 0.0;
  if (k >= 1) {
    v[1] = 2 * x - 1;
    dv[1] = 2.0;
  }
  for (int n = 2; n <= k; n++) {
    v[n] = ((2 * n - 1) * (2 * x - 1) * v[n - 1] - (n - 1) * v[n - 2]) / n;
    dv[n] = (2 * x - 1) * dv[n - 1] + 2 * n * v[n - 1];
  }
}

/* GaussLobattoLagrangePolynomials (qkdglobatto.hh:21-117): Lagrange
   polynomials on the k+1 Gauss-Lobatto points, ascending. */
static const double *lobatto_nodes(int k) {
  static double nodes[MAXK + 1][MAXN1];
  static int ready[MAXK + 1];
  if (!ready[k]) {
    double w[MAXN1];
    pdgo_gauss_lobatto(k + 1, nodes[k], w);
    ready[k] = 1;
  }
  return nodes[k];
}

double pdgo_basis1d(int basis, int k, int i, double x) {
  if (basis == PDGO_LEGENDRE) {
    double v[MAXN1], dv[MAXN1];
    legendre01(k, x, v, dv);
    return v[i];
  }
  if (basis == PDGO_LOBATTO) {
    const double *xi = lobatto_nodes(k);
    double r = 1.0;
    for (int j = 0; j <= k; j++)
      if (j != i) r *= (x - xi[j]) / (xi[i] - xi[j]);
    return r;
  }
  return pdgo_lagrange(k, i, x);
}

double pdgo_dbasis1d(int basis, int k, int i, double x) {
  if (basis == PDGO_LEGENDRE) {
    double v[MAXN1], dv[MAXN1];
    legendre01(k, x, v, dv);
    return dv[i];
  }
  if (basis == PDGO_LOBATTO) {
    const double *xi = lobatto_nodes(k);
    double r = 0.0;
    for (int j = 0; j <= k; j++)
      if (j != i) {
        double prod = 1.0 / (xi[i] - xi[j]);
        for (int l = 0; l <= k; l++)
          if (l != i && l != j) prod *= (x - xi[l]) / (xi[i] - xi[l]);
        r += prod;
      }
    return r;
  }
  return pdgo_dlagrange(k, i, x);
}

/* Gauss-Legendre rule with m points on [0,1] (dune-geometry's default
   QuadratureType::GaussLegendre, selected by quadratureRule() at
   common/quadraturerules.hh:110-120).  Newton on P_m in long double. */
int pdgo_gauss_legendre(int m, double *x, double *w) {
  if (m < 1 || m > 32) return PDGO_EARG;
  for (int i = 0; i < m; i++) {
    long double z = cosl(3.14159265358979323846264338327950288L * (i + 0.75L) / (m + 0.5L));
    long double dp = 0;
    for (int it = 0; it < 100; it++) {
      long double p0 = 1.0L, p1 = 0.0L;
      for (int j = 1; j <= m; j++) {
        long double p2 = p1;
        p1 = p0;
        p0 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p2) / j;
      }
      dp = m * (z * p0 - p1) / (z * z - 1.0L);
      long double dz = p0 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-19L) break;
    }
    /* recompute derivative at the converged root */
    {
      long double p0 = 1.0L, p1 = 0.0L;
      for (int j = 1; j <= m; j++) {
        long double p2 = p1;
        p1 = p0;
        p0 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p2) / j;
      }
      dp = m * (z * p0 - p1) / (z * z - 1.0L);
    }
    /* roots z descend with i, so (1 - z)/2 ascends on [0,1] */
    x[i] = (double)((1.0L - z) * 0.5L);
    w[i] = (double)(1.0L / ((1.0L - z * z) * dp * dp));
  }
  return PDGO_OK;
}

/* ------------------------------------------------------------------ */
/* geometry and tables                                                 */
/* ------------------------------------------------------------------ */

typedef struct tables {
  int d, k, n1, nb, nq, nqv, nqf;
  double gx[MAXN1], gw[MAXN1];
  /* volume points: phi [nqv][nb], js [nqv][nb][d], weight [nqv], local [nqv][d] */
  double *vphi, *vjs, *vw, *vloc;
  /* face points for face f = 2*dir+hi: phi [2d][nqf][nb], js, weight, local,
     face-local coordinates mapped into the cell */
  double *fphi, *fjs, *fw, *floc;
  double theta;
} tables;

static int get_theta(int method, double *theta) {
  /* convectiondiffusiondg.hh:99-101 */
  if (method == PDGO_NIPG) *theta = 1.0;
  else if (method == PDGO_SIPG) *theta = -1.0;
  else if (method == PDGO_IIPG) *theta = 0.0;
  else return PDGO_EARG;
  return PDGO_OK;
}

/* QkLocalBasis::evaluateFunction / evaluateJacobian
   (qkdglagrange.hh:153-198) with multiindex (qkdglagrange.hh:118-128);
   DGLegendreLocalBasis (qkdglegendre.hh:236-328, same multiindex,
   :63-73) and QkGLLocalBasis (qkdglobatto.hh:130-220) have the same tensor
   structure with other 1D factors. */
static void eval_basis(int basis, int d, int k, const double *xi, double *phi, double *js) {
  int n1 = k + 1, nb = 1;
  for (int j = 0; j < d; j++) nb *= n1;
  for (int i = 0; i < nb; i++) {
    int alpha[MAXD], t = i;
    for (int j = 0; j < d; j++) { alpha[j] = t % n1; t /= n1; }
    double v = 1.0;
    for (int j = 0; j < d; j++) v *= pdgo_basis1d(basis, k, alpha[j], xi[j]);
    phi[i] = v;
    for (int j = 0; j < d; j++) {
      double g = pdgo_dbasis1d(basis, k, alpha[j], xi[j]);
      for (int l = 0; l < d; l++)
        if (l != j) g *= pdgo_basis1d(basis, k, alpha[l], xi[l]);
      js[i * d + j] = g;
    }
  }
}

static int tables_init(const pdgo_problem *p, tables *T) {
  memset(T, 0, sizeof(*T));
  if (p->dim < 2 || p->dim > 3 || p->k < 1 || p->k > MAXK) return PDGO_EARG;
  for (int j = 0; j < p->dim; j++)
    if (p->nc[j] < 1 || !(p->L[j] > 0)) return PDGO_EARG;
  if (get_theta(p->method, &T->theta)) return PDGO_EARG;
  int d = T->d = p->dim;
  int k = T->k = p->k;
  int n1 = T->n1 = k + 1;
  T->nb = 1;
  for (int j = 0; j < d; j++) T->nb *= n1;
  /* intorder = quadrature_factor * order = 2k (convectiondiffusiondg.hh:139,
     360, 745, 1061) -> m = k+1 Gauss points per direction */
  int nq = T->nq = k + 1;
  pdgo_gauss_legendre(nq, T->gx, T->gw);
  T->nqv = 1; T->nqf = 1;
  for (int j = 0; j < d; j++) T->nqv *= nq;
  for (int j = 0; j < d - 1; j++) T->nqf *= nq;
  int nb = T->nb, nqv = T->nqv, nqf = T->nqf;
  T->vphi = malloc(sizeof(double) * nqv * nb);
  T->vjs = malloc(sizeof(double) * nqv * nb * d);
  T->vw = malloc(sizeof(double) * nqv);
  T->vloc = malloc(sizeof(double) * nqv * d);
  T->fphi = malloc(sizeof(double) * 2 * d * nqf * nb);
  T->fjs = malloc(sizeof(double) * 2 * d * nqf * nb * d);
  T->fw = malloc(sizeof(double) * 2 * d * nqf);
  T->floc = malloc(sizeof(double) * 2 * d * nqf * d);
  for (int q = 0; q < nqv; q++) {
    int t = q;
    double w = 1.0;
    for (int j = 0; j < d; j++) {
      int a = t % nq; t /= nq;
      T->vloc[q * d + j] = T->gx[a];
      w *= T->gw[a];
    }
    T->vw[q] = w;
    eval_basis(p->basis, d, k, &T->vloc[q * d], &T->vphi[q * nb], &T->vjs[q * nb * d]);
  }
  for (int f = 0; f < 2 * d; f++) {
    int dir = f / 2, hi = f % 2;
    for (int q = 0; q < nqf; q++) {
      int t = q;
      double w = 1.0;
      double *loc = &T->floc[(f * nqf + q) * d];
      /* face-local coordinates map to the remaining directions in order */
      for (int j = 0; j < d; j++) {
        if (j == dir) { loc[j] = hi ? 1.0 : 0.0; continue; }
        int a = t % nq; t /= nq;
        loc[j] = T->gx[a];
        w *= T->gw[a];
      }
      T->fw[f * nqf + q] = w;
      eval_basis(p->basis, d, k, loc, &T->fphi[(f * nqf + q) * nb], &T->fjs[(f * nqf + q) * nb * d]);
    }
  }
  return PDGO_OK;
}

static void tables_free(tables *T) {
  free(T->vphi); free(T->vjs); free(T->vw); free(T->vloc);
  free(T->fphi); free(T->fjs); free(T->fw); free(T->floc);
}

long pdgo_ncell(const pdgo_problem *p) {
  long n = 1;
  for (int j = 0; j < p->dim; j++) n *= p->nc[j];
  return n;
}
int pdgo_nbasis(const pdgo_problem *p) {
  int n = 1;
  for (int j = 0; j < p->dim; j++) n *= p->k + 1;
  return n;
}
long pdgo_ndof(const pdgo_problem *p) { return pdgo_ncell(p) * pdgo_nbasis(p); }

long pdgo_nbpts_side(const pdgo_problem *p, int side) {
  int dir = side / 2;
  long n = 1;
  for (int j = 0; j < p->dim; j++)
    if (j != dir) n *= (long)p->nc[j] * (p->k + 1);
  return n;
}
long pdgo_bpts_offset(const pdgo_problem *p, int side) {
  long off = 0;
  for (int s = 0; s < side; s++) off += pdgo_nbpts_side(p, s);
  return off;
}
long pdgo_nbpts_total(const pdgo_problem *p) { return pdgo_bpts_offset(p, 2 * p->dim); }

static void cell_index(const pdgo_problem *p, long e, int *ix) {
  long t = e;
  for (int j = 0; j < p->dim; j++) { ix[j] = (int)(t % p->nc[j]); t /= p->nc[j]; }
}
static long cell_of(const pdgo_problem *p, const int *ix) {
  long e = 0;
  for (int j = p->dim - 1; j >= 0; j--) e = e * p->nc[j] + ix[j];
  return e;
}
static double cell_h(const pdgo_problem *p, int j) { return p->L[j] / p->nc[j]; }

/* index of a boundary face (cell e on side s) among that side's faces */
static long boundary_face_index(const pdgo_problem *p, const int *ix, int side) {
  int dir = side / 2;
  long idx = 0;
  for (int j = p->dim - 1; j >= 0; j--) {
    if (j == dir) continue;
    idx = idx * p->nc[j] + ix[j];
  }
  return idx;
}

static double Kof(const pdgo_problem *p, long e) { return p->K ? p->K[e] : 1.0; }

static void velocity(const pdgo_problem *p, const double *xg, double *b) {
  for (int j = 0; j < MAXD; j++) b[j] = 0.0;
  for (int m = 0; m < p->nmodes; m++) {
    const double *md = &p->modes[7 * m];
    double arg = md[3];
    for (int j = 0; j < p->dim; j++) arg += 2.0 * M_PI * md[j] * xg[j];
    double s = sin(arg);
    for (int j = 0; j < p->dim; j++) b[j] += md[4 + j] * s;
  }
}

/* ---- coefficients (ConvectionDiffusionModelProblem, convectiondiffusion-
   parameter.hh:148-183): A as a d x d tensor, row-major ---- */
static int pointwise_A(const pdgo_problem *p) { return p->Aq_vol && p->Aq_face; }
static void A_scalar(int d, double k, double *A) {
  for (int i = 0; i < d; i++)
    for (int j = 0; j < d; j++) A[i * d + j] = i == j ? k : 0.0;
}
/* A(cell, centre) (:124-127, :305-309, :710-713) */
static void A_centre(const pdgo_problem *p, long e, double *A) {
  int d = p->dim;
  if (p->Acell) memcpy(A, &p->Acell[e * d * d], sizeof(double) * d * d);
  else A_scalar(d, Kof(p, e), A);
}
/* A(cell, volume point q) and A(cell, point q of the cell's face f) */
static void A_vol_point(const pdgo_problem *p, int nqv, long e, int q, double *A) {
  int d = p->dim;
  memcpy(A, &p->Aq_vol[(e * nqv + q) * d * d], sizeof(double) * d * d);
}
static void A_face_point(const pdgo_problem *p, int nqf, long e, int f, int q, double *A) {
  int d = p->dim;
  memcpy(A, &p->Aq_face[((e * 2 * d + f) * nqf + q) * d * d], sizeof(double) * d * d);
}
/* y = A x (FieldMatrix::mv) */
static void mat_vec(int d, const double *A, const double *x, double *y) {
  for (int i = 0; i < d; i++) {
    y[i] = 0.0;
    for (int j = 0; j < d; j++) y[i] += A[i * d + j] * x[j];
  }
}
/* y = A^T x */
static void mat_tvec(int d, const double *A, const double *x, double *y) {
  for (int i = 0; i < d; i++) {
    y[i] = 0.0;
    for (int j = 0; j < d; j++) y[i] += A[j * d + i] * x[j];
  }
}
static double dotd(int d, const double *a, const double *b) {
  double s = 0.0;
  for (int j = 0; j < d; j++) s += a[j] * b[j];
  return s;
}
/* c(cell, volume point q) (:181): per-cell c plus the per-point part */
static double c_at(const pdgo_problem *p, int nqv, long e, int q) {
  return (p->c ? p->c[e] : 0.0) + (p->cq ? p->cq[e * nqv + q] : 0.0);
}

/* face lattice: see pdgo_face_lattice_index in pdg_oracle.h */
static long faces_in_plane(const pdgo_problem *p, int dir) {
  long n = 1;
  for (int j = 0; j < p->dim; j++)
    if (j != dir) n *= p->nc[j];
  return n;
}
long pdgo_nface_lattice(const pdgo_problem *p) {
  long n = 0;
  for (int dir = 0; dir < p->dim; dir++) n += (p->nc[dir] + 1) * faces_in_plane(p, dir);
  return n;
}
long pdgo_face_lattice_index(const pdgo_problem *p, int dir, int plane, const int *ix) {
  long off = 0;
  for (int j = 0; j < dir; j++) off += (p->nc[j] + 1) * faces_in_plane(p, j);
  long idx = 0;
  for (int j = p->dim - 1; j >= 0; j--) {
    if (j == dir) continue;
    idx = idx * p->nc[j] + ix[j];
  }
  return off + (long)plane * faces_in_plane(p, dir) + idx;
}

/* b(cell, x) at volume point q of cell e (:178) and at point q of face f
   of the inside cell e (:426, :797): per-point data when given, else the
   Fourier-mode field at the point's coordinates xg */
static int have_velocity(const pdgo_problem *p) {
  return p->nmodes > 0 || (p->bq_vol && p->bq_face);
}
static void b_vol(const pdgo_problem *p, int nqv, long e, int q, const double *xg, double *b) {
  if (p->bq_vol && p->bq_face) {
    for (int j = 0; j < MAXD; j++) b[j] = j < p->dim ? p->bq_vol[(e * nqv + q) * p->dim + j] : 0.0;
    return;
  }
  velocity(p, xg, b);
}
static void b_face(const pdgo_problem *p, int nqf, const int *ix, int f, int q, const double *xg,
                   double *b) {
  if (p->bq_vol && p->bq_face) {
    int dir = f / 2, hi = f % 2;
    long fi = pdgo_face_lattice_index(p, dir, ix[dir] + hi, ix);
    for (int j = 0; j < MAXD; j++) b[j] = j < p->dim ? p->bq_face[(fi * nqf + q) * p->dim + j] : 0.0;
    return;
  }
  velocity(p, xg, b);
}

int pdgo_volume_points(const pdgo_problem *p, double *xyz) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  long nc = pdgo_ncell(p);
  int d = T.d;
  for (long e = 0; e < nc; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    for (int q = 0; q < T.nqv; q++)
      for (int j = 0; j < d; j++)
        xyz[(e * T.nqv + q) * d + j] = (ix[j] + T.vloc[q * d + j]) * cell_h(p, j);
  }
  tables_free(&T);
  return PDGO_OK;
}

int pdgo_boundary_points(const pdgo_problem *p, double *xyz) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d;
  long nc = pdgo_ncell(p);
  for (long e = 0; e < nc; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    for (int side = 0; side < 2 * d; side++) {
      int dir = side / 2, hi = side % 2;
      if (ix[dir] != (hi ? p->nc[dir] - 1 : 0)) continue;
      long base = pdgo_bpts_offset(p, side) + boundary_face_index(p, ix, side) * T.nqf;
      for (int q = 0; q < T.nqf; q++)
        for (int j = 0; j < d; j++)
          xyz[(base + q) * d + j] = (ix[j] + T.floc[(side * T.nqf + q) * d + j]) * cell_h(p, j);
    }
  }
  tables_free(&T);
  return PDGO_OK;
}

int pdgo_face_lattice_points(const pdgo_problem *p, double *xyz) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d;
  long nc = pdgo_ncell(p);
  for (long e = 0; e < nc; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    for (int f = 0; f < 2 * d; f++) {
      int dir = f / 2, hi = f % 2;
      if (hi && ix[dir] != p->nc[dir] - 1) continue;   /* upper faces of the last cell only */
      long fi = pdgo_face_lattice_index(p, dir, ix[dir] + hi, ix);
      for (int q = 0; q < T.nqf; q++)
        for (int j = 0; j < d; j++)
          xyz[(fi * T.nqf + q) * d + j] = (ix[j] + T.floc[(f * T.nqf + q) * d + j]) * cell_h(p, j);
    }
  }
  tables_free(&T);
  return PDGO_OK;
}

int pdgo_cell_face_points(const pdgo_problem *p, double *xyz) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d;
  long nc = pdgo_ncell(p);
  for (long e = 0; e < nc; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    for (int f = 0; f < 2 * d; f++)
      for (int q = 0; q < T.nqf; q++)
        for (int j = 0; j < d; j++)
          xyz[((e * 2 * d + f) * T.nqf + q) * d + j] =
              (ix[j] + T.floc[(f * T.nqf + q) * d + j]) * cell_h(p, j);
  }
  tables_free(&T);
  return PDGO_OK;
}

/* ------------------------------------------------------------------ */
/* local operator (residual / jacobian_apply form)                     */
/* ------------------------------------------------------------------ */

typedef struct coef_override {
  int active;       /* 1: use Ks/Kn below, drop convection + reaction */
  double Ks, Kn;
} coef_override;

/* alpha_volume (convectiondiffusiondg.hh:105-188); also
   jacobian_apply_volume (:191-195) */
static void alpha_volume(const pdgo_problem *p, const tables *T, long e,
                         const double *x, double *r, const coef_override *co) {
  int d = T->d, nb = T->nb;
  int ix[MAXD];
  cell_index(p, e, ix);
  double h[MAXD], detJ = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); detJ *= h[j]; }
  /* A at the cell centre (:124-127), per point if not constant (:143-146) */
  int act = co && co->active;
  double A[MAXD * MAXD];
  if (act) A_scalar(d, co->Ks, A); else A_centre(p, e, A);
  double gradphi[MAXNB][MAXD];
  for (int q = 0; q < T->nqv; q++) {
    if (!act && pointwise_A(p)) A_vol_point(p, T->nqv, e, q, A);
    const double *phi = &T->vphi[q * nb];
    const double *js = &T->vjs[q * nb * d];
    double u = 0.0;
    for (int i = 0; i < nb; i++) u += x[i] * phi[i];
    /* jac = J^{-T} = diag(1/h) on axis-parallel cells */
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < d; j++) gradphi[i][j] = js[i * d + j] / h[j];
    double gradu[MAXD] = {0, 0, 0}, Agradu[MAXD];
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < d; j++) gradu[j] += x[i] * gradphi[i][j];
    mat_vec(d, A, gradu, Agradu);
    double b[MAXD] = {0, 0, 0};
    if (!act && have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ix[j] + T->vloc[q * d + j]) * h[j];
      b_vol(p, T->nqv, e, q, xg, b);
    }
    double cc = act ? 0.0 : c_at(p, T->nqv, e, q);
    double factor = T->vw[q] * detJ;
    for (int i = 0; i < nb; i++) {
      double ag = 0.0, bg = 0.0;
      for (int j = 0; j < d; j++) { ag += Agradu[j] * gradphi[i][j]; bg += b[j] * gradphi[i][j]; }
      r[i] += (ag - u * bg + cc * u * phi[i]) * factor;
    }
  }
}

/* nonlinear volume term (nonlinearconvectiondiffusiondg.hh:93-176):
   mode 0: r += int q(u) psi (alpha_volume), u from x;
   mode 1: r += int q'(u_lin) z psi (jacobian_apply_volume), x = z. */
static double nl_q(const pdgo_problem *p, double u) {
  double s = 0.0;
  for (int m = p->nl_deg; m >= 0; m--) s = s * u + p->nl_coef[m];
  return s;
}
static double nl_qprime(const pdgo_problem *p, double u) {
  double s = 0.0;
  for (int m = p->nl_deg; m >= 1; m--) s = s * u + m * p->nl_coef[m];
  return s;
}
static void nl_volume(const pdgo_problem *p, const tables *T, long e, const double *x,
                      double *r, int mode) {
  if (p->nl_deg <= 0 || (mode == 1 && !p->xlin)) return;
  int d = T->d, nb = T->nb;
  double detJ = 1.0;
  for (int j = 0; j < d; j++) detJ *= cell_h(p, j);
  const double *xl = mode == 1 ? &p->xlin[e * nb] : x;
  for (int q = 0; q < T->nqv; q++) {
    const double *phi = &T->vphi[q * nb];
    double u = 0.0, zq = 0.0;
    for (int i = 0; i < nb; i++) u += xl[i] * phi[i];
    if (mode == 1)
      for (int i = 0; i < nb; i++) zq += x[i] * phi[i];
    const double v = mode == 1 ? nl_qprime(p, u) * zq : nl_q(p, u);
    const double factor = T->vw[q] * detJ;
    for (int i = 0; i < nb; i++) r[i] += v * phi[i] * factor;
  }
}

/* lambda_volume (convectiondiffusiondg.hh:1047-1075) */
static void lambda_volume(const pdgo_problem *p, const tables *T, long e, double *r) {
  int d = T->d, nb = T->nb;
  double detJ = 1.0;
  for (int j = 0; j < d; j++) detJ *= cell_h(p, j);
  for (int q = 0; q < T->nqv; q++) {
    const double *phi = &T->vphi[q * nb];
    double f = 0.0;
    if (p->fq) f += p->fq[e * T->nqv + q];
    if (p->fc) f += p->fc[e];
    double factor = T->vw[q] * detJ;
    for (int i = 0; i < nb; i++) r[i] += -f * phi[i] * factor;
  }
}

/* skeleton weights (convectiondiffusiondg.hh:308-346) from
   delta = (A n).n of both sides */
static void face_weights(const pdgo_problem *p, double delta_s, double delta_n, double hF,
                         double *omega_s, double *omega_n, double *penalty) {
  double harmonic_average;
  if (p->weights == PDGO_WEIGHTS_ON) {
    *omega_s = delta_n / (delta_s + delta_n + 1e-20);
    *omega_n = delta_s / (delta_s + delta_n + 1e-20);
    harmonic_average = 2.0 * delta_s * delta_n / (delta_s + delta_n + 1e-20);
  } else {
    *omega_s = *omega_n = 0.5;
    harmonic_average = 1.0;
  }
  int degree = p->k;
  *penalty = (p->alpha / hF) * harmonic_average * degree * (degree + p->dim - 1);
}

/* The coefficient state of one side pair of an interior face: A_s n, A_n n,
   the weights and the penalty (:305-346), refreshed per point when A is not
   constant per cell (:365-382). */
typedef struct face_coef {
  double As[MAXD * MAXD], An[MAXD * MAXD];
  double AnFs[MAXD], AnFn[MAXD];
  double omega_s, omega_n, penalty;
} face_coef;

static void face_coef_update(const pdgo_problem *p, int d, const double *nF, double hF,
                             face_coef *fc) {
  mat_vec(d, fc->As, nF, fc->AnFs);
  mat_vec(d, fc->An, nF, fc->AnFn);
  face_weights(p, dotd(d, fc->AnFs, nF), dotd(d, fc->AnFn, nF), hF, &fc->omega_s, &fc->omega_n,
               &fc->penalty);
}

static void face_coef_init(const pdgo_problem *p, int d, long s, long n, const double *nF,
                           double hF, const coef_override *co, face_coef *fc) {
  if (co && co->active) { A_scalar(d, co->Ks, fc->As); A_scalar(d, co->Kn, fc->An); }
  else { A_centre(p, s, fc->As); A_centre(p, n, fc->An); }
  face_coef_update(p, d, nF, hF, fc);
}

static void face_coef_point(const pdgo_problem *p, int d, int nqf, long s, long n, int fs, int fn,
                            int q, const double *nF, double hF, const coef_override *co,
                            face_coef *fc) {
  if ((co && co->active) || !pointwise_A(p)) return;
  A_face_point(p, nqf, s, fs, q, fc->As);
  A_face_point(p, nqf, n, fn, q, fc->An);
  face_coef_update(p, d, nF, hF, fc);
}

/* alpha_skeleton (convectiondiffusiondg.hh:270-471) for the interior face
   between inside cell s and outside cell n; the face is normal to `dir`,
   and n lies on side `hi_s` of s (0 = lower, 1 = upper).  With transpose
   set it adds J^T instead: the same point quantities, with the roles of
   the trial traces (u, A n . grad u) and of the test traces (psi,
   A n . grad psi) exchanged term by term. */
static void skeleton_form(const pdgo_problem *p, const tables *T, long s, long n,
                          int dir, int hi_s, const double *x_s, const double *x_n,
                          double *r_s, double *r_n, const coef_override *co, int transpose) {
  int d = T->d, nb = T->nb, nqf = T->nqf;
  double h[MAXD], vol = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); vol *= h[j]; }
  double area = vol / h[dir];
  double vol_s = vol, vol_n = vol;                   /* uniform grid */
  double hF = (vol_s < vol_n ? vol_s : vol_n) / area; /* min(|T_s|,|T_n|)/|F| (:313) */
  double nF[MAXD] = {0, 0, 0};
  nF[dir] = hi_s ? 1.0 : -1.0;
  face_coef fc;
  face_coef_init(p, d, s, n, nF, hF, co, &fc);
  int fs = 2 * dir + hi_s, fn = 2 * dir + (1 - hi_s);
  int ixs[MAXD];
  cell_index(p, s, ixs);
  int act = co && co->active;
  double tgs[MAXNB][MAXD], tgn[MAXNB][MAXD], ans[MAXNB], ann[MAXNB];
  for (int q = 0; q < nqf; q++) {
    face_coef_point(p, d, nqf, s, n, fs, fn, q, nF, hF, co, &fc);
    const double *phi_s = &T->fphi[(fs * nqf + q) * nb];
    const double *phi_n = &T->fphi[(fn * nqf + q) * nb];
    const double *js_s = &T->fjs[(fs * nqf + q) * nb * d];
    const double *js_n = &T->fjs[(fn * nqf + q) * nb * d];
    double u_s = 0.0, u_n = 0.0;
    for (int i = 0; i < nb; i++) u_s += x_s[i] * phi_s[i];
    for (int i = 0; i < nb; i++) u_n += x_n[i] * phi_n[i];
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < d; j++) { tgs[i][j] = js_s[i * d + j] / h[j]; tgn[i][j] = js_n[i * d + j] / h[j]; }
    /* A n . grad(phi_i) on both sides */
    for (int i = 0; i < nb; i++) { ans[i] = dotd(d, fc.AnFs, tgs[i]); ann[i] = dotd(d, fc.AnFn, tgn[i]); }
    double b[MAXD] = {0, 0, 0};
    if (!act && have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ixs[j] + T->floc[(fs * nqf + q) * d + j]) * h[j];
      b_face(p, nqf, ixs, fs, q, xg, b);
    }
    double normalflux = dotd(d, b, nF);
    double omegaup_s, omegaup_n;
    if (normalflux >= 0.0) { omegaup_s = 1.0; omegaup_n = 0.0; }
    else { omegaup_s = 0.0; omegaup_n = 1.0; }
    double factor = T->fw[fs * nqf + q] * area;
    double omega_s = fc.omega_s, omega_n = fc.omega_n, penalty = fc.penalty;
    if (!transpose) {
      double gus[MAXD] = {0, 0, 0}, gun[MAXD] = {0, 0, 0};
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < d; j++) { gus[j] += x_s[i] * tgs[i][j]; gun[j] += x_n[i] * tgn[i][j]; }
      /* A_s n . grad u_s, A_n n . grad u_n */
      double Ags = dotd(d, fc.AnFs, gus), Agn = dotd(d, fc.AnFn, gun);
      double term1 = (omegaup_s * u_s + omegaup_n * u_n) * normalflux * factor;
      double term2 = -(omega_s * Ags + omega_n * Agn) * factor;
      double term3 = (u_s - u_n) * factor;
      double term4 = penalty * (u_s - u_n) * factor;
      for (int i = 0; i < nb; i++) {
        r_s[i] += term1 * phi_s[i];
        r_n[i] += -term1 * phi_n[i];
        r_s[i] += term2 * phi_s[i];
        r_n[i] += -term2 * phi_n[i];
        r_s[i] += term3 * T->theta * omega_s * ans[i];
        r_n[i] += term3 * T->theta * omega_n * ann[i];
        r_s[i] += term4 * phi_s[i];
        r_n[i] += -term4 * phi_n[i];
      }
    } else {
      /* x holds the test-side vector z: jump [z] = z_s - z_n of the value
         traces and the weighted A n . grad z traces */
      double jz = u_s - u_n;
      double az = 0.0;
      for (int i = 0; i < nb; i++) az += T->theta * (omega_s * x_s[i] * ans[i] + omega_n * x_n[i] * ann[i]);
      for (int j = 0; j < nb; j++) {
        /* term1: trial value of side s (n) times the upwind weight */
        r_s[j] += omegaup_s * normalflux * factor * jz * phi_s[j];
        r_n[j] += omegaup_n * normalflux * factor * jz * phi_n[j];
        /* term2: trial A n . grad */
        r_s[j] += -omega_s * factor * jz * ans[j];
        r_n[j] += -omega_n * factor * jz * ann[j];
        /* term3: trial jump against the test A n . grad traces */
        r_s[j] += factor * az * phi_s[j];
        r_n[j] += -factor * az * phi_n[j];
        /* term4 */
        r_s[j] += penalty * factor * jz * phi_s[j];
        r_n[j] += -penalty * factor * jz * phi_n[j];
      }
    }
  }
}

static void alpha_skeleton(const pdgo_problem *p, const tables *T, long s, long n,
                           int dir, int hi_s, const double *x_s, const double *x_n,
                           double *r_s, double *r_n, const coef_override *co) {
  skeleton_form(p, T, s, n, dir, hi_s, x_s, x_n, r_s, r_n, co, 0);
}

/* residual_boundary_integral (convectiondiffusiondg.hh:683-879), called by
   alpha_boundary (:883-889, jacobian_apply=false) and
   jacobian_apply_boundary (:892-899, jacobian_apply=true).  transpose = 1
   (only with jacobian_apply) adds the transposed boundary form. */
static int boundary_form(const pdgo_problem *p, const tables *T, long e, int side,
                         const double *x_s, double *r_s, int jacobian_apply,
                         const coef_override *co, int transpose) {
  int d = T->d, nb = T->nb, nqf = T->nqf;
  int dir = side / 2, hi = side % 2;
  double h[MAXD], vol = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); vol *= h[j]; }
  double area = vol / h[dir];
  double hF = vol / area;
  double nF[MAXD] = {0, 0, 0};
  nF[dir] = hi ? 1.0 : -1.0;
  int act = co && co->active;
  double A[MAXD * MAXD], An_F_s[MAXD];
  if (act) A_scalar(d, co->Ks, A); else A_centre(p, e, A);
  int degree = p->k;
  int ix[MAXD];
  cell_index(p, e, ix);
  long base = pdgo_bpts_offset(p, side) + boundary_face_index(p, ix, side) * nqf;
  int bctype = p->bctype[side];
  double tg[MAXNB][MAXD], an[MAXNB];
  for (int q = 0; q < nqf; q++) {
    /* A n and the penalty (:710-734), per point if A is not constant (:750-761) */
    if (!act && pointwise_A(p)) A_face_point(p, nqf, e, side, q, A);
    mat_vec(d, A, nF, An_F_s);
    double harmonic_average = (p->weights == PDGO_WEIGHTS_ON) ? dotd(d, An_F_s, nF) : 1.0;
    double penalty_factor = (p->alpha / hF) * harmonic_average * degree * (degree + d - 1);
    if (bctype == PDGO_BC_NONE) continue;
    const double *phi = &T->fphi[(side * nqf + q) * nb];
    const double *js = &T->fjs[(side * nqf + q) * nb * d];
    double factor = T->fw[side * nqf + q] * area;
    if (bctype == PDGO_BC_NEUMANN) {
      if (!jacobian_apply) {
        double jv = p->jq ? p->jq[base + q] : 0.0;
        for (int i = 0; i < nb; i++) r_s[i] += jv * phi[i] * factor;
      }
      continue;
    }
    double u_s = 0.0;
    for (int i = 0; i < nb; i++) u_s += x_s[i] * phi[i];
    double b[MAXD] = {0, 0, 0};
    if (!act && have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ix[j] + T->floc[(side * nqf + q) * d + j]) * h[j];
      b_face(p, nqf, ix, side, q, xg, b);
    }
    double normalflux = dotd(d, b, nF);
    if (bctype == PDGO_BC_OUTFLOW) {
      if (normalflux < -1e-30) return PDGO_EOUTFLOW_ON_INFLOW;
      double term1 = u_s * normalflux * factor;   /* symmetric in test and trial */
      for (int i = 0; i < nb; i++) r_s[i] += term1 * phi[i];
      if (!jacobian_apply) {
        double ov = p->oq ? p->oq[base + q] : 0.0;
        for (int i = 0; i < nb; i++) r_s[i] += ov * phi[i] * factor;
      }
      continue;
    }
    /* Dirichlet */
    for (int i = 0; i < nb; i++) {
      for (int j = 0; j < d; j++) tg[i][j] = js[i * d + j] / h[j];
      an[i] = dotd(d, An_F_s, tg[i]);
    }
    double g = p->gq ? p->gq[base + q] : 0.0;
    if (jacobian_apply) g = 0.0;
    double omegaup_s, omegaup_n;
    if (normalflux >= 0.0) { omegaup_s = 1.0; omegaup_n = 0.0; }
    else { omegaup_s = 0.0; omegaup_n = 1.0; }
    if (!transpose) {
      double gu[MAXD] = {0, 0, 0};
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < d; j++) gu[j] += x_s[i] * tg[i][j];
      double Ag = dotd(d, An_F_s, gu);
      double term1 = (omegaup_s * u_s + omegaup_n * g) * normalflux * factor;
      double term2 = Ag * factor;
      double term3 = (u_s - g) * factor;
      double term4 = penalty_factor * (u_s - g) * factor;
      for (int i = 0; i < nb; i++) {
        r_s[i] += term1 * phi[i];
        r_s[i] += -term2 * phi[i];
        r_s[i] += term3 * T->theta * an[i];
        r_s[i] += term4 * phi[i];
      }
    } else {
      double az = 0.0;
      for (int i = 0; i < nb; i++) az += x_s[i] * an[i];
      for (int j = 0; j < nb; j++) {
        r_s[j] += omegaup_s * normalflux * factor * u_s * phi[j];
        r_s[j] += -factor * u_s * an[j];
        r_s[j] += T->theta * factor * az * phi[j];
        r_s[j] += penalty_factor * factor * u_s * phi[j];
      }
    }
  }
  return PDGO_OK;
}

static int boundary_integral(const pdgo_problem *p, const tables *T, long e, int side,
                             const double *x_s, double *r_s, int jacobian_apply,
                             const coef_override *co) {
  return boundary_form(p, T, e, side, x_s, r_s, jacobian_apply, co, 0);
}

/* transposed jacobian_apply_volume: y_j += sum_q w [A grad phi_j . grad z
   - phi_j b . grad z + c phi_j z] (the volume form with test and trial
   exchanged) */
static void volume_transpose(const pdgo_problem *p, const tables *T, long e,
                             const double *z, double *y) {
  int d = T->d, nb = T->nb;
  int ix[MAXD];
  cell_index(p, e, ix);
  double h[MAXD], detJ = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); detJ *= h[j]; }
  double A[MAXD * MAXD];
  A_centre(p, e, A);
  double gradphi[MAXNB][MAXD];
  for (int q = 0; q < T->nqv; q++) {
    if (pointwise_A(p)) A_vol_point(p, T->nqv, e, q, A);
    const double *phi = &T->vphi[q * nb];
    const double *js = &T->vjs[q * nb * d];
    double zq = 0.0, gz[MAXD] = {0, 0, 0}, Atgz[MAXD];
    for (int i = 0; i < nb; i++) zq += z[i] * phi[i];
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < d; j++) { gradphi[i][j] = js[i * d + j] / h[j]; gz[j] += z[i] * gradphi[i][j]; }
    mat_tvec(d, A, gz, Atgz);    /* (A grad phi_j) . grad z = grad phi_j . (A^T grad z) */
    double b[MAXD] = {0, 0, 0};
    if (have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ix[j] + T->vloc[q * d + j]) * h[j];
      b_vol(p, T->nqv, e, q, xg, b);
    }
    double bz = dotd(d, b, gz);
    double cc = c_at(p, T->nqv, e, q);
    double factor = T->vw[q] * detJ;
    for (int j = 0; j < nb; j++)
      y[j] += (dotd(d, Atgz, gradphi[j]) - phi[j] * bz + cc * phi[j] * zq) * factor;
  }
}

/* DefaultAssembler::assemble (gridoperator/default/assembler.hh:85-279):
   element loop, volume terms, then intersections; an interior face is
   visited once, from the cell with the larger index (:181). */
static int assemble_vector(const pdgo_problem *p, const double *x, double *r, int jacobian_apply,
                           long e_begin, long e_end) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d, nb = T.nb;
  long nc = pdgo_ncell(p);
  if (e_end > nc) e_end = nc;
  int st = PDGO_OK;
  for (long e = e_begin; e < e_end && !st; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    if (!jacobian_apply) lambda_volume(p, &T, e, &r[e * nb]);
    alpha_volume(p, &T, e, &x[e * nb], &r[e * nb], NULL);
    nl_volume(p, &T, e, &x[e * nb], &r[e * nb], jacobian_apply);
    for (int f = 0; f < 2 * d && !st; f++) {
      int dir = f / 2, hi = f % 2;
      int jx[MAXD];
      memcpy(jx, ix, sizeof(jx));
      jx[dir] += hi ? 1 : -1;
      if (jx[dir] < 0 || jx[dir] >= p->nc[dir]) {
        st = boundary_integral(p, &T, e, f, &x[e * nb], &r[e * nb], jacobian_apply, NULL);
        continue;
      }
      long n = cell_of(p, jx);
      if (!(e > n)) continue;
      alpha_skeleton(p, &T, e, n, dir, hi, &x[e * nb], &x[n * nb], &r[e * nb], &r[n * nb], NULL);
    }
  }
  tables_free(&T);
  return st;
}

int pdgo_jacobian_apply(const pdgo_problem *p, const double *z, double *y) {
  return assemble_vector(p, z, y, 1, 0, pdgo_ncell(p));
}
int pdgo_jacobian_apply_range(const pdgo_problem *p, const double *z, double *y,
                              long e_begin, long e_end) {
  return assemble_vector(p, z, y, 1, e_begin, e_end);
}
/* y += J^T z over the traversal of assemble_vector: volume and boundary
   blocks transposed in place, each interior face's four blocks transposed
   and exchanged between the two sides.  The nonlinear Jacobian term
   int q'(u_lin) z psi is symmetric and enters unchanged. */
static int assemble_transpose(const pdgo_problem *p, const double *z, double *y, long e_begin,
                              long e_end) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d, nb = T.nb;
  long nc = pdgo_ncell(p);
  if (e_end > nc) e_end = nc;
  int st = PDGO_OK;
  for (long e = e_begin; e < e_end && !st; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    volume_transpose(p, &T, e, &z[e * nb], &y[e * nb]);
    nl_volume(p, &T, e, &z[e * nb], &y[e * nb], 1);
    for (int f = 0; f < 2 * d && !st; f++) {
      int dir = f / 2, hi = f % 2;
      int jx[MAXD];
      memcpy(jx, ix, sizeof(jx));
      jx[dir] += hi ? 1 : -1;
      if (jx[dir] < 0 || jx[dir] >= p->nc[dir]) {
        st = boundary_form(p, &T, e, f, &z[e * nb], &y[e * nb], 1, NULL, 1);
        continue;
      }
      long n = cell_of(p, jx);
      if (!(e > n)) continue;
      skeleton_form(p, &T, e, n, dir, hi, &z[e * nb], &z[n * nb], &y[e * nb], &y[n * nb], NULL, 1);
    }
  }
  tables_free(&T);
  return st;
}

int pdgo_jacobian_apply_transpose(const pdgo_problem *p, const double *z, double *y) {
  return assemble_transpose(p, z, y, 0, pdgo_ncell(p));
}
int pdgo_jacobian_apply_transpose_range(const pdgo_problem *p, const double *z, double *y,
                                        long e_begin, long e_end) {
  return assemble_transpose(p, z, y, e_begin, e_end);
}
int pdgo_residual(const pdgo_problem *p, const double *x, double *r) {
  return assemble_vector(p, x, r, 0, 0, pdgo_ncell(p));
}

/* ------------------------------------------------------------------ */
/* assembled local blocks (jacobian_volume / _skeleton / _boundary)    */
/* mat[i*nb + j]: test i, trial j                                     */
/* ------------------------------------------------------------------ */

/* jacobian_volume (convectiondiffusiondg.hh:198-266) */
static void jacobian_volume(const pdgo_problem *p, const tables *T, long e,
                            double *mat, const coef_override *co) {
  int d = T->d, nb = T->nb;
  int ix[MAXD];
  cell_index(p, e, ix);
  double h[MAXD], detJ = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); detJ *= h[j]; }
  int act = co && co->active;
  double A[MAXD * MAXD];
  if (act) A_scalar(d, co->Ks, A); else A_centre(p, e, A);
  double gradphi[MAXNB][MAXD], Agradphi[MAXNB][MAXD];
  for (int q = 0; q < T->nqv; q++) {
    if (!act && pointwise_A(p)) A_vol_point(p, T->nqv, e, q, A);
    const double *phi = &T->vphi[q * nb];
    const double *js = &T->vjs[q * nb * d];
    for (int i = 0; i < nb; i++) {
      for (int j = 0; j < d; j++) gradphi[i][j] = js[i * d + j] / h[j];
      mat_vec(d, A, gradphi[i], Agradphi[i]);
    }
    double b[MAXD] = {0, 0, 0};
    if (!act && have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ix[j] + T->vloc[q * d + j]) * h[j];
      b_vol(p, T->nqv, e, q, xg, b);
    }
    double cc = act ? 0.0 : c_at(p, T->nqv, e, q);
    double factor = T->vw[q] * detJ;
    /* nonlinear part at the linearization point (jacobian_volume of
       nonlinearconvectiondiffusiondg.hh:178-223) */
    double qp = 0.0;
    if (!(co && co->active) && p->nl_deg > 0 && p->xlin) {
      double u = 0.0;
      for (int i = 0; i < nb; i++) u += p->xlin[e * nb + i] * phi[i];
      qp = nl_qprime(p, u);
    }
    for (int jj = 0; jj < nb; jj++)
      for (int i = 0; i < nb; i++) {
        double ag = 0.0, bg = 0.0;
        for (int j = 0; j < d; j++) { ag += Agradphi[jj][j] * gradphi[i][j]; bg += b[j] * gradphi[i][j]; }
        mat[i * nb + jj] += (ag - phi[jj] * bg + (cc + qp) * phi[jj] * phi[i]) * factor;
      }
  }
}

/* jacobian_skeleton (convectiondiffusiondg.hh:483-669); any of the output
   blocks may be NULL (the block-diagonal wrapper keeps only mat_ss,
   blockdiagonalwrapper.hh:141-153). */
static void jacobian_skeleton(const pdgo_problem *p, const tables *T, long s, long n,
                              int dir, int hi_s, double *mat_ss, double *mat_sn,
                              double *mat_ns, double *mat_nn, const coef_override *co) {
  int d = T->d, nb = T->nb, nqf = T->nqf;
  double h[MAXD], vol = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); vol *= h[j]; }
  double area = vol / h[dir];
  double hF = vol / area;
  double nF[MAXD] = {0, 0, 0};
  nF[dir] = hi_s ? 1.0 : -1.0;
  face_coef fc;
  face_coef_init(p, d, s, n, nF, hF, co, &fc);
  int fs = 2 * dir + hi_s, fn = 2 * dir + (1 - hi_s);
  int ixs[MAXD];
  cell_index(p, s, ixs);
  double tgs[MAXNB][MAXD], tgn[MAXNB][MAXD];
  double theta = T->theta;
  for (int q = 0; q < nqf; q++) {
    face_coef_point(p, d, nqf, s, n, fs, fn, q, nF, hF, co, &fc);
    const double *An_F_s = fc.AnFs, *An_F_n = fc.AnFn;
    double omega_s = fc.omega_s, omega_n = fc.omega_n, penalty = fc.penalty;
    const double *phi_s = &T->fphi[(fs * nqf + q) * nb];
    const double *phi_n = &T->fphi[(fn * nqf + q) * nb];
    const double *js_s = &T->fjs[(fs * nqf + q) * nb * d];
    const double *js_n = &T->fjs[(fn * nqf + q) * nb * d];
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < d; j++) { tgs[i][j] = js_s[i * d + j] / h[j]; tgn[i][j] = js_n[i * d + j] / h[j]; }
    double b[MAXD] = {0, 0, 0};
    if (!(co && co->active) && have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ixs[j] + T->floc[(fs * nqf + q) * d + j]) * h[j];
      b_face(p, nqf, ixs, fs, q, xg, b);
    }
    double normalflux = 0.0;
    for (int j = 0; j < d; j++) normalflux += b[j] * nF[j];
    double omegaup_s, omegaup_n;
    if (normalflux >= 0.0) { omegaup_s = 1.0; omegaup_n = 0.0; }
    else { omegaup_s = 0.0; omegaup_n = 1.0; }
    double factor = T->fw[fs * nqf + q] * area;
    double ipfactor = penalty * factor;
    double ans[MAXNB], ann[MAXNB];
    for (int i = 0; i < nb; i++) {
      ans[i] = 0.0; ann[i] = 0.0;
      for (int j = 0; j < d; j++) { ans[i] += An_F_s[j] * tgs[i][j]; ann[i] += An_F_n[j] * tgn[i][j]; }
    }
    if (mat_ss)
      for (int jj = 0; jj < nb; jj++) {
        double temp1 = -ans[jj] * omega_s * factor;
        for (int i = 0; i < nb; i++) {
          double *m = &mat_ss[i * nb + jj];
          *m += omegaup_s * phi_s[jj] * normalflux * factor * phi_s[i];
          *m += temp1 * phi_s[i];
          *m += phi_s[jj] * factor * theta * omega_s * ans[i];
          *m += phi_s[jj] * ipfactor * phi_s[i];
        }
      }
    if (mat_sn)
      for (int jj = 0; jj < nb; jj++) {
        double temp1 = -ann[jj] * omega_n * factor;
        for (int i = 0; i < nb; i++) {
          double *m = &mat_sn[i * nb + jj];
          *m += omegaup_n * phi_n[jj] * normalflux * factor * phi_s[i];
          *m += temp1 * phi_s[i];
          *m += -phi_n[jj] * factor * theta * omega_s * ans[i];
          *m += -phi_n[jj] * ipfactor * phi_s[i];
        }
      }
    if (mat_ns)
      for (int jj = 0; jj < nb; jj++) {
        double temp1 = -ans[jj] * omega_s * factor;
        for (int i = 0; i < nb; i++) {
          double *m = &mat_ns[i * nb + jj];
          *m += -omegaup_s * phi_s[jj] * normalflux * factor * phi_n[i];
          *m += -temp1 * phi_n[i];
          *m += phi_s[jj] * factor * theta * omega_n * ann[i];
          *m += -phi_s[jj] * ipfactor * phi_n[i];
        }
      }
    if (mat_nn)
      for (int jj = 0; jj < nb; jj++) {
        double temp1 = -ann[jj] * omega_n * factor;
        for (int i = 0; i < nb; i++) {
          double *m = &mat_nn[i * nb + jj];
          *m += -omegaup_n * phi_n[jj] * normalflux * factor * phi_n[i];
          *m += -temp1 * phi_n[i];
          *m += -phi_n[jj] * factor * theta * omega_n * ann[i];
          *m += phi_n[jj] * ipfactor * phi_n[i];
        }
      }
  }
}

/* jacobian_boundary (convectiondiffusiondg.hh:901-1044) */
static int jacobian_boundary(const pdgo_problem *p, const tables *T, long e, int side,
                             double *mat_ss, const coef_override *co) {
  int d = T->d, nb = T->nb, nqf = T->nqf;
  int dir = side / 2, hi = side % 2;
  double h[MAXD], vol = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); vol *= h[j]; }
  double area = vol / h[dir];
  double hF = vol / area;
  double nF[MAXD] = {0, 0, 0};
  nF[dir] = hi ? 1.0 : -1.0;
  int act = co && co->active;
  double A[MAXD * MAXD], An_F_s[MAXD];
  if (act) A_scalar(d, co->Ks, A); else A_centre(p, e, A);
  int degree = p->k;
  int ix[MAXD];
  cell_index(p, e, ix);
  int bctype = p->bctype[side];
  double tg[MAXNB][MAXD], an[MAXNB];
  for (int q = 0; q < nqf; q++) {
    if (!act && pointwise_A(p)) A_face_point(p, nqf, e, side, q, A);
    mat_vec(d, A, nF, An_F_s);
    double harmonic_average = (p->weights == PDGO_WEIGHTS_ON) ? dotd(d, An_F_s, nF) : 1.0;
    double penalty_factor = (p->alpha / hF) * harmonic_average * degree * (degree + d - 1);
    if (bctype == PDGO_BC_NONE || bctype == PDGO_BC_NEUMANN) continue;
    const double *phi = &T->fphi[(side * nqf + q) * nb];
    const double *js = &T->fjs[(side * nqf + q) * nb * d];
    double factor = T->fw[side * nqf + q] * area;
    double b[MAXD] = {0, 0, 0};
    if (!act && have_velocity(p)) {
      double xg[MAXD];
      for (int j = 0; j < d; j++) xg[j] = (ix[j] + T->floc[(side * nqf + q) * d + j]) * h[j];
      b_face(p, nqf, ix, side, q, xg, b);
    }
    double normalflux = 0.0;
    for (int j = 0; j < d; j++) normalflux += b[j] * nF[j];
    if (bctype == PDGO_BC_OUTFLOW) {
      if (normalflux < -1e-30) return PDGO_EOUTFLOW_ON_INFLOW;
      for (int jj = 0; jj < nb; jj++)
        for (int i = 0; i < nb; i++)
          mat_ss[i * nb + jj] += phi[jj] * normalflux * factor * phi[i];
      continue;
    }
    for (int i = 0; i < nb; i++) {
      an[i] = 0.0;
      for (int j = 0; j < d; j++) { tg[i][j] = js[i * d + j] / h[j]; an[i] += An_F_s[j] * tg[i][j]; }
    }
    double omegaup_s = normalflux >= 0.0 ? 1.0 : 0.0;
    for (int jj = 0; jj < nb; jj++)
      for (int i = 0; i < nb; i++)
        mat_ss[i * nb + jj] += omegaup_s * phi[jj] * normalflux * factor * phi[i];
    for (int jj = 0; jj < nb; jj++)
      for (int i = 0; i < nb; i++)
        mat_ss[i * nb + jj] += -an[jj] * factor * phi[i];
    for (int jj = 0; jj < nb; jj++)
      for (int i = 0; i < nb; i++)
        mat_ss[i * nb + jj] += phi[jj] * factor * T->theta * an[i];
    for (int jj = 0; jj < nb; jj++)
      for (int i = 0; i < nb; i++)
        mat_ss[i * nb + jj] += penalty_factor * phi[jj] * phi[i] * factor;
  }
  return PDGO_OK;
}

int pdgo_assemble_jacobian(const pdgo_problem *p, double *blocks) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d, nb = T.nb, ns = 2 * d + 1;
  long nc = pdgo_ncell(p);
  long bs = (long)nb * nb;
  memset(blocks, 0, sizeof(double) * nc * ns * bs);
  int st = PDGO_OK;
  /* jacobian engine over the same one-sided traversal
     (gridoperator/default/jacobianengine.hh:247-294) */
  for (long e = 0; e < nc && !st; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    jacobian_volume(p, &T, e, &blocks[(e * ns) * bs], NULL);
    for (int f = 0; f < 2 * d && !st; f++) {
      int dir = f / 2, hi = f % 2;
      int jx[MAXD];
      memcpy(jx, ix, sizeof(jx));
      jx[dir] += hi ? 1 : -1;
      if (jx[dir] < 0 || jx[dir] >= p->nc[dir]) {
        st = jacobian_boundary(p, &T, e, f, &blocks[(e * ns) * bs], NULL);
        continue;
      }
      long n = cell_of(p, jx);
      if (!(e > n)) continue;
      int fn = 2 * dir + (1 - hi);
      jacobian_skeleton(p, &T, e, n, dir, hi,
                        &blocks[(e * ns) * bs], &blocks[(e * ns + 1 + f) * bs],
                        &blocks[(n * ns + 1 + fn) * bs], &blocks[(n * ns) * bs], NULL);
    }
  }
  tables_free(&T);
  return st;
}

static long neighbor(const pdgo_problem *p, long e, int f) {
  int ix[MAXD];
  cell_index(p, e, ix);
  int dir = f / 2, hi = f % 2;
  ix[dir] += hi ? 1 : -1;
  if (ix[dir] < 0 || ix[dir] >= p->nc[dir]) return -1;
  return cell_of(p, ix);
}

int pdgo_blocks_apply(const pdgo_problem *p, const double *blocks, const double *x, double *y) {
  int d = p->dim, nb = pdgo_nbasis(p), ns = 2 * d + 1;
  long nc = pdgo_ncell(p), bs = (long)nb * nb;
  for (long e = 0; e < nc; e++) {
    double *ye = &y[e * nb];
    for (int i = 0; i < nb; i++) ye[i] = 0.0;
    for (int sl = 0; sl < ns; sl++) {
      long n = sl == 0 ? e : neighbor(p, e, sl - 1);
      if (n < 0) continue;
      const double *B = &blocks[(e * ns + sl) * bs];
      const double *xn = &x[n * nb];
      for (int i = 0; i < nb; i++) {
        double s = 0.0;
        for (int j = 0; j < nb; j++) s += B[i * nb + j] * xn[j];
        ye[i] += s;
      }
    }
  }
  return PDGO_OK;
}

int pdgo_blocks_apply_transpose(const pdgo_problem *p, const double *blocks, const double *x, double *y) {
  int d = p->dim, nb = pdgo_nbasis(p), ns = 2 * d + 1;
  long nc = pdgo_ncell(p), bs = (long)nb * nb;
  memset(y, 0, sizeof(double) * nc * nb);
  for (long e = 0; e < nc; e++) {
    const double *xe = &x[e * nb];
    for (int sl = 0; sl < ns; sl++) {
      long n = sl == 0 ? e : neighbor(p, e, sl - 1);
      if (n < 0) continue;
      const double *B = &blocks[(e * ns + sl) * bs];
      double *yn = &y[n * nb];
      for (int j = 0; j < nb; j++) {
        double s = 0.0;
        for (int i = 0; i < nb; i++) s += B[i * nb + j] * xe[i];
        yn[j] += s;
      }
    }
  }
  return PDGO_OK;
}

/* assembleLocalDiagonalBlock (localoperator/blockdiagonalwrapper.hh:225-257):
   volume + self-self part of every interior face visited from this cell
   (two-sided) + boundary faces. */
int pdgo_block_diagonal(const pdgo_problem *p, double *diag) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d, nb = T.nb;
  long nc = pdgo_ncell(p), bs = (long)nb * nb;
  memset(diag, 0, sizeof(double) * nc * bs);
  int st = PDGO_OK;
  for (long e = 0; e < nc && !st; e++) {
    jacobian_volume(p, &T, e, &diag[e * bs], NULL);
    for (int f = 0; f < 2 * d && !st; f++) {
      long n = neighbor(p, e, f);
      if (n < 0) { st = jacobian_boundary(p, &T, e, f, &diag[e * bs], NULL); continue; }
      jacobian_skeleton(p, &T, e, n, f / 2, f % 2, &diag[e * bs], NULL, NULL, NULL, NULL);
    }
  }
  tables_free(&T);
  return st;
}

/* Eigen::PartialPivLU restated: in-place LU with row pivoting.  piv[i] is
   the original row now stored at row i. */
int pdgo_lu_factor(int nb, long nblocks, double *a, int *piv) {
  int st = PDGO_OK;
  for (long b = 0; b < nblocks; b++) {
    double *A = &a[b * (long)nb * nb];
    int *P = &piv[b * nb];
    for (int i = 0; i < nb; i++) P[i] = i;
    for (int c = 0; c < nb; c++) {
      int pr = c;
      double best = fabs(A[c * nb + c]);
      for (int r = c + 1; r < nb; r++)
        if (fabs(A[r * nb + c]) > best) { best = fabs(A[r * nb + c]); pr = r; }
      if (best == 0.0) { st = PDGO_ESINGULAR; continue; }
      if (pr != c) {
        for (int j = 0; j < nb; j++) { double t = A[c * nb + j]; A[c * nb + j] = A[pr * nb + j]; A[pr * nb + j] = t; }
        int t = P[c]; P[c] = P[pr]; P[pr] = t;
      }
      for (int r = c + 1; r < nb; r++) {
        double l = A[r * nb + c] / A[c * nb + c];
        A[r * nb + c] = l;
        for (int j = c + 1; j < nb; j++) A[r * nb + j] -= l * A[c * nb + j];
      }
    }
  }
  return st;
}

/* AssembledBlockJacobiPreconditionerLocalOperator::jacobian_apply_volume
   (backend/istl/matrixfree/assembledblockjacobipreconditioner.hh:202-233):
   forward solve with unit-lower L, backward solve with U. */
void pdgo_lu_apply(int nb, long nblocks, const double *lu, const int *piv,
                   const double *dvec, double *v) {
  double tmp[MAXNB];
  for (long b = 0; b < nblocks; b++) {
    const double *A = &lu[b * (long)nb * nb];
    const int *P = &piv[b * nb];
    const double *z = &dvec[b * nb];
    double *y = &v[b * nb];
    for (int i = 0; i < nb; i++) {
      double rhs = z[P[i]];
      for (int j = 0; j < i; j++) rhs -= A[i * nb + j] * tmp[j];
      tmp[i] = rhs;
    }
    for (int i = nb - 1; i >= 0; i--) {
      double rhs = tmp[i];
      for (int j = nb - 1; j > i; j--) rhs -= A[i * nb + j] * y[j];
      y[i] = rhs / A[i * nb + i];
    }
  }
}

/* ------------------------------------------------------------------ */
/* Krylov solvers                                                      */
/* ------------------------------------------------------------------ */

typedef struct opctx {
  const pdgo_problem *p;
  int op;
  const double *blocks;
  const double *lu;
  const int *piv;
  long n;
  int nb;
  /* optional: block SOR / iterative block Jacobi (pdgo_prec_apply_cfg) */
  const pdgo_prec_config *pc;
  const double *diag;      /* diagonal blocks, row-major */
  const double *ablocks;   /* assembled blocks (SOR coupling) */
  int transpose;
} opctx;

/* OnTheFlyOperator::apply (backend/istl/seqistlsolverbackend.hh:66-76):
   y = 0; jacobian_apply(x, y). */
static int op_apply(const opctx *o, const double *x, double *y) {
  if (o->op == 0) {
    memset(y, 0, sizeof(double) * o->n);
    return pdgo_jacobian_apply(o->p, x, y);
  } else if (o->op == 1) {
    return pdgo_blocks_apply(o->p, o->blocks, x, y);
  }
  return pdgo_blocks_apply_transpose(o->p, o->blocks, x, y);
}
/* OnTheFlyOperator::applyscaleadd (:78-90): temp = J x; y += alpha temp */
static int op_applyscaleadd(const opctx *o, double alpha, const double *x, double *y) {
  double *t = malloc(sizeof(double) * o->n);
  int st = op_apply(o, x, t);
  for (long i = 0; i < o->n; i++) y[i] += alpha * t[i];
  free(t);
  return st;
}
/* GridOperatorPreconditioner::apply (gridoperatorpreconditioner.hh:78-84) */
static void prec_apply(const opctx *o, double *v, const double *dvec) {
  if (o->pc) {
    pdgo_prec_apply_cfg(o->p, o->pc, o->diag, o->lu, o->piv, o->ablocks, o->transpose, dvec, v,
                        NULL);
    return;
  }
  if (o->lu) pdgo_lu_apply(o->nb, o->n / o->nb, o->lu, o->piv, dvec, v);
  else memcpy(v, dvec, sizeof(double) * o->n);
}
static double dot(long n, const double *a, const double *b) {
  double s = 0.0;
  for (long i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* IterativeSolver::Iteration::step (dune-istl): converged when
   def < def0 * reduction or def < 1e-30; non-finite defects abort. */
typedef struct iteration { double def0, def; double i; int converged, valid; } iteration;
static int iter_step(iteration *it, double i, double def, double reduction) {
  if (!isfinite(def)) { it->valid = 0; it->i = i; it->def = def; return 1; }
  if (i == 0) it->def0 = def;
  it->def = def;
  it->i = i;
  it->converged = (def < it->def0 * reduction) || (def < 1e-30);
  return it->converged;
}
static void iter_finalize(const iteration *it, pdgo_result *res) {
  res->converged = it->converged && it->valid;
  res->iterations = (int)ceil(it->i);
  res->reduction = it->def0 > 0 ? it->def / it->def0 : 0.0;
  res->conv_rate = res->iterations > 0 ? pow(res->reduction, 1.0 / res->iterations) : 0.0;
  res->defect = it->def;
  res->first_defect = it->def0;
}

/* dune-istl CGSolver::apply restated */
static int cg_run(const opctx *op_, double *x, double *b, double reduction, int maxit,
                  pdgo_result *res);
static int bicgstab_run(const opctx *op_, double *x, double *b, double reduction, int maxit,
                        pdgo_result *res);

int pdgo_cg(const pdgo_problem *p, int op, const double *blocks, const double *lu,
            const int *piv, double *x, double *b, double reduction, int maxit, pdgo_result *res) {
  opctx o = {p, op, blocks, lu, piv, pdgo_ndof(p), pdgo_nbasis(p), NULL, NULL, NULL, 0};
  return cg_run(&o, x, b, reduction, maxit, res);
}

static int cg_run(const opctx *op_, double *x, double *b, double reduction, int maxit,
                  pdgo_result *res) {
  const opctx o = *op_;
  long n = o.n;
  memset(res, 0, sizeof(*res));
  iteration it = {0, 0, 0, 0, 1};
  int st = op_applyscaleadd(&o, -1.0, x, b);       /* b = b - A x */
  if (st) return st;
  double *pv = malloc(sizeof(double) * n), *q = malloc(sizeof(double) * n);
  double def = sqrt(dot(n, b, b));
  if (iter_step(&it, 0, def, reduction)) { iter_finalize(&it, res); free(pv); free(q); return PDGO_OK; }
  prec_apply(&o, pv, b);
  double rholast = dot(n, pv, b);
  int i = 1;
  for (; i <= maxit; i++) {
    op_apply(&o, pv, q);
    double alpha = dot(n, pv, q);
    double lambda = rholast / alpha;
    for (long j = 0; j < n; j++) x[j] += lambda * pv[j];
    for (long j = 0; j < n; j++) b[j] -= lambda * q[j];
    def = sqrt(dot(n, b, b));
    if (iter_step(&it, i, def, reduction)) break;
    prec_apply(&o, q, b);
    double rho = dot(n, q, b);
    double beta = rho / rholast;
    for (long j = 0; j < n; j++) pv[j] = beta * pv[j] + q[j];
    rholast = rho;
  }
  if (i > maxit) it.i = maxit;
  iter_finalize(&it, res);
  free(pv); free(q);
  return PDGO_OK;
}

/* dune-istl BiCGSTABSolver::apply restated */
int pdgo_bicgstab(const pdgo_problem *p, int op, const double *blocks, const double *lu,
                  const int *piv, double *x, double *b, double reduction, int maxit, pdgo_result *res) {
  opctx o = {p, op, blocks, lu, piv, pdgo_ndof(p), pdgo_nbasis(p), NULL, NULL, NULL, 0};
  return bicgstab_run(&o, x, b, reduction, maxit, res);
}

static int bicgstab_run(const opctx *op_, double *x, double *b, double reduction, int maxit,
                        pdgo_result *res) {
  const opctx o = *op_;
  long n = o.n;
  const double EPSILON = 1e-80;
  memset(res, 0, sizeof(*res));
  iteration iter = {0, 0, 0, 0, 1};
  double *r = b;
  double *pv = calloc(n, sizeof(double)), *v = calloc(n, sizeof(double));
  double *t = calloc(n, sizeof(double)), *y = calloc(n, sizeof(double));
  double *rt = calloc(n, sizeof(double));
  int st = op_applyscaleadd(&o, -1.0, x, r);
  if (st) goto done;
  memcpy(rt, r, sizeof(double) * n);
  double norm = sqrt(dot(n, r, r));
  if (iter_step(&iter, 0, norm, reduction)) goto fin;
  double rho = 1, alpha = 1, omega = 1, rho_new, beta, h;
  double it;
  for (it = 0.5; it < maxit; it += .5) {
    rho_new = dot(n, rt, r);
    if (fabs(rho) <= EPSILON || fabs(omega) <= EPSILON) { st = PDGO_EBREAKDOWN; goto fin; }
    if (it < 1) memcpy(pv, r, sizeof(double) * n);
    else {
      beta = (rho_new / rho) * (alpha / omega);
      for (long j = 0; j < n; j++) pv[j] = beta * (pv[j] - omega * v[j]) + r[j];
    }
    prec_apply(&o, y, pv);
    op_apply(&o, y, v);
    h = dot(n, rt, v);
    if (fabs(h) < EPSILON) { st = PDGO_EBREAKDOWN; goto fin; }
    alpha = rho_new / h;
    for (long j = 0; j < n; j++) x[j] += alpha * y[j];
    for (long j = 0; j < n; j++) r[j] -= alpha * v[j];
    norm = sqrt(dot(n, r, r));
    if (iter_step(&iter, it, norm, reduction)) break;
    it += .5;
    prec_apply(&o, y, r);
    op_apply(&o, y, t);
    omega = dot(n, t, r) / dot(n, t, t);
    for (long j = 0; j < n; j++) x[j] += omega * y[j];
    for (long j = 0; j < n; j++) r[j] -= omega * t[j];
    rho = rho_new;
    norm = sqrt(dot(n, r, r));
    if (iter_step(&iter, it, norm, reduction)) break;
  }
fin:
  iter_finalize(&iter, res);
done:
  free(pv); free(v); free(t); free(y); free(rt);
  res->status = st;
  return st;
}

int pdgo_solve_linear_problem(const pdgo_problem *p, int solver, int op, double *x,
                              double reduction, double min_defect, int maxit, pdgo_result *res) {
  long n = pdgo_ndof(p);
  int nb = pdgo_nbasis(p);
  long nc = pdgo_ncell(p);
  double *r = calloc(n, sizeof(double));
  double *z = calloc(n, sizeof(double));
  double *blocks = NULL, *lu = NULL;
  int *piv = NULL;
  int st = pdgo_residual(p, x, r);
  if (st) goto out;
  double defect = sqrt(dot(n, r, r));
  double red = reduction;
  if (defect > 0 && min_defect / defect > red) red = min_defect / defect;
  if (op != 0) {
    blocks = malloc(sizeof(double) * nc * (2 * p->dim + 1) * nb * nb);
    st = pdgo_assemble_jacobian(p, blocks);
    if (st) goto out;
  }
  /* GridOperatorPreconditioner::pre -> block-diagonal setup + LU
     (assembledblockjacobipreconditioner.hh:162-186) */
  lu = malloc(sizeof(double) * nc * nb * nb);
  piv = malloc(sizeof(int) * nc * nb);
  st = pdgo_block_diagonal(p, lu);
  if (st) goto out;
  if (op == 2) {
    /* transpose each diagonal block for the A^T solve */
    for (long e = 0; e < nc; e++) {
      double *B = &lu[e * nb * nb];
      for (int i = 0; i < nb; i++)
        for (int j = i + 1; j < nb; j++) { double t = B[i * nb + j]; B[i * nb + j] = B[j * nb + i]; B[j * nb + i] = t; }
    }
  }
  st = pdgo_lu_factor(nb, nc, lu, piv);
  if (st) goto out;
  if (solver == 0) st = pdgo_cg(p, op, blocks, lu, piv, z, r, red, maxit, res);
  else st = pdgo_bicgstab(p, op, blocks, lu, piv, z, r, red, maxit, res);
  res->first_defect = defect;
  res->defect = defect * res->reduction;
  for (long i = 0; i < n; i++) x[i] -= z[i];
out:
  free(r); free(z); free(blocks); free(lu); free(piv);
  res->status = st;
  return st;
}

/* ------------------------------------------------------------------ */
/* Matrix-free block preconditioners beyond block Jacobi               */
/* ------------------------------------------------------------------ */

/* dune-istl BiCGSTABSolver on one dense block system D x = d (row-major D,
   D^T with `transpose`), x = 0 initially, preconditioned by
   LocalPointJacobiPreconditioner (iterativeblockjacobipreconditioner.hh:
   28-80): v = weight * d / diag(D) (copy when precond = 0).  As
   IterativeBlockJacobiPreconditionerLocalOperator::jacobian_apply_volume
   (:357-394) drives it; a breakdown ends the solve with the last iterate. */
int pdgo_block_bicgstab(int nb, const double *D, int transpose, const double *d, double *x,
                        double red, int maxit, int precond, double weight, int *iterations) {
  double r[MAXNB], rt[MAXNB], pv[MAXNB], v[MAXNB], t[MAXNB], y[MAXNB], idg[MAXNB];
  const double EPSILON = 1e-80;
  for (int i = 0; i < nb; i++) {
    x[i] = 0.0;
    r[i] = d[i];
    rt[i] = d[i];
    pv[i] = v[i] = 0.0;
    idg[i] = 1.0 / D[i * nb + i];
  }
#define BAPPLY(in, out)                                                         \
  for (int i = 0; i < nb; i++) {                                                \
    double s_ = 0.0;                                                            \
    for (int j = 0; j < nb; j++) s_ += (transpose ? D[j * nb + i] : D[i * nb + j]) * in[j]; \
    out[i] = s_;                                                                \
  }
#define BPREC(in, out)                                                          \
  for (int i = 0; i < nb; i++) out[i] = precond ? weight * in[i] * idg[i] : in[i];
  iteration iter = {0, 0, 0, 0, 1};
  double norm = sqrt(dot(nb, r, r));
  int st = PDGO_OK;
  if (iter_step(&iter, 0, norm, red)) goto fin;
  double rho = 1, alpha = 1, omega = 1, rho_new, beta, h;
  for (double it = 0.5; it < maxit; it += .5) {
    rho_new = dot(nb, rt, r);
    if (fabs(rho) <= EPSILON || fabs(omega) <= EPSILON) { st = PDGO_EBREAKDOWN; iter.i = it; break; }
    if (it < 1) memcpy(pv, r, sizeof(double) * nb);
    else {
      beta = (rho_new / rho) * (alpha / omega);
      for (int j = 0; j < nb; j++) pv[j] = beta * (pv[j] - omega * v[j]) + r[j];
    }
    BPREC(pv, y);
    BAPPLY(y, v);
    h = dot(nb, rt, v);
    if (fabs(h) < EPSILON) { st = PDGO_EBREAKDOWN; iter.i = it; break; }
    alpha = rho_new / h;
    for (int j = 0; j < nb; j++) x[j] += alpha * y[j];
    for (int j = 0; j < nb; j++) r[j] -= alpha * v[j];
    norm = sqrt(dot(nb, r, r));
    if (iter_step(&iter, it, norm, red)) break;
    it += .5;
    BPREC(r, y);
    BAPPLY(y, t);
    omega = dot(nb, t, r) / dot(nb, t, t);
    for (int j = 0; j < nb; j++) x[j] += omega * y[j];
    for (int j = 0; j < nb; j++) r[j] -= omega * t[j];
    rho = rho_new;
    norm = sqrt(dot(nb, r, r));
    if (iter_step(&iter, it, norm, red)) break;
  }
#undef BAPPLY
#undef BPREC
fin:
  if (iterations) *iterations = (int)ceil(iter.i);
  return st;
}

/* One block solve b = scale * D_e^{-1} a of the configured kind. */
static void block_solve_cfg(const pdgo_problem *p, const pdgo_prec_config *pc, const double *diag,
                            const double *lu, const int *piv, int transpose, long e,
                            const double *a, double *b, double scale, int *iters) {
  const int nb = pdgo_nbasis(p);
  const int base = pc->kind & 15;
  if (base == 3) {
    int it = 0;
    pdgo_block_bicgstab(nb, &diag[e * nb * nb], transpose, a, b, pc->block_reduction,
                        pc->block_maxit, pc->block_precondition, pc->block_weight, &it);
    if (iters) iters[e] = it;
  } else if (base == 0 && !lu) {
    for (int i = 0; i < nb; i++) b[i] = a[i];
  } else {
    /* lu / piv hold the factors of D_e (of D_e^T for transposed solves) */
    pdgo_lu_apply(nb, 1, &lu[e * nb * nb], &piv[e * nb], a, b);
  }
  for (int i = 0; i < nb; i++) b[i] *= scale;
}

/* Block Jacobi of the configured block kind, or (kind & 16) one block-SOR
   sweep from v = 0 (BlockSORPreconditionerLocalOperator,
   blocksorpreconditioner.hh:37-296): cells in grid order,
     a = d_e - sum_{n != e} A_en v_n;   v_e = omega D_e^{-1} a
   (unvisited neighbours still hold 0).  The transposed preconditioner runs
   the cells backwards with the transposed blocks. */
int pdgo_prec_apply_cfg(const pdgo_problem *p, const pdgo_prec_config *pc, const double *diag,
                        const double *lu, const int *piv, const double *ablocks, int transpose,
                        const double *d, double *v, int *iters) {
  const int nb = pdgo_nbasis(p), ns = 2 * p->dim + 1;
  const long nc = pdgo_ncell(p), bs = (long)nb * nb;
  double a[MAXNB];
  if (!(pc->kind & 16)) {
    for (long e = 0; e < nc; e++)
      block_solve_cfg(p, pc, diag, lu, piv, transpose, e, &d[e * nb], &v[e * nb], 1.0, iters);
    return PDGO_OK;
  }
  if (!ablocks) return PDGO_EARG;
  memset(v, 0, sizeof(double) * nc * nb);
  for (long q = 0; q < nc; q++) {
    const long e = transpose ? nc - 1 - q : q;
    for (int i = 0; i < nb; i++) a[i] = d[e * nb + i];
    for (int sl = 1; sl < ns; sl++) {
      const long n = neighbor(p, e, sl - 1);
      if (n < 0) continue;
      const double *vn = &v[n * nb];
      if (!transpose) {
        const double *B = &ablocks[(e * ns + sl) * bs];
        for (int i = 0; i < nb; i++) {
          double s = 0.0;
          for (int j = 0; j < nb; j++) s += B[i * nb + j] * vn[j];
          a[i] -= s;
        }
      } else {
        /* (A^T)_(e,n) = (A_(n,e))^T; A_(n,e) sits in n's row at the opposite face */
        const int f = sl - 1, msl = 1 + (f ^ 1);
        const double *B = &ablocks[(n * ns + msl) * bs];
        for (int i = 0; i < nb; i++) {
          double s = 0.0;
          for (int j = 0; j < nb; j++) s += B[j * nb + i] * vn[j];
          a[i] -= s;
        }
      }
    }
    block_solve_cfg(p, pc, diag, lu, piv, transpose, e, a, &v[e * nb], pc->omega, iters);
  }
  return PDGO_OK;
}

/* pdgo_solve_linear_problem with a configured preconditioner (block kind
   0 = none, 1/2 = LU block Jacobi, 3 = iterative block Jacobi; | 16 block
   SOR).  op as for pdgo_solve_linear_problem (op = 2: A^T). */
int pdgo_solve_linear_problem_prec(const pdgo_problem *p, int solver, int op,
                                   const pdgo_prec_config *pc, double *x, double reduction,
                                   double min_defect, int maxit, pdgo_result *res) {
  long n = pdgo_ndof(p);
  int nb = pdgo_nbasis(p);
  long nc = pdgo_ncell(p);
  const int transpose = op == 2;
  double *r = calloc(n, sizeof(double));
  double *z = calloc(n, sizeof(double));
  double *ablocks = malloc(sizeof(double) * nc * (2 * p->dim + 1) * nb * nb);
  double *diag = malloc(sizeof(double) * nc * nb * nb);
  double *lu = NULL;
  int *piv = NULL;
  int st = pdgo_residual(p, x, r);
  if (st) goto out;
  double defect = sqrt(dot(n, r, r));
  double red = reduction;
  if (defect > 0 && min_defect / defect > red) red = min_defect / defect;
  st = pdgo_assemble_jacobian(p, ablocks);
  if (st) goto out;
  st = pdgo_block_diagonal(p, diag);
  if (st) goto out;
  const int base = pc->kind & 15;
  if (base == 1 || base == 2) {
    lu = malloc(sizeof(double) * nc * nb * nb);
    piv = malloc(sizeof(int) * nc * nb);
    memcpy(lu, diag, sizeof(double) * nc * nb * nb);
    if (transpose)
      for (long e = 0; e < nc; e++) {
        double *B = &lu[e * nb * nb];
        for (int i = 0; i < nb; i++)
          for (int j = i + 1; j < nb; j++) { double t = B[i * nb + j]; B[i * nb + j] = B[j * nb + i]; B[j * nb + i] = t; }
      }
    st = pdgo_lu_factor(nb, nc, lu, piv);
    if (st) goto out;
  }
  opctx o = {p, op, op ? ablocks : NULL, lu, piv, n, nb, pc, diag, ablocks, transpose};
  if (solver == 0) st = cg_run(&o, z, r, red, maxit, res);
  else st = bicgstab_run(&o, z, r, red, maxit, res);
  res->first_defect = defect;
  res->defect = defect * res->reduction;
  for (long i = 0; i < n; i++) x[i] -= z[i];
out:
  free(r); free(z); free(ablocks); free(diag); free(lu); free(piv);
  res->status = st;
  return st;
}

int pdgo_mass_apply(const pdgo_problem *p, const double *x, double *y) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  const int d = T.d, nb = T.nb;
  const long nc = pdgo_ncell(p);
  double detJ = 1.0;
  for (int j = 0; j < d; j++) detJ *= cell_h(p, j);
  for (long e = 0; e < nc; e++) {
    double *ye = &y[e * nb];
    for (int i = 0; i < nb; i++) ye[i] = 0.0;
    for (int q = 0; q < T.nqv; q++) {
      const double *phi = &T.vphi[q * nb];
      double u = 0.0;
      for (int i = 0; i < nb; i++) u += x[e * nb + i] * phi[i];
      for (int i = 0; i < nb; i++) ye[i] += u * phi[i] * T.vw[q] * detJ;
    }
  }
  tables_free(&T);
  return PDGO_OK;
}

/* per-cell mass block (identical for all cells of the uniform grid) */
static int mass_block(const pdgo_problem *p, double *Mb) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  const int d = T.d, nb = T.nb;
  double detJ = 1.0;
  for (int j = 0; j < d; j++) detJ *= cell_h(p, j);
  memset(Mb, 0, sizeof(double) * nb * nb);
  for (int q = 0; q < T.nqv; q++) {
    const double *phi = &T.vphi[q * nb];
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) Mb[i * nb + j] += phi[i] * phi[j] * T.vw[q] * detJ;
  }
  tables_free(&T);
  return PDGO_OK;
}

int pdgo_onestep(pdgo_problem *p, int s, const double *A, const double *B, double dt,
                 int solver, const pdgo_prec_config *pc, double reduction, int maxit,
                 const double *xold, double *xnew, int *linear_iterations) {
  const long n = pdgo_ndof(p), nc = pdgo_ncell(p);
  const int nb = pdgo_nbasis(p);
  if (s < 1 || s > 4) return PDGO_EARG;
  double *X[5], *RX[5], *MX[5];
  for (int j = 0; j <= s; j++) {
    X[j] = j == 0 ? (double *)xold : (j == s ? xnew : calloc(n, sizeof(double)));
    RX[j] = calloc(n, sizeof(double));
    MX[j] = calloc(n, sizeof(double));
  }
  double *Cv = calloc(n, sizeof(double)), *r = calloc(n, sizeof(double));
  double *z = calloc(n, sizeof(double)), *cs = calloc(nc, sizeof(double));
  double *Mb = malloc(sizeof(double) * nb * nb), *Mlu = NULL, *diag = NULL, *lu = NULL;
  double *ablocks = NULL;
  int *Mpiv = malloc(sizeof(int) * nb), *piv = NULL;
  const double *c_orig = p->c;
  int st = mass_block(p, Mb);
  if (st) goto out;
  Mlu = malloc(sizeof(double) * nb * nb);
  memcpy(Mlu, Mb, sizeof(double) * nb * nb);
  st = pdgo_lu_factor(nb, 1, Mlu, Mpiv);
  if (st) goto out;
  if (linear_iterations) *linear_iterations = 0;
  /* R(x_0), M x_0 with the original coefficients */
  st = pdgo_residual(p, X[0], RX[0]);
  if (st) goto out;
  pdgo_mass_apply(p, X[0], MX[0]);
  for (int rr = 1; rr <= s; rr++) {
    const double *a = A + (rr - 1) * (s + 1), *b = B + (rr - 1) * (s + 1);
    memset(Cv, 0, sizeof(double) * n);
    for (int j = 0; j < rr; j++)
      for (long i = 0; i < n; i++) Cv[i] += b[j] * dt * RX[j][i] + a[j] * MX[j][i];
    const double arr = a[rr], brr = b[rr];
    if (brr == 0.0) {
      for (long i = 0; i < n; i++) Cv[i] *= -1.0 / arr;
      pdgo_lu_apply(nb, 1, Mlu, Mpiv, Cv, X[rr]);   /* one block at a time */
      for (long e = 1; e < nc; e++) pdgo_lu_apply(nb, 1, Mlu, Mpiv, &Cv[e * nb], &X[rr][e * nb]);
    } else {
      const double sigma = arr / (brr * dt);
      for (long e = 0; e < nc; e++) cs[e] = (c_orig ? c_orig[e] : 0.0) + sigma;
      p->c = cs;
      /* preconditioner on the shifted operator */
      free(diag); free(lu); free(piv); free(ablocks);
      diag = malloc(sizeof(double) * nc * nb * nb);
      lu = NULL; piv = NULL; ablocks = NULL;
      st = pdgo_block_diagonal(p, diag);
      if (st) goto out;
      const int base = pc->kind & 15;
      if (base == 1 || base == 2) {
        lu = malloc(sizeof(double) * nc * nb * nb);
        piv = malloc(sizeof(int) * nc * nb);
        memcpy(lu, diag, sizeof(double) * nc * nb * nb);
        st = pdgo_lu_factor(nb, nc, lu, piv);
        if (st) goto out;
      }
      if (pc->kind & 16) {
        ablocks = malloc(sizeof(double) * nc * (2 * p->dim + 1) * nb * nb);
        st = pdgo_assemble_jacobian(p, ablocks);
        if (st) goto out;
      }
      memcpy(X[rr], X[rr - 1], sizeof(double) * n);
      memset(r, 0, sizeof(double) * n);
      st = pdgo_residual(p, X[rr], r);            /* J_sigma x + R(0) */
      if (st) goto out;
      for (long i = 0; i < n; i++) r[i] += Cv[i] / (brr * dt);
      memset(z, 0, sizeof(double) * n);
      opctx oc = {p, 0, NULL, lu, piv, n, nb, pc, diag, ablocks, 0};
      pdgo_result lr;
      st = solver == 0 ? cg_run(&oc, z, r, reduction, maxit, &lr)
                       : bicgstab_run(&oc, z, r, reduction, maxit, &lr);
      if (linear_iterations) *linear_iterations += lr.iterations;
      if (st) goto out;
      for (long i = 0; i < n; i++) X[rr][i] -= z[i];
      p->c = c_orig;
    }
    if (rr < s) {
      p->c = c_orig;
      st = pdgo_residual(p, X[rr], RX[rr]);
      if (st) goto out;
      pdgo_mass_apply(p, X[rr], MX[rr]);
    }
  }
out:
  p->c = c_orig;
  for (int j = 0; j <= s; j++) {
    if (j != 0 && j != s) free(X[j]);
    free(RX[j]);
    free(MX[j]);
  }
  free(Cv); free(r); free(z); free(cs); free(Mb); free(Mlu); free(Mpiv);
  free(diag); free(lu); free(piv); free(ablocks);
  return st;
}

/* NewtonMethod::apply (solver/newton.hh:177-335) restated. */
int pdgo_newton(pdgo_problem *p, int solver, const pdgo_prec_config *pc,
                const pdgo_newton_opts *o, double *x, pdgo_newton_result *res) {
  const long n = pdgo_ndof(p), nc = pdgo_ncell(p);
  const int nb = pdgo_nbasis(p);
  memset(res, 0, sizeof(*res));
  double *r = calloc(n, sizeof(double)), *z = calloc(n, sizeof(double));
  double *xprev = calloc(n, sizeof(double)), *xl = calloc(n, sizeof(double));
  double *diag = NULL, *lu = NULL, *ablocks = NULL;
  int *piv = NULL;
  int st = PDGO_OK, prec_ready = 0;
  double defect = 0.0;
  const double *saved = p->xlin;
#define UPDATE_DEFECT()                                   \
  do {                                                    \
    memset(r, 0, sizeof(double) * n);                     \
    st = pdgo_residual(p, x, r);                          \
    defect = sqrt(dot(n, r, r));                          \
  } while (0)
  UPDATE_DEFECT();
  if (st) goto out;
  res->first_defect = defect;
  double prev = defect;
  for (;;) {
    if (!(o->force_iteration && res->iterations == 0)) {
      res->converged = defect < o->absolute_limit || defect < res->first_defect * o->reduction;
      if (res->converged) break;
      if (res->iterations >= o->max_iterations) { st = PDGO_ENOTCONV; goto out; }
    }
    if (!isfinite(defect)) { st = PDGO_ENOTCONV; goto out; }
    double linred = o->min_linear_reduction;
    if (!o->fixed_linear_reduction &&
        !(res->iterations == 0 && res->first_defect < o->absolute_limit)) {
      double stop = fmax(res->first_defect * o->reduction, o->absolute_limit);
      linred = fmax(stop / (10 * defect), fmin(o->min_linear_reduction, defect * defect / (prev * prev)));
    }
    prev = defect;
    memcpy(xl, x, sizeof(double) * n);
    p->xlin = xl;
    if (!prec_ready) {
      diag = malloc(sizeof(double) * nc * nb * nb);
      st = pdgo_block_diagonal(p, diag);
      if (st) goto out;
      const int base = pc->kind & 15;
      if (base == 1 || base == 2) {
        lu = malloc(sizeof(double) * nc * nb * nb);
        piv = malloc(sizeof(int) * nc * nb);
        memcpy(lu, diag, sizeof(double) * nc * nb * nb);
        st = pdgo_lu_factor(nb, nc, lu, piv);
        if (st) goto out;
      }
      if (pc->kind & 16) {
        ablocks = malloc(sizeof(double) * nc * (2 * p->dim + 1) * nb * nb);
        st = pdgo_assemble_jacobian(p, ablocks);
        if (st) goto out;
      }
      prec_ready = 1;
    }
    memset(z, 0, sizeof(double) * n);
    {
      opctx oc = {p, 0, NULL, lu, piv, n, nb, pc, diag, ablocks, 0};
      pdgo_result lr;
      int ls = solver == 0 ? cg_run(&oc, z, r, linred, o->linear_maxit, &lr)
                           : bicgstab_run(&oc, z, r, linred, o->linear_maxit, &lr);
      res->linear_iterations += lr.iterations;
      if (ls != PDGO_OK) { st = ls; goto out; }
    }
    if (!o->line_search || defect < o->absolute_limit) {
      for (long i = 0; i < n; i++) x[i] -= z[i];
      UPDATE_DEFECT();
      if (st) goto out;
    } else {
      double lambda = 1.0, best_lambda = 0.0, best = defect, previous = defect;
      int ok = 0;
      memcpy(xprev, x, sizeof(double) * n);
      for (int it = 0; it < o->line_search_max_iterations; it++) {
        for (long i = 0; i < n; i++) x[i] -= lambda * z[i];
        UPDATE_DEFECT();
        if (st) goto out;
        if (defect <= (1.0 - lambda / 4) * previous) { ok = 1; break; }
        if (defect < best) { best = defect; best_lambda = lambda; }
        lambda *= o->line_search_damping;
        memcpy(x, xprev, sizeof(double) * n);
      }
      if (!ok) {
        if (!o->line_search_accept_best || best_lambda == 0.0) {
          memcpy(x, xprev, sizeof(double) * n);
          UPDATE_DEFECT();
          st = PDGO_ENOTCONV;
          goto out;
        }
        if (best_lambda != lambda) {
          memcpy(x, xprev, sizeof(double) * n);
          for (long i = 0; i < n; i++) x[i] -= best_lambda * z[i];
          UPDATE_DEFECT();
          if (st) goto out;
        }
      }
    }
    res->iterations++;
    res->defect = defect;
    res->reduction = defect / res->first_defect;
    res->conv_rate = pow(res->reduction, 1.0 / res->iterations);
  }
#undef UPDATE_DEFECT
out:
  res->defect = defect;
  if (res->first_defect > 0) res->reduction = defect / res->first_defect;
  res->status = st;
  p->xlin = saved;
  free(r); free(z); free(xprev); free(xl); free(diag); free(lu); free(piv); free(ablocks);
  return st;
}

int pdgo_eval_points(const pdgo_problem *p, const double *u, int m, double *xyz, double *w, double *val) {
  int d = p->dim, k = p->k, nb = pdgo_nbasis(p);
  if (m < 1 || m > 32) return PDGO_EARG;
  double gx[32], gw[32];
  pdgo_gauss_legendre(m, gx, gw);
  long nc = pdgo_ncell(p);
  int mq = 1;
  for (int j = 0; j < d; j++) mq *= m;
  double phi[MAXNB], js[MAXNB * MAXD];
  double h[MAXD], detJ = 1.0;
  for (int j = 0; j < d; j++) { h[j] = cell_h(p, j); detJ *= h[j]; }
  for (long e = 0; e < nc; e++) {
    int ix[MAXD];
    cell_index(p, e, ix);
    for (int q = 0; q < mq; q++) {
      double loc[MAXD];
      double wt = 1.0;
      int t = q;
      for (int j = 0; j < d; j++) { int a = t % m; t /= m; loc[j] = gx[a]; wt *= gw[a]; }
      eval_basis(p->basis, d, k, loc, phi, js);
      double s = 0.0;
      for (int i = 0; i < nb; i++) s += u[e * nb + i] * phi[i];
      val[e * mq + q] = s;
      w[e * mq + q] = wt * detJ;
      for (int j = 0; j < d; j++) xyz[(e * mq + q) * d + j] = (ix[j] + loc[j]) * h[j];
    }
  }
  return PDGO_OK;
}

/* Gradient of J w.r.t. log K from assembled local blocks at unit
   coefficient.  With weightsOn every diffusion term of a face is
   proportional to H = 2 Ks Kn / (Ks + Kn + 1e-20) (:326-346), the volume
   term to K_e (:124-127) and the Dirichlet face terms to K_s (:720-734). */
int pdgo_grad_logK(const pdgo_problem *p, const double *u, const double *lam, double *g) {
  /* defined for A = K I with K per cell only */
  if (p->weights != PDGO_WEIGHTS_ON || p->Acell || pointwise_A(p)) return PDGO_EARG;
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int d = T.d, nb = T.nb;
  long nc = pdgo_ncell(p), bs = (long)nb * nb;
  double *m1 = malloc(sizeof(double) * bs), *m2 = malloc(sizeof(double) * bs);
  double *m3 = malloc(sizeof(double) * bs), *m4 = malloc(sizeof(double) * bs);
  double *rb = malloc(sizeof(double) * nb);
  coef_override unit = {1, 1.0, 1.0};
  int st = PDGO_OK;
  for (long e = 0; e < nc; e++) g[e] = 0.0;
  for (long e = 0; e < nc && !st; e++) {
    const double *ue = &u[e * nb], *le = &lam[e * nb];
    double Ke = Kof(p, e);
    /* volume */
    memset(m1, 0, sizeof(double) * bs);
    jacobian_volume(p, &T, e, m1, &unit);
    double s = 0.0;
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) s += le[i] * m1[i * nb + j] * ue[j];
    g[e] -= Ke * s;
    for (int f = 0; f < 2 * d; f++) {
      long n = neighbor(p, e, f);
      if (n < 0) {
        /* Dirichlet boundary: residual form incl. g, unit K, no convection */
        for (int i = 0; i < nb; i++) rb[i] = 0.0;
        st = boundary_integral(p, &T, e, f, ue, rb, 0, &unit);
        double sb = 0.0;
        for (int i = 0; i < nb; i++) sb += le[i] * rb[i];
        g[e] -= Ke * sb;
        continue;
      }
      if (!(e > n)) continue;
      memset(m1, 0, sizeof(double) * bs); memset(m2, 0, sizeof(double) * bs);
      memset(m3, 0, sizeof(double) * bs); memset(m4, 0, sizeof(double) * bs);
      jacobian_skeleton(p, &T, e, n, f / 2, f % 2, m1, m2, m3, m4, &unit);
      const double *un = &u[n * nb], *ln = &lam[n * nb];
      double a = 0.0;
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < nb; j++)
          a += le[i] * (m1[i * nb + j] * ue[j] + m2[i * nb + j] * un[j]) +
               ln[i] * (m3[i * nb + j] * ue[j] + m4[i * nb + j] * un[j]);
      double Ks = Ke, Kn = Kof(p, n);
      double S = Ks + Kn + 1e-20;
      double dH_dKs = 2.0 * Kn * (Kn + 1e-20) / (S * S);
      double dH_dKn = 2.0 * Ks * (Ks + 1e-20) / (S * S);
      g[e] -= Ks * dH_dKs * a;
      g[n] -= Kn * dH_dKn * a;
    }
  }
  free(m1); free(m2); free(m3); free(m4); free(rb);
  tables_free(&T);
  return st;
}

/* dR/dfc_e = -int_e psi_i (lambda_volume, :1047-1075) */
int pdgo_grad_fc(const pdgo_problem *p, const double *lam, double *g) {
  tables T;
  if (tables_init(p, &T)) return PDGO_EARG;
  int nb = T.nb;
  long nc = pdgo_ncell(p);
  double detJ = 1.0;
  for (int j = 0; j < T.d; j++) detJ *= cell_h(p, j);
  for (long e = 0; e < nc; e++) {
    double s = 0.0;
    for (int q = 0; q < T.nqv; q++) {
      const double *phi = &T.vphi[q * nb];
      double factor = T.vw[q] * detJ;
      for (int i = 0; i < nb; i++) s += lam[e * nb + i] * phi[i] * factor;
    }
    g[e] = s;
  }
  tables_free(&T);
  return PDGO_OK;
}
