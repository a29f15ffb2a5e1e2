// pdg_abi.cu -- the C ABI (include/pdg.h): context, 1D tables, parameter
// uploads, operator entry points, and the device-resident Krylov drivers.
//
// Solver semantics follow the reference's call chain:
//   StationaryLinearProblemSolver::apply   (stationary/linearproblem.hh:188-302)
//   ISTLBackend_SEQ_MatrixFree_Base::apply (backend/istl/matrixfree/backends.hh:116-126)
//   OnTheFlyOperator / GridOperatorPreconditioner (seqistlsolverbackend.hh:45-100,
//     matrixfree/gridoperatorpreconditioner.hh:45-84)
// with dune-istl's CGSolver / BiCGSTABSolver recurrences (external to the
// reference; restated from the published algorithms).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pdg_gmres.cuh"
#include "pdg_internal.cuh"
#include "pdg_vec.cuh"

namespace pdg {

static thread_local std::string g_err;

int set_error(int status, const std::string &msg) {
  g_err = msg;
  return status;
}


// Lagrange basis at equidistant nodes j/k, as QkStuff::p / dp
// (finiteelement/qkdglagrange.hh:55-79).
static double lag(int k, int i, double x) {
  double r = 1.0;
  for (int j = 0; j <= k; j++)
    if (j != i) r *= (k * x - j) / (i - j);
  return r;
}
static double dlag(int k, int i, double x) {
  double r = 0.0;
  for (int j = 0; j <= k; j++)
    if (j != i) {
      double prod = (k * 1.0) / (i - j);
      for (int l = 0; l <= k; l++)
        if (l != i && l != j) prod *= (k * x - l) / (i - l);
      r += prod;
    }
  return r;
}

// The nodal basis the kernels work in: Lagrange polynomials on the Gauss-
// Lobatto points for PDG_BASIS_LOBATTO (GaussLobattoLagrangePolynomials::p /
// dp, finiteelement/qkdglobatto.hh:69-107), else on the equidistant nodes
// (the Legendre basis maps onto the latter, pdg_basis.cu).
static double nlag(const pdg_context *c, int i, double x) {
  if (c->basis != PDG_BASIS_LOBATTO) return lag(c->k, i, x);
  const double *xi = c->nodes;
  double r = 1.0;
  for (int j = 0; j <= c->k; j++)
    if (j != i) r *= (x - xi[j]) / (xi[i] - xi[j]);
  return r;
}
static double ndlag(const pdg_context *c, int i, double x) {
  if (c->basis != PDG_BASIS_LOBATTO) return dlag(c->k, i, x);
  const double *xi = c->nodes;
  double r = 0.0;
  for (int j = 0; j <= c->k; j++)
    if (j != i) {
      double prod = 1.0 / (xi[i] - xi[j]);
      for (int l = 0; l <= c->k; l++)
        if (l != i && l != j) prod *= (x - xi[l]) / (xi[i] - xi[l]);
      r += prod;
    }
  return r;
}

// Gauss-Lobatto points on [0,1], ascending (the rule of the Lobatto basis,
// qkdglobatto.hh:27-67): the end points and the roots of P'_n, n = m-1, by
// Newton's method on P'_n with P''_n from Legendre's equation
// (1-z^2) P''_n = 2 z P'_n - n(n+1) P_n, started at cos(pi j/n).
static void gauss_lobatto_points(int m, double *x) {
  const int n = m - 1;
  for (int j = 0; j <= n; j++) {
    long double z = cosl(3.14159265358979323846264338327950288L * j / n);
    if (j > 0 && j < n) {
      for (int it = 0; it < 100; it++) {
        long double p0 = 1.0L, p1 = 0.0L;
        for (int i = 1; i <= n; i++) {
          const long double p2 = p1;
          p1 = p0;
          p0 = ((2.0L * i - 1.0L) * z * p1 - (i - 1.0L) * p2) / i;
        }
        const long double dp = n * (p1 - z * p0) / (1.0L - z * z);
        const long double d2 = (2.0L * z * dp - n * (n + 1.0L) * p0) / (1.0L - z * z);
        const long double dz = dp / d2;
        z -= dz;
        if (fabsl(dz) < 1e-19L) break;
      }
    }
    x[j] = (double)((1.0L - z) * 0.5L);
  }
  x[0] = 0.0;
  x[n] = 1.0;
}

// Legendre polynomials on [0,1] at x (DGLegendreLocalBasis's 1D factors,
// qkdglegendre.hh:80-88): P_0 = 1, P_1 = 2x-1, recurrence in n.
static void legendre01(int k, double x, double *v) {
  v[0] = 1.0;
  if (k >= 1) v[1] = 2 * x - 1;
  for (int n = 2; n <= k; n++)
    v[n] = ((2 * n - 1) * (2 * x - 1) * v[n - 1] - (n - 1) * v[n - 2]) / n;
}

// T[j][i] = P_i(j/k) and its inverse (Gauss-Jordan with partial pivoting),
// row-major, into t[0 .. N*N) and t[N*N .. 2 N*N)
static void legendre_change_of_basis(int k, double *t) {
  const int N = k + 1;
  double a[kMaxN1][2 * kMaxN1];
  for (int j = 0; j < N; j++) {
    double v[kMaxN1];
    legendre01(k, (double)j / k, v);
    for (int i = 0; i < N; i++) {
      t[j * N + i] = v[i];
      a[j][i] = v[i];
      a[j][N + i] = i == j ? 1.0 : 0.0;
    }
  }
  for (int c = 0; c < N; c++) {
    int piv = c;
    for (int r = c + 1; r < N; r++)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    for (int q = 0; q < 2 * N; q++) std::swap(a[c][q], a[piv][q]);
    const double inv = 1.0 / a[c][c];
    for (int q = 0; q < 2 * N; q++) a[c][q] *= inv;
    for (int r = 0; r < N; r++)
      if (r != c) {
        const double f = a[r][c];
        for (int q = 0; q < 2 * N; q++) a[r][q] -= f * a[c][q];
      }
  }
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) t[N * N + j * N + i] = a[j][N + i];
}
// Gauss-Legendre points/weights on [0,1] (Newton on P_m, long double).
static void gauss_legendre(int m, double *x, double *w) {
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
    long double p0 = 1.0L, p1 = 0.0L;
    for (int j = 1; j <= m; j++) {
      long double p2 = p1;
      p1 = p0;
      p0 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p2) / j;
    }
    dp = m * (z * p0 - p1) / (z * z - 1.0L);
    x[i] = (double)((1.0L - z) * 0.5L);
    w[i] = (double)(1.0L / ((1.0L - z * z) * dp * dp));
  }
}

double lagrange_derivative(const pdg_context *ctx, int i, double x) { return ndlag(ctx, i, x); }

RhsTables make_rhs_tables(const pdg_context *ctx) {
  RhsTables t;
  std::memset(&t, 0, sizeof(t));
  const int N = ctx->N;
  gauss_legendre(N, t.x, t.w);
  for (int q = 0; q < N; q++)
    for (int a = 0; a < N; a++) t.B[q * N + a] = nlag(ctx, a, t.x[q]);
  for (int a = 0; a < N; a++) {
    t.d0[a] = ndlag(ctx, a, 0.0);
    t.d1[a] = ndlag(ctx, a, 1.0);
  }
  return t;
}

double *rhs_r0K(pdg_context *ctx, bool alloc) {
  if (!ctx->r0K && alloc) {
    if (cudaMalloc(&ctx->r0K, sizeof(double) * ctx->ndof) != cudaSuccess) {
      ctx->r0K = nullptr;
      return nullptr;
    }
  }
  return ctx->r0K;
}

template <typename T> static const T *Kp(const pdg_context *c);
template <> const double *Kp<double>(const pdg_context *c) { return c->K64; }
template <> const float *Kp<float>(const pdg_context *c) { return c->K32; }
template <typename T> static const T *Cp(const pdg_context *c);
template <> const double *Cp<double>(const pdg_context *c) { return c->c64; }
template <> const float *Cp<float>(const pdg_context *c) { return c->c32; }
template <typename T> static const T *Tp(const pdg_context *c);
template <> const double *Tp<double>(const pdg_context *c) { return c->tab64; }
template <> const float *Tp<float>(const pdg_context *c) { return c->tab32; }

template <typename T>
static int op_launch(pdg_context *ctx, const T *x, T *y, const T *add, T alpha, int acc,
                     int transpose, const int *skip) {
  if (std::is_same<T, double>::value && ctx->use_matrix)
    return matrix_apply(ctx, (const double *)x, (double *)y, (const double *)add,
                        (double)alpha, acc, transpose, skip);
  if (std::is_same<T, double>::value && ctx->ops32) {
    // FP64 Krylov vectors, FP32 operator: convert, apply in FP32, combine in FP64
    float *s0 = ctx->w32[0], *s1 = ctx->w32[1];
    PDG_TRY(vec_to_f32_skip(ctx, ctx->ndof, (const double *)x, s0, skip));
    ApplyArgs<float> a{s0, s1, nullptr, 1.f, 0, transpose, 0, skip};
    PDG_TRY(launch_apply<float>(ctx, a, ctx->K32, ctx->c32, ctx->tab32));
    return vec_from_f32_combine(ctx, ctx->ndof, s1, (double *)y, (const double *)add,
                                (double)alpha, acc, skip);
  }
  ApplyArgs<T> a{x, y, add, alpha, acc, transpose, 0, skip};
  return launch_apply<T>(ctx, a, Kp<T>(ctx), Cp<T>(ctx), Tp<T>(ctx));
}

// preconditioner inside a Krylov solve (FP32 block Jacobi under ctx->ops32)
template <typename T>
static int prec_op(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip) {
  if (std::is_same<T, double>::value && ctx->ops32) {
    float *s0 = ctx->w32[0], *s1 = ctx->w32[1];
    PDG_TRY(vec_to_f32_skip(ctx, ctx->ndof, (const double *)d, s0, skip));
    PDG_TRY(prec_apply_skip<float>(ctx, s0, s1, transpose, skip));
    return vec_from_f32_combine(ctx, ctx->ndof, s1, (double *)v, nullptr, 1.0, 0, skip);
  }
  return prec_apply_skip<T>(ctx, d, v, transpose, skip);
}

static int ensure_r0(pdg_context *ctx) {
  if (!ctx->r0_valid) {
    PDG_TRY(launch_rhs(ctx));
    if (ctx->basis == PDG_BASIS_LEGENDRE) {
      // R(0) is a residual: r_L = T^T r_nodal per cell (the K-proportional
      // part kept for the log-K gradient stays nodal, it meets nodal lambda)
      PDG_TRY(basis_change<double>(ctx, 0, 1, ctx->r0, ctx->legw64[0], 1.0, 0, nullptr,
                                   nullptr));
      PDG_CUDA_TRY(cudaMemcpyAsync(ctx->r0, ctx->legw64[0], sizeof(double) * ctx->ndof,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ctx->r0_valid = 1;
  }
  return PDG_OK;
}

static int ensure_work(pdg_context *ctx, bool f32) {
  for (int i = 0; i < (f32 ? 10 : 8); i++)
    if (!ctx->w64[i]) PDG_CUDA_TRY(cudaMalloc(&ctx->w64[i], sizeof(double) * ctx->ndof));
  if (f32)
    for (int i = 0; i < 8; i++)
      if (!ctx->w32[i]) PDG_CUDA_TRY(cudaMalloc(&ctx->w32[i], sizeof(float) * ctx->ndof));
  return PDG_OK;
}

static RedCtx red_ctx(pdg_context *ctx) {
  return RedCtx{ctx->red_partials, ctx->red_out, ctx->d_flag};
}

// pinned host mirror: h_red[0..S_COUNT) scalars, then F_COUNT ints
static int fetch_state(pdg_context *ctx, double *scal, int *flags) {
  PDG_CUDA_TRY(cudaMemcpyAsync(ctx->h_red, ctx->red_out, sizeof(double) * S_COUNT,
                               cudaMemcpyDeviceToHost, ctx->stream));
  int *hf = reinterpret_cast<int *>(ctx->h_red + S_COUNT);
  PDG_CUDA_TRY(cudaMemcpyAsync(hf, ctx->d_flag, sizeof(int) * F_COUNT, cudaMemcpyDeviceToHost,
                               ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (scal) std::memcpy(scal, ctx->h_red, sizeof(double) * S_COUNT);
  if (flags) std::memcpy(flags, hf, sizeof(int) * F_COUNT);
  if (hf[F_TMA]) return set_error(PDG_ETIMEOUT, "TMA staging of the FP32 operator timed out");
  return PDG_OK;
}

__global__ void k_set_scal(double *scal, int slot, double v) { scal[slot] = v; }
__global__ void k_init_solve(double *scal, int *flags, double red, double guard = 0.0) {
  for (int i = 0; i < S_COUNT; i++) scal[i] = 0.0;
  scal[S_RED] = red;
  scal[S_GUARD] = guard;
  scal[S_RHO] = 1.0;
  scal[S_ALPHA] = 1.0;
  scal[S_OMEGA] = 1.0;
  flags[F_STATE] = 0;
  flags[F_COUNTER] = 0;
  flags[F_XPEND] = 0;
  flags[F_TMA] = 0;   // a staging timeout is reported by the solve it happened in only
}

template <typename T>
static int dot(pdg_context *ctx, const RedCtx &rc, const T *a, const T *b, const T *c,
               const T *d, int fin, int s0, int s1, bool respect) {
  if (std::is_same<T, double>::value)
    return red_dot(ctx, rc, ctx->ndof, (const double *)a, (const double *)b, (const double *)c,
                   (const double *)d, fin, s0, s1, respect);
  return red_dot_f32(ctx, rc, ctx->ndof, (const float *)a, (const float *)b, (const float *)c,
                     (const float *)d, fin, s0, s1, respect);
}

struct KrylovOut {
  int state;       // 0 running/maxit, 1 converged, 2 non-finite, 3 breakdown
  int iterations;
  double def0, def;
};

// The inner FP32 CG can fuse its two dot products into the kernels that
// produce one operand: <p, q> into the staged FP32 operator writing q = A p,
// <z, r> into the FDM block Jacobi writing z = M^{-1} r.  Only where those are
// the kernels that run: 3D, degree <= 3, plain diffusion-reaction operator
// (no convection, nonlinear term, modal basis or assembled matrix) and the
// FDM block Jacobi.
static bool cg_fusable(const pdg_context *ctx) {
  return ctx->dim == 3 && ctx->N <= 4 && !convection_on(ctx) && ctx->nl_deg == 0 &&
         !general_coefficients(ctx) &&
         ctx->basis != PDG_BASIS_LEGENDRE && !ctx->use_matrix &&
         ctx->prec[PDG_F32].ready && ctx->prec[PDG_F32].kind == PDG_PREC_BJ_FDM;
}

// FP64 CG with three launches per iteration on 2D grids (<p, A p> in the
// operator, the residual update and <M^-1 r, r> in the FDM block Jacobi): 2D
// grids are small and launch-bound.  In 3D the FP64 kernels are bound by the
// FP64 pipe, and the fused products made the 64^3 Q2 iteration slower.
static bool cg_fusable64(const pdg_context *ctx, int transpose) {
  return !transpose && ctx->dim == 2 && !convection_on(ctx) && ctx->nl_deg == 0 &&
         !general_coefficients(ctx) && ctx->basis != PDG_BASIS_LEGENDRE && !ctx->use_matrix &&
         !ctx->ops32 && ctx->prec[PDG_F64].ready && ctx->prec[PDG_F64].kind == PDG_PREC_BJ_FDM;
}

static int ensure_fuse(pdg_context *ctx) {
  if (ctx->fuse_part) return PDG_OK;
  // the fused kernels run at least 5 cells per block
  const long maxb = ctx->ncell / 5 + 2;
  const long ngroups = (maxb + kFuseGroup - 1) / kFuseGroup;
  PDG_CUDA_TRY(cudaMalloc(&ctx->fuse_part, sizeof(double) * 2 * (maxb + ngroups)));
  PDG_CUDA_TRY(cudaMalloc(&ctx->fuse_cnt, sizeof(int) * ngroups));
  PDG_CUDA_TRY(cudaMemsetAsync(ctx->fuse_cnt, 0, sizeof(int) * ngroups, ctx->stream));
  ctx->fuse_max_blocks = maxb;
  return PDG_OK;
}

// dune-istl CGSolver::apply restated on the device.  x: initial guess and
// result; b: right-hand side, overwritten by the defect.  w0, w1: work.
template <typename T>
static int cg_device(pdg_context *ctx, T *x, T *b, T *p, T *q, double reduction, int maxit,
                     int transpose, KrylovOut *out) {
  const RedCtx rc = red_ctx(ctx);
  const int *skip = ctx->d_flag + F_STATE;
  k_init_solve<<<1, 1, 0, ctx->stream>>>(rc.scal, rc.flags, reduction);
  // b -= A x   (applyscaleadd(-1, x, b))
  PDG_TRY(op_launch<T>(ctx, x, b, nullptr, T(-1), 1, transpose, nullptr));
  PDG_TRY(dot<T>(ctx, rc, b, b, nullptr, nullptr, FIN_DEF0, -1, -1, false));
  // p = M^{-1} b ; rholast = <p, b>
  PDG_TRY(prec_op<T>(ctx, b, p, transpose, skip));
  PDG_TRY(dot<T>(ctx, rc, p, b, nullptr, nullptr, FIN_STORE, S_RHO, -1, true));
  double scal[S_COUNT];
  int flags[F_COUNT];
  int i = 1;
  const int batch = 8;
  bool done = false;
  const bool fuse = std::is_same<T, float>::value ? cg_fusable(ctx)
                                                  : cg_fusable64(ctx, transpose);
  if (fuse) PDG_TRY(ensure_fuse(ctx));
  // one iteration's launches (the iteration count advances on the device)
  auto body = [&]() -> int {
    PDG_TRY(inc_iter(ctx, rc, 1.0));
    if (fuse) {
      // q = A p with lambda = rholast / <p, q> in the same launch
      ctx->fuse_fin = FIN_CG_LAMBDA;
      int st = op_launch<T>(ctx, p, q, nullptr, T(1), 0, transpose, skip);
      ctx->fuse_fin = 0;
      PDG_TRY(st);
      // one block-Jacobi launch: b -= lambda q, defect check, q = M^{-1} b,
      // beta = <q, b> / rholast; then x += lambda p and p = q + beta p
      ctx->fuse_fin = FIN_CG_DEF_BETA;
      ctx->fuse_q = q;
      st = prec_op<T>(ctx, b, q, transpose, skip);
      ctx->fuse_fin = 0;
      ctx->fuse_q = nullptr;
      PDG_TRY(st);
      PDG_TRY(cg_update_px<T>(ctx, rc, ctx->ndof, x, p, q));
    } else {
      PDG_TRY(op_launch<T>(ctx, p, q, nullptr, T(1), 0, transpose, skip));          // q = A p
      PDG_TRY(dot<T>(ctx, rc, p, q, nullptr, nullptr, FIN_CG_LAMBDA, -1, -1, true)); // lambda
      PDG_TRY(cg_update_xr<T>(ctx, rc, ctx->ndof, x, b, p, q));                   // x, b, def
      PDG_TRY(prec_op<T>(ctx, b, q, transpose, skip));                        // q = M^-1 b
      PDG_TRY(dot<T>(ctx, rc, q, b, nullptr, nullptr, FIN_CG_BETA, -1, -1, true));   // beta
      PDG_TRY(cg_update_p<T>(ctx, rc, ctx->ndof, p, q));                           // p = q + beta p
    }
    return PDG_OK;
  };
  // After two batches run one by one (lazy set-up done, the solve not yet
  // converged), a batch of iterations is captured once into a CUDA graph and
  // replayed: one launch per batch instead of one per kernel, which is what
  // small grids are bound by.  Launches after convergence skip their work.
  cudaGraphExec_t gexec = nullptr;
  const bool graphs = ctx->stream != nullptr && ctx->stream != cudaStreamLegacy &&
                      ctx->stream != cudaStreamPerThread && !ctx->use_matrix;
  int st = PDG_OK;
  while (i <= maxit && !done) {
    if (graphs && i > 2 * batch && i + batch - 1 <= maxit && (i - 1) % batch == 0) {
      if (!gexec) {
        cudaGraph_t g = nullptr;
        PDG_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < batch && st == PDG_OK; k++) st = body();
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
        if (st != PDG_OK || ce != cudaSuccess || !g ||
            cudaGraphInstantiate(&gexec, g, 0) != cudaSuccess) {
          if (g) cudaGraphDestroy(g);
          if (gexec) cudaGraphExecDestroy(gexec);
          cudaGetLastError();
          return st != PDG_OK ? st : set_error(PDG_ECUDA, "CUDA graph capture of the CG batch failed");
        }
        cudaGraphDestroy(g);
      }
      if (cudaGraphLaunch(gexec, ctx->stream) != cudaSuccess) {
        cudaGraphExecDestroy(gexec);
        return set_error(PDG_ECUDA, "CUDA graph launch failed");
      }
      i += batch;
    } else {
      st = body();
      if (st != PDG_OK) break;
      i++;
    }
    if ((i - 1) % batch == 0 || i > maxit || i == 2) {
      st = fetch_state(ctx, scal, flags);
      if (st != PDG_OK) break;
      if (flags[F_STATE]) done = true;
    }
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  PDG_TRY(st);
  if (fuse) PDG_TRY(cg_finish_x<T>(ctx, rc, ctx->ndof, x, p));
  PDG_TRY(fetch_state(ctx, scal, flags));
  out->state = flags[F_STATE];
  out->def0 = scal[S_DEF0];
  out->def = scal[S_DEF];
  out->iterations = (int)scal[S_ITER];
  return PDG_OK;
}

// dune-istl BiCGSTABSolver::apply restated on the device.
template <typename T>
static int bicgstab_device(pdg_context *ctx, T *x, T *b, T *w[8], double reduction, int maxit,
                           int transpose, KrylovOut *out, double guard, int replace) {
  const RedCtx rc = red_ctx(ctx);
  const int *skip = ctx->d_flag + F_STATE;
  T *r = b, *p = w[0], *v = w[1], *t = w[2], *y = w[3], *rt = w[4], *bk = w[7];
  // guard > 0 (FP32 inner solves) adds relative breakdown tests to dune-istl's.
  // replace > 0 (FP32 inner solves): every `replace` iterations the
  // recursively updated residual is replaced by the true one, r = b - A x,
  // keeping the recurrence (p, v, rt, rho, alpha, omega) -- reliable updating
  // (Sleijpen & van der Vorst 1996; van der Vorst & Ye 2000).  In FP32 the
  // recursive residual of a long BiCGStab run otherwise drifts away from the
  // true residual.
  if (replace > 0) PDG_TRY(vec_copy<T>(ctx, ctx->ndof, b, bk));
  k_init_solve<<<1, 1, 0, ctx->stream>>>(rc.scal, rc.flags, reduction, guard);
  PDG_TRY(op_launch<T>(ctx, x, r, nullptr, T(-1), 1, transpose, nullptr));
  PDG_TRY(vec_copy<T>(ctx, ctx->ndof, r, rt));
  PDG_TRY(dot<T>(ctx, rc, r, r, nullptr, nullptr, FIN_DEF0, -1, -1, false));
  PDG_TRY(vec_fill<T>(ctx, ctx->ndof, p, T(0)));
  PDG_TRY(vec_fill<T>(ctx, ctx->ndof, v, T(0)));
  double scal[S_COUNT];
  int flags[F_COUNT];
  bool done = false;
  int loop = 0;
  for (double it = 0.5; it < maxit && !done; it += 0.5, loop++) {
    PDG_TRY(set_iter(ctx, rc, it));
    PDG_TRY(dot<T>(ctx, rc, rt, r, nullptr, nullptr, FIN_BI_RHONEW, -1, -1, true));
    PDG_TRY(bi_update_p<T>(ctx, rc, ctx->ndof, p, r, v, it < 1));
    PDG_TRY(prec_op<T>(ctx, p, y, transpose, skip));
    PDG_TRY(op_launch<T>(ctx, y, v, nullptr, T(1), 0, transpose, skip));
    PDG_TRY(dot<T>(ctx, rc, rt, v, v, v, FIN_BI_ALPHA, -1, -1, true));
    PDG_TRY(bi_update_half<T>(ctx, rc, ctx->ndof, x, r, y, v));
    it += 0.5;
    PDG_TRY(set_iter(ctx, rc, it));
    PDG_TRY(prec_op<T>(ctx, r, y, transpose, skip));
    PDG_TRY(op_launch<T>(ctx, y, t, nullptr, T(1), 0, transpose, skip));
    PDG_TRY(dot<T>(ctx, rc, t, r, t, t, FIN_BI_OMEGA, -1, -1, true));
    PDG_TRY(bi_update_full<T>(ctx, rc, ctx->ndof, x, r, y, t));
    if (replace > 0 && (loop + 1) % replace == 0)
      PDG_TRY(op_launch<T>(ctx, x, r, bk, T(-1), 0, transpose, skip));   // r = b - A x
    if (loop % 4 == 3 || it + 0.5 >= maxit || loop == 0) {
      PDG_TRY(fetch_state(ctx, scal, flags));
      if (flags[F_STATE]) done = true;
    }
  }
  PDG_TRY(fetch_state(ctx, scal, flags));
  out->state = flags[F_STATE];
  out->def0 = scal[S_DEF0];
  out->def = scal[S_DEF];
  out->iterations = (int)std::ceil(scal[S_ITER]);
  return PDG_OK;
}

template <typename T>
static int krylov_device(pdg_context *ctx, int method, T *x, T *b, T **w, double reduction,
                         int maxit, int transpose, KrylovOut *out, double guard = 0.0,
                         int restart = 30, int replace = 0) {
  if (method == PDG_CG) return cg_device<T>(ctx, x, b, w[0], w[1], reduction, maxit, transpose, out);
  if (method == PDG_BICGSTAB)
    return bicgstab_device<T>(ctx, x, b, w, reduction, maxit, transpose, out, guard, replace);
  if (method == PDG_GMRES) {
    // b is the right-hand side; GMRES keeps the residual in place of b.
    // Work vectors w[2], w[3] (free of the defect-correction loop's slots).
    const bool f32 = std::is_same<T, float>::value;
    void *&V = f32 ? ctx->gm_V32 : ctx->gm_V64;
    int &Vm = f32 ? ctx->gm_m32 : ctx->gm_m64;
    auto op = [&](const T *in, T *o) -> int {
      return op_launch<T>(ctx, in, o, nullptr, T(1), 0, transpose, nullptr);
    };
    auto prec = [&](const T *in, T *o) -> int { return prec_op<T>(ctx, in, o, transpose, nullptr); };
    GmresOut go;
    PDG_TRY(gmres_core<T>(ctx, x, b, w[2], w[3], V, Vm, reduction, maxit, restart, false, false, op,
                          prec, &go));
    out->state = go.state;
    out->iterations = go.iterations;
    out->def0 = go.def0;
    out->def = go.def;
    return PDG_OK;
  }
  return set_error(PDG_EINVAL, "unknown Krylov method");
}

static int state_status(int state) {
  if (state == 2) return set_error(PDG_ENONFINITE, "non-finite defect");
  if (state == 3) return set_error(PDG_EBREAKDOWN, "breakdown in BiCGStab");
  return PDG_OK;
}

static void fill_result(pdg_solver_result *res, const KrylovOut &o, double elapsed) {
  res->converged = o.state == 1;
  res->iterations = o.iterations;
  res->elapsed = elapsed;
  res->reduction = o.def0 > 0 ? o.def / o.def0 : 0.0;
  res->conv_rate = o.iterations > 0 ? std::pow(res->reduction, 1.0 / o.iterations) : 0.0;
  res->first_defect = o.def0;
  res->defect = o.def;
  res->outer_iterations = 0;
}

static int ensure_prec(pdg_context *ctx, int kind, int precision) {
  PrecData &pd = ctx->prec[precision];
  if (pd.ready && pd.kind == kind) return PDG_OK;
  return prec_setup_impl(ctx, kind, precision);
}

static double elapsed_since_ev0(pdg_context *ctx) {
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaEventSynchronize(ctx->ev1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  return ms * 1e-3;
}

// Mixed precision for non-symmetric operators: FP64 flexible GMRES with the
// exact FP64 operator, whose preconditioner for each new direction v is a
// short inner Krylov solve J c = v with the FP32 operator and FP32 block
// Jacobi (inner_reduction / inner_maxit).  Every outer step minimises the
// true FP64 residual over all inner corrections so far, so an inaccurate
// inner solve slows the outer iteration but cannot make it diverge.  An inner
// solve that ends non-finite is replaced by one FP32 block-Jacobi application.
static int solve_fgmres_ir(pdg_context *ctx, const pdg_solver_options *opt, double *z, double *r,
                           int transpose, pdg_solver_result *res) {
  PDG_TRY(ensure_prec(ctx, opt->preconditioner, PDG_F32));
  const long n = ctx->ndof;
  const int inner = opt->inner_method >= 0 ? opt->inner_method : opt->method;
  const bool vec64 = opt->inner_vectors == PDG_F64;
  int total_inner = 0, fallbacks = 0;
  auto op = [&](const double *in, double *o) -> int {
    return op_launch<double>(ctx, in, o, nullptr, 1.0, 0, transpose, nullptr);
  };
  auto prec = [&](const double *v, double *o) -> int {
    KrylovOut ko{};
    if (!vec64) {
      float *d32 = ctx->w32[5], *c32 = ctx->w32[6];
      PDG_TRY(vec_to_f32(ctx, n, v, d32));
      PDG_TRY(vec_fill<float>(ctx, n, c32, 0.f));
      PDG_TRY(krylov_device<float>(ctx, inner, c32, d32, ctx->w32, opt->inner_reduction,
                                   opt->inner_maxit, transpose, &ko, opt->inner_breakdown,
                                   opt->restart, opt->inner_replace));
      total_inner += ko.iterations;
      if (ko.state != 2) return vec_from_f32_combine(ctx, n, c32, o, nullptr, 1.0, 0, nullptr);
    } else {
      double *c64 = ctx->w64[8], *d64 = ctx->w64[9];
      PDG_TRY(vec_copy<double>(ctx, n, v, d64));
      PDG_TRY(vec_fill<double>(ctx, n, c64, 0.0));
      ctx->ops32 = 1;
      const int ks = krylov_device<double>(ctx, inner, c64, d64, ctx->w64, opt->inner_reduction,
                                           opt->inner_maxit, transpose, &ko, 0.0, opt->restart, 0);
      ctx->ops32 = 0;
      PDG_TRY(ks);
      total_inner += ko.iterations;
      if (ko.state != 2) return vec_copy<double>(ctx, n, c64, o);
    }
    fallbacks++;
    ctx->ops32 = 1;
    const int s = prec_op<double>(ctx, v, o, transpose, nullptr);
    ctx->ops32 = 0;
    return s;
  };
  const int m = std::max(1, std::min(opt->restart, opt->max_outer));
  GmresOut go;
  PDG_TRY(gmres_core<double>(ctx, z, r, ctx->w64[5], ctx->w64[6], ctx->gm_F64, ctx->gm_mF,
                             opt->reduction, opt->max_outer, m, true, opt->verbose != 0, op, prec,
                             &go));
  if (opt->verbose && fallbacks)
    std::fprintf(stderr, "pdg fgmres: %d inner solves replaced by block Jacobi\n", fallbacks);
  res->converged = go.state == 1;
  res->iterations = total_inner;
  res->outer_iterations = go.iterations;
  res->elapsed = elapsed_since_ev0(ctx);
  res->first_defect = go.def0;
  res->defect = go.def;
  res->reduction = go.def0 > 0 ? go.def / go.def0 : 0.0;
  res->conv_rate = total_inner > 0 ? std::pow(res->reduction, 1.0 / total_inner) : 0.0;
  res->status = state_status(go.state);
  if (res->status) return res->status;
  return res->converged ? PDG_OK
                        : set_error(PDG_ENOTCONVERGED, "flexible GMRES did not converge");
}

// Solve J z = r (transposed when `transpose`) from z = 0 or the given z.
// FP64 Krylov; with opt->mixed, FP32 Krylov inside FP64 defect correction
// (CG, or mixed = 2) or inside FP64 flexible GMRES (BiCGStab / GMRES, or
// mixed = 3).  r is overwritten by the final defect.
struct UseMatrixScope {
  pdg_context *ctx;
  int saved;
  UseMatrixScope(pdg_context *c, int on) : ctx(c), saved(c->use_matrix) { c->use_matrix = on; }
  ~UseMatrixScope() { ctx->use_matrix = saved; }
};

static int solve_correction(pdg_context *ctx, const pdg_solver_options *opt, double *z,
                            double *r, int transpose, pdg_solver_result *res) {
  PDG_TRY(ensure_work(ctx, opt->mixed != 0));
  if (opt->assembled) {
    if (opt->mixed) return set_error(PDG_EUNSUPPORTED, "the assembled operator is FP64 only");
    if (!ctx->A_valid) PDG_TRY(assemble_jacobian(ctx));
  }
  UseMatrixScope use_matrix(ctx, opt->assembled != 0);
  cudaEventRecord(ctx->ev0, ctx->stream);
  if (opt->mixed == 3 || (opt->mixed == 1 && opt->method != PDG_CG))
    return solve_fgmres_ir(ctx, opt, z, r, transpose, res);
  if (!opt->mixed) {
    PDG_TRY(ensure_prec(ctx, opt->preconditioner, PDG_F64));
    KrylovOut o{};
    PDG_TRY(krylov_device<double>(ctx, opt->method, z, r, ctx->w64, opt->reduction, opt->maxit,
                                  transpose, &o, 0.0, opt->restart));
    cudaEventRecord(ctx->ev1, ctx->stream);
    cudaEventSynchronize(ctx->ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    fill_result(res, o, ms * 1e-3);
    res->status = state_status(o.state);
    if (res->status) return res->status;
    return res->converged ? PDG_OK : set_error(PDG_ENOTCONVERGED, "Krylov solver did not converge");
  }
  // ---- mixed precision: FP64 defect correction around FP32 Krylov ----
  PDG_TRY(ensure_prec(ctx, opt->preconditioner, PDG_F32));
  const long n = ctx->ndof;
  double *rhs = ctx->w64[5], *d = ctx->w64[6];
  float *d32 = ctx->w32[5], *c32 = ctx->w32[6];
  const RedCtx rc = red_ctx(ctx);
  PDG_TRY(vec_copy<double>(ctx, n, r, rhs));
  // d = rhs - J z
  PDG_TRY(op_launch<double>(ctx, z, d, rhs, -1.0, 0, transpose, nullptr));
  double scal[S_COUNT];
  k_init_solve<<<1, 1, 0, ctx->stream>>>(rc.scal, rc.flags, opt->reduction);
  PDG_TRY(red_dot(ctx, rc, n, d, d, nullptr, nullptr, FIN_NORM, S_DOT, -1, false));
  PDG_TRY(fetch_state(ctx, scal, nullptr));
  const double def0 = scal[S_DOT];
  double def = def0;
  const double target = opt->reduction * def0;
  int total_inner = 0, outer = 0, weak = 0;
  int st = PDG_OK;
  while (def >= target && def >= 1e-30 && outer < opt->max_outer) {
    if (!std::isfinite(def)) { st = set_error(PDG_ENONFINITE, "non-finite defect"); break; }
    KrylovOut o{};
    const int inner = opt->inner_method >= 0 ? opt->inner_method : opt->method;
    const int vec64 = opt->inner_vectors >= 0 ? opt->inner_vectors == PDG_F64
                                              : inner != PDG_CG;
    if (!vec64) {
      // FP32 inner solve of the scaled defect: d32 = d / |d|, c32 = 0
      k_set_scal<<<1, 1, 0, ctx->stream>>>(rc.scal, S_SCALE, def);
      PDG_TRY(vec_to_f32_scaled(ctx, n, d, d32, rc.scal));
      PDG_TRY(vec_fill<float>(ctx, n, c32, 0.f));
      PDG_TRY(krylov_device<float>(ctx, inner, c32, d32, ctx->w32, opt->inner_reduction,
                                   opt->inner_maxit, transpose, &o, opt->inner_breakdown,
                                   opt->restart, opt->inner_replace));
    } else {
      // FP64 Krylov vectors, FP32 operator and block Jacobi (ctx->ops32)
      double *c64 = ctx->w64[8], *d64 = ctx->w64[9];
      PDG_TRY(vec_copy<double>(ctx, n, d, d64));
      PDG_TRY(vec_fill<double>(ctx, n, c64, 0.0));
      ctx->ops32 = 1;
      const int ks = krylov_device<double>(ctx, inner, c64, d64, ctx->w64, opt->inner_reduction,
                                           opt->inner_maxit, transpose, &o, 0.0, opt->restart, 0);
      ctx->ops32 = 0;
      PDG_TRY(ks);
    }
    total_inner += o.iterations;
    // a non-finite inner solve leaves no usable correction; after an inner
    // breakdown (state 3) the last finite iterate is applied and the outer
    // loop restarts the Krylov method from the new defect
    if (o.state == 2) { st = state_status(o.state); break; }
    // z += correction ; d = rhs - J z
    if (!vec64) {
      k_set_scal<<<1, 1, 0, ctx->stream>>>(rc.scal, S_SCALE, def);
      PDG_TRY(vec_add_f32_scaled(ctx, n, c32, z, rc.scal, 1.0));
    } else {
      PDG_TRY(vec_axpy(ctx, n, 1.0, ctx->w64[8], z));
    }
    PDG_TRY(op_launch<double>(ctx, z, d, rhs, -1.0, 0, transpose, nullptr));
    PDG_TRY(red_dot(ctx, rc, n, d, d, nullptr, nullptr, FIN_NORM, S_DOT, -1, false));
    PDG_TRY(fetch_state(ctx, scal, nullptr));
    const double prev = def;
    def = scal[S_DOT];
    outer++;
    // the FP64 defect has reached its rounding floor when corrections stop
    // reducing it: no decrease at all, or three weak steps (< 2x) in a row
    weak = def > 0.5 * prev ? weak + 1 : 0;
    if ((def >= prev || weak >= 3) && def >= target) {
      if (opt->verbose)
        std::fprintf(stderr, "pdg mixed: stagnation at defect %.3e (reduction %.3e)\n", def,
                     def / def0);
      break;
    }
    if (opt->verbose)
      std::fprintf(stderr, "pdg mixed: outer %d inner %d defect %.3e (reduction %.3e)\n", outer,
                   o.iterations, def, def / def0);
  }
  PDG_TRY(vec_copy<double>(ctx, n, d, r));
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaEventSynchronize(ctx->ev1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  res->converged = st == PDG_OK && (def < target || def < 1e-30);
  res->iterations = total_inner;
  res->outer_iterations = outer;
  res->elapsed = ms * 1e-3;
  res->first_defect = def0;
  res->defect = def;
  res->reduction = def0 > 0 ? def / def0 : 0.0;
  res->conv_rate = total_inner > 0 ? std::pow(res->reduction, 1.0 / total_inner) : 0.0;
  res->status = st;
  if (st) return st;
  return res->converged ? PDG_OK
                        : set_error(PDG_ENOTCONVERGED, "defect correction did not converge");
}

// ---- host-pointer staging --------------------------------------------------
static bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template <typename T>
struct Staged {
  T *dev;
  T *host;
  size_t n;
  bool staged;
};

template <typename T>
static int stage_in(pdg_context *ctx, const T *p, size_t n, T *buf, bool copy, Staged<T> *s) {
  s->n = n;
  if (is_device_ptr(p)) {
    s->dev = const_cast<T *>(p);
    s->host = nullptr;
    s->staged = false;
    return PDG_OK;
  }
  s->dev = buf;
  s->host = const_cast<T *>(p);
  s->staged = true;
  if (copy)
    PDG_CUDA_TRY(cudaMemcpyAsync(buf, p, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  return PDG_OK;
}
template <typename T>
static int stage_out(pdg_context *ctx, const Staged<T> &s) {
  if (!s.staged) return PDG_OK;
  PDG_CUDA_TRY(cudaMemcpyAsync(s.host, s.dev, s.n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

static int upload(pdg_context *ctx, double **dst, const double *src, size_t n) {
  if (!src) {
    if (*dst) cudaFree(*dst);
    *dst = nullptr;
    return PDG_OK;
  }
  if (!*dst) PDG_CUDA_TRY(cudaMalloc(dst, n * sizeof(double)));
  PDG_CUDA_TRY(cudaMemcpyAsync(*dst, src, n * sizeof(double),
                               is_device_ptr(src) ? cudaMemcpyDeviceToDevice
                                                  : cudaMemcpyHostToDevice,
                               ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

__global__ void k_perm(long n, const double *__restrict__ src, int is_log,
                       double *__restrict__ K64, float *__restrict__ K32) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = is_log ? exp(src[i]) : src[i];
  K64[i] = v;
  K32[i] = (float)v;
}

// an FP64 upload and its FP32 copy (src null frees both)
static int upload_dual(pdg_context *ctx, double **d64, float **d32, const double *src, size_t n) {
  PDG_TRY(upload(ctx, d64, src, n));
  if (!src) {
    if (*d32) cudaFree(*d32);
    *d32 = nullptr;
    return PDG_OK;
  }
  if (!*d32) PDG_CUDA_TRY(cudaMalloc(d32, sizeof(float) * n));
  PDG_TRY(vec_to_f32(ctx, (long)n, *d64, *d32));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

// 2D grids: an outflow boundary side must not see inflow, b.n < -1e-30 at a
// boundary quadrature point (convectiondiffusiondg.hh:802-806); b from the
// Fourier modes or the velocity point data (face lattice)
static int check_outflow_2d(pdg_context *ctx) {
  const RhsTables t = make_rhs_tables(ctx);
  const int nc[3] = {ctx->cfg.cells[0], ctx->cfg.cells[1], 1};
  const int N = ctx->N;
  std::vector<double> bf;
  if (ctx->vel_points) {
    bf.resize((size_t)face_lattice_count(ctx) * ctx->nqf * 3);
    PDG_CUDA_TRY(cudaMemcpy(bf.data(), ctx->bqf64, sizeof(double) * bf.size(),
                            cudaMemcpyDeviceToHost));
  }
  for (int side = 0; side < 4; side++) {
    if (ctx->cfg.bctype[side] != PDG_BC_OUTFLOW) continue;
    const int dir = side >> 1, hi = side & 1, o = 1 - dir;
    int ix[3] = {0, 0, 0};
    ix[dir] = hi ? nc[dir] - 1 : 0;
    for (int a = 0; a < nc[o]; a++) {
      ix[o] = a;
      const long fi = face_lattice_index(nc, 2, dir, ix[dir] + hi, ix);
      for (int q = 0; q < N; q++) {
        double b[2] = {0.0, 0.0};
        if (ctx->vel_points) {
          b[dir] = bf[((size_t)fi * N + q) * 3 + dir];
        } else {
          double xg[2];
          xg[dir] = (ix[dir] + hi) * ctx->h[dir];
          xg[o] = (a + t.x[q]) * ctx->h[o];
          for (int m = 0; m < ctx->vel.nmodes; m++) {
            double arg = ctx->vel.m[m][3];
            for (int j = 0; j < 2; j++) arg += 2.0 * M_PI * ctx->vel.m[m][j] * xg[j];
            const double sv = std::sin(arg);
            for (int j = 0; j < 2; j++) b[j] += ctx->vel.m[m][4 + j] * sv;
          }
        }
        if ((hi ? b[dir] : -b[dir]) < -1e-30)
          return set_error(PDG_EOUTFLOW, "outflow boundary condition on inflow");
      }
    }
  }
  return PDG_OK;
}

// drop the tensor fields (per cell and per point)
static void free_tensors(pdg_context *ctx) {
  double **d[] = {&ctx->Ac64, &ctx->Aqv64, &ctx->Aqf64, &ctx->Kd64};
  float **f[] = {&ctx->Ac32, &ctx->Aqv32, &ctx->Aqf32, &ctx->Kd32};
  for (double **p : d)
    if (*p) { cudaFree(*p); *p = nullptr; }
  for (float **p : f)
    if (*p) { cudaFree(*p); *p = nullptr; }
}

static void invalidate(pdg_context *ctx, bool operator_changed) {
  ctx->r0_valid = 0;
  if (operator_changed) {
    ctx->op_gen++;
    ctx->rec_valid = 0;
    ctx->rec64m_valid = 0;
    ctx->rec64mT_valid = 0;
    ctx->recfp_valid = 0;
    ctx->rec32_valid = 0;
    ctx->rec32q_valid = 0;
    ctx->A_valid = 0;
    ctx->prec[0].ready = 0;
    ctx->prec[1].ready = 0;
  }
}

}  // namespace pdg

using namespace pdg;

#define PDG_CHECK_CTX(ctx)                                                     \
  do {                                                                         \
    if (!(ctx)) return set_error(PDG_EINVAL, "null context");                 \
    PDG_CUDA_TRY(cudaSetDevice((ctx)->device));                                \
  } while (0)

extern "C" {

const char *pdg_last_error(void) { return g_err.c_str(); }

void pdg_default_solver_options(pdg_solver_options *o) {
  if (!o) return;
  o->method = PDG_CG;
  o->preconditioner = PDG_PREC_BJ_FDM;
  o->reduction = 1e-10;
  o->min_defect = 1e-99;
  o->maxit = 5000;
  o->mixed = 0;
  o->inner_reduction = 1e-3;
  o->inner_maxit = 5000;
  o->max_outer = 30;
  o->verbose = 0;
  o->inner_breakdown = 1e-9;
  o->inner_method = -1;
  o->restart = 30;
  o->inner_replace = 25;
  o->inner_vectors = -1;
  o->assembled = 0;
}

void pdg_default_prec_options(pdg_prec_options *o) {
  if (!o) return;
  o->omega = 1.0;
  o->block_reduction = 1e-5;
  o->block_maxit = 100;
  o->block_precondition = 1;
  o->block_weight = 1.0;
  o->dense_fp16 = 0;
}

int pdg_set_prec_options(pdg_context *ctx, const pdg_prec_options *o) {
  PDG_CHECK_CTX(ctx);
  if (!o) return set_error(PDG_EINVAL, "null options");
  if (!(o->omega > 0.0 && o->omega < 2.0)) return set_error(PDG_EINVAL, "omega must be in (0,2)");
  if (!(o->block_reduction > 0.0) || o->block_maxit < 1)
    return set_error(PDG_EINVAL, "bad block solver options");
  // the FP32 dense block inverses are stored per dense_fp16: a set-up made
  // under the other setting is dropped (the next solve sets it up again)
  if (o->dense_fp16 != ctx->popt.dense_fp16 &&
      (ctx->prec[PDG_F32].kind & PDG_PREC_BLOCK_MASK) == PDG_PREC_BJ_DENSE)
    prec_free(ctx, PDG_F32);
  ctx->popt = *o;
  ctx->op_gen++;
  return PDG_OK;
}

int pdg_prec_block_iterations(pdg_context *ctx, int precision, int *iterations) {
  PDG_CHECK_CTX(ctx);
  if (!iterations || (precision != PDG_F64 && precision != PDG_F32))
    return set_error(PDG_EINVAL, "bad argument");
  const PrecData &pd = ctx->prec[precision];
  if (!pd.ready || !pd.iters)
    return set_error(PDG_ESTATE, "no iterative block Jacobi set up in this precision");
  PDG_CUDA_TRY(cudaMemcpyAsync(iterations, pd.iters, sizeof(int) * ctx->ncell,
                               is_device_ptr(iterations) ? cudaMemcpyDeviceToDevice
                                                         : cudaMemcpyDeviceToHost,
                               ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

int pdg_create(const pdg_config *cfg, pdg_context **out) {
  if (!cfg || !out) return set_error(PDG_EINVAL, "null argument");
  *out = nullptr;
  if (cfg->dim < 2 || cfg->dim > 3) return set_error(PDG_EINVAL, "dim must be 2 or 3");
  if (cfg->degree < 1 || cfg->degree > kMaxDeg)
    return set_error(PDG_EUNSUPPORTED, "degree must be 1..4");
  for (int j = 0; j < cfg->dim; j++) {
    if (cfg->cells[j] < 1) return set_error(PDG_EINVAL, "cells must be >= 1");
    if (!(cfg->extent[j] > 0)) return set_error(PDG_EINVAL, "extent must be > 0");
  }
  if (cfg->method < PDG_NIPG || cfg->method > PDG_IIPG)
    return set_error(PDG_EINVAL, "bad method");
  if (cfg->weights != PDG_WEIGHTS_ON && cfg->weights != PDG_WEIGHTS_OFF)
    return set_error(PDG_EINVAL, "bad weights");
  for (int s = 0; s < 2 * cfg->dim; s++) {
    const int b = cfg->bctype[s];
    if (b != PDG_BC_DIRICHLET && b != PDG_BC_NEUMANN && b != PDG_BC_OUTFLOW && b != PDG_BC_NONE)
      return set_error(PDG_EINVAL, "bad boundary type");
  }
  if (cfg->basis < PDG_BASIS_LAGRANGE || cfg->basis > PDG_BASIS_LOBATTO)
    return set_error(PDG_EINVAL, "bad basis");
  PDG_CUDA_TRY(cudaSetDevice(cfg->device));
  pdg_context *c = new pdg_context;
  std::memset(c, 0, sizeof(*c));
  c->cfg = *cfg;
  pdg_default_prec_options(&c->popt);
  c->device = cfg->device;
  c->dim = cfg->dim;
  c->k = cfg->degree;
  c->N = c->k + 1;
  c->basis = cfg->basis;
  if (c->basis == PDG_BASIS_LOBATTO) gauss_lobatto_points(c->N, c->nodes);
  else
    for (int j = 0; j < c->N; j++) c->nodes[j] = (double)j / c->k;
  c->nb = 1;
  c->nqv = 1;
  c->nqf = 1;
  c->ncell = 1;
  for (int j = 0; j < c->dim; j++) {
    c->nb *= c->N;
    c->ncell *= cfg->cells[j];
    c->h[j] = cfg->extent[j] / cfg->cells[j];
  }
  for (int j = c->dim; j < 3; j++) c->h[j] = 1.0;
  c->nqv = c->nb;
  for (int j = 0; j < c->dim - 1; j++) c->nqf *= c->N;
  c->ndof = c->ncell * c->nb;
  c->nbpts = 0;
  for (int s = 0; s < 2 * c->dim; s++) {
    long cnt = 1;
    for (int j = 0; j < c->dim; j++)
      if (j != s / 2) cnt *= cfg->cells[j];
    c->nbpts += cnt * c->nqf;
  }
  c->theta = cfg->method == PDG_SIPG ? -1.0 : (cfg->method == PDG_NIPG ? 1.0 : 0.0);
  c->pen_fac = cfg->alpha * c->k * (c->k + c->dim - 1);
  auto fail = [&](int st) {
    pdg_destroy(c);
    return st;
  };
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_error(PDG_ECUDA, "cudaStreamCreate failed"));
  c->stream = c->own_stream;
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  // 1D tables
  RhsTables t = make_rhs_tables(c);
  const int N = c->N;
  std::vector<double> tab(2 * N * N + 2 * N);
  for (int i = 0; i < N; i++)
    for (int a = 0; a < N; a++) {
      double m = 0.0, s = 0.0;
      for (int q = 0; q < N; q++) {
        m += t.w[q] * nlag(c, i, t.x[q]) * nlag(c, a, t.x[q]);
        s += t.w[q] * ndlag(c, i, t.x[q]) * ndlag(c, a, t.x[q]);
      }
      tab[i * N + a] = m;
      tab[N * N + i * N + a] = s;
    }
  for (int a = 0; a < N; a++) {
    tab[2 * N * N + a] = t.d0[a];
    tab[2 * N * N + N + a] = t.d1[a];
  }
  std::vector<float> tab32(tab.begin(), tab.end());
  std::vector<double> ones(c->ncell, 1.0);
  std::vector<float> ones32(c->ncell, 1.0f);
  if (cudaMalloc(&c->tab64, sizeof(double) * tab.size()) != cudaSuccess ||
      cudaMalloc(&c->tab32, sizeof(float) * tab.size()) != cudaSuccess ||
      cudaMalloc(&c->K64, sizeof(double) * c->ncell) != cudaSuccess ||
      cudaMalloc(&c->K32, sizeof(float) * c->ncell) != cudaSuccess ||
      cudaMalloc(&c->r0, sizeof(double) * c->ndof) != cudaSuccess ||
      cudaMalloc(&c->red_partials, sizeof(double) * 2 * kRedBlocks) != cudaSuccess ||
      cudaMalloc(&c->red_out, sizeof(double) * S_COUNT) != cudaSuccess ||
      cudaMalloc(&c->d_flag, sizeof(int) * F_COUNT) != cudaSuccess ||
      cudaMallocHost(&c->h_red, sizeof(double) * S_COUNT + sizeof(int) * F_COUNT) != cudaSuccess)
    return fail(set_error(PDG_ECUDA, "device allocation failed"));
  cudaMemcpy(c->tab64, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice);
  if (c->dim == 3) {
    // the mass-factored operator's tables: Mhat, Mhat^-1 applied to the face
    // vectors e0, e_{N-1}, d0, d1, and Mhat^-1 (Gauss-Jordan, partial pivoting)
    std::vector<double> a(tab.begin(), tab.begin() + N * N), inv(N * N, 0.0);
    for (int i = 0; i < N; i++) inv[i * N + i] = 1.0;
    for (int col = 0; col < N; col++) {
      int piv = col;
      for (int r = col + 1; r < N; r++)
        if (std::fabs(a[r * N + col]) > std::fabs(a[piv * N + col])) piv = r;
      for (int j = 0; j < N; j++) {
        std::swap(a[col * N + j], a[piv * N + j]);
        std::swap(inv[col * N + j], inv[piv * N + j]);
      }
      const double d = a[col * N + col];
      for (int j = 0; j < N; j++) {
        a[col * N + j] /= d;
        inv[col * N + j] /= d;
      }
      for (int r = 0; r < N; r++)
        if (r != col) {
          const double f = a[r * N + col];
          for (int j = 0; j < N; j++) {
            a[r * N + j] -= f * a[col * N + j];
            inv[r * N + j] -= f * inv[col * N + j];
          }
        }
    }
    std::vector<double> tm(2 * N * N + 4 * N);
    for (int i = 0; i < N * N; i++) {
      tm[i] = tab[i];
      tm[N * N + 4 * N + i] = inv[i];
    }
    for (int i = 0; i < N; i++) {
      double m0 = inv[i * N], m1 = inv[i * N + N - 1], md0 = 0.0, md1 = 0.0;
      for (int k = 0; k < N; k++) {
        md0 += inv[i * N + k] * tab[2 * N * N + k];
        md1 += inv[i * N + k] * tab[2 * N * N + N + k];
      }
      tm[N * N + i] = m0;
      tm[N * N + N + i] = m1;
      tm[N * N + 2 * N + i] = md0;
      tm[N * N + 3 * N + i] = md1;
    }
    if (cudaMalloc(&c->tabm64, sizeof(double) * tm.size()) != cudaSuccess)
      return fail(set_error(PDG_ECUDA, "device allocation failed"));
    cudaMemcpy(c->tabm64, tm.data(), sizeof(double) * tm.size(), cudaMemcpyHostToDevice);
  }
  cudaMemcpy(c->tab32, tab32.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(c->K64, ones.data(), sizeof(double) * c->ncell, cudaMemcpyHostToDevice);
  cudaMemcpy(c->K32, ones32.data(), sizeof(float) * c->ncell, cudaMemcpyHostToDevice);
  cudaMemset(c->d_flag, 0, sizeof(int) * F_COUNT);
  cudaMemset(c->red_out, 0, sizeof(double) * S_COUNT);
  if (c->basis == PDG_BASIS_LEGENDRE) {
    double lt[2 * kMaxN1 * kMaxN1];
    legendre_change_of_basis(c->k, lt);
    std::vector<float> lt32(lt, lt + 2 * N * N);
    if (cudaMalloc(&c->leg64, sizeof(double) * 2 * N * N) != cudaSuccess ||
        cudaMalloc(&c->leg32, sizeof(float) * 2 * N * N) != cudaSuccess ||
        cudaMalloc(&c->legw64[0], sizeof(double) * c->ndof) != cudaSuccess ||
        cudaMalloc(&c->legw64[1], sizeof(double) * c->ndof) != cudaSuccess ||
        cudaMalloc(&c->legw32[0], sizeof(float) * c->ndof) != cudaSuccess ||
        cudaMalloc(&c->legw32[1], sizeof(float) * c->ndof) != cudaSuccess)
      return fail(set_error(PDG_ECUDA, "device allocation failed"));
    cudaMemcpy(c->leg64, lt, sizeof(double) * 2 * N * N, cudaMemcpyHostToDevice);
    cudaMemcpy(c->leg32, lt32.data(), sizeof(float) * 2 * N * N, cudaMemcpyHostToDevice);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(set_error(PDG_ECUDA, "init failed"));
  c->r0_valid = 0;
  *out = c;
  return PDG_OK;
}

int pdg_destroy(pdg_context *c) {
  if (!c) return PDG_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->pipe_h2d) {
    cudaStreamSynchronize(c->pipe_h2d);
    cudaStreamSynchronize(c->pipe_d2h);
    cudaStreamSynchronize(c->pipe_k2);
  }
  prec_free(c, 0);
  prec_free(c, 1);
  sor_free(c);
  void *bufs[] = {c->K64, c->K32, c->c64, c->c32, c->tab64, c->tab32, c->fq, c->fc, c->gq,
                  c->jq, c->oq, c->r0, c->r0K, c->red_partials, c->red_out, c->d_flag,
                  c->stage_a, c->stage_b, c->rec64, c->conv64, c->conv32, c->convtab64,
                  c->convtab32, c->gm_V32, c->gm_V64, c->gm_F64, c->gm_partial, c->gm_coef,
                  c->A64, c->rec32, c->nlW64, c->nlW32, c->nlB64, c->nlB32,
                  c->massW, c->massWi, c->massB, c->massBiT, c->cstage64, c->cstage32,
                  c->leg64, c->leg32, c->legw64[0], c->legw64[1], c->legw32[0], c->legw32[1],
                  c->fuse_part, c->fuse_cnt, c->Ac64, c->Aqv64, c->Aqf64, c->cq64, c->Ac32,
                  c->Aqv32, c->Aqf32, c->cq32, c->bqv64, c->bqf64, c->Kd64, c->Kd32,
                  c->recfp, c->tabfp, c->rec32q, c->rec64m, c->rec64mT, c->tabm64};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (int i = 0; i < 10; i++)
    if (c->w64[i]) cudaFree(c->w64[i]);
  for (int i = 0; i < 8; i++)
    if (c->w32[i]) cudaFree(c->w32[i]);
  if (c->h_red) cudaFreeHost(c->h_red);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  if (c->pipe_h2d) {
    cudaStreamDestroy(c->pipe_h2d);
    cudaStreamDestroy(c->pipe_d2h);
    cudaStreamDestroy(c->pipe_k2);
    for (cudaEvent_t e : c->pipe_ev)
      if (e) cudaEventDestroy(e);
  }
  delete c;
  return PDG_OK;
}

int pdg_set_stream(pdg_context *ctx, void *stream) {
  PDG_CHECK_CTX(ctx);
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return PDG_OK;
}

int pdg_get_stream(const pdg_context *ctx, void **stream) {
  if (!ctx || !stream) return set_error(PDG_EINVAL, "null argument");
  *stream = (void *)ctx->stream;
  return PDG_OK;
}

int pdg_sizes(const pdg_context *ctx, long *ncell, int *nbasis, long *ndof, int *nqv,
              long *nbp) {
  if (!ctx) return set_error(PDG_EINVAL, "null context");
  if (ncell) *ncell = ctx->ncell;
  if (nbasis) *nbasis = ctx->nb;
  if (ndof) *ndof = ctx->ndof;
  if (nqv) *nqv = ctx->nqv;
  if (nbp) *nbp = ctx->nbpts;
  return PDG_OK;
}

int pdg_volume_points(const pdg_context *ctx, double *xyz) {
  if (!ctx || !xyz) return set_error(PDG_EINVAL, "null argument");
  double gx[kMaxN1], gw[kMaxN1];
  gauss_legendre(ctx->N, gx, gw);
  const int N = ctx->N, d = ctx->dim;
  const int *nc = ctx->cfg.cells;
  for (long e = 0; e < ctx->ncell; e++) {
    int ix[3] = {(int)(e % nc[0]), (int)((e / nc[0]) % nc[1]), (int)(e / ((long)nc[0] * nc[1]))};
    for (int q = 0; q < ctx->nqv; q++) {
      int qa[3] = {q % N, (q / N) % N, q / (N * N)};
      for (int j = 0; j < d; j++) xyz[(e * ctx->nqv + q) * d + j] = (ix[j] + gx[qa[j]]) * ctx->h[j];
    }
  }
  return PDG_OK;
}

int pdg_boundary_points(const pdg_context *ctx, double *xyz) {
  if (!ctx || !xyz) return set_error(PDG_EINVAL, "null argument");
  double gx[kMaxN1], gw[kMaxN1];
  gauss_legendre(ctx->N, gx, gw);
  const int N = ctx->N, d = ctx->dim;
  const int *nc = ctx->cfg.cells;
  long base = 0;
  for (int s = 0; s < 2 * d; s++) {
    const int dir = s / 2, hi = s % 2;
    int od[2], no = 0;
    for (int j = 0; j < d; j++)
      if (j != dir) od[no++] = j;
    const long nf0 = nc[od[0]], nf1 = no > 1 ? nc[od[1]] : 1;
    for (long f1 = 0; f1 < nf1; f1++)
      for (long f0 = 0; f0 < nf0; f0++) {
        const long fidx = f0 + nf0 * f1;
        for (int q = 0; q < ctx->nqf; q++) {
          const int qt[2] = {q % N, q / N};
          double *pt = xyz + (base + fidx * ctx->nqf + q) * d;
          pt[dir] = hi ? ctx->cfg.extent[dir] : 0.0;
          pt[od[0]] = (f0 + gx[qt[0]]) * ctx->h[od[0]];
          if (no > 1) pt[od[1]] = (f1 + gx[qt[1]]) * ctx->h[od[1]];
        }
      }
    base += nf0 * nf1 * ctx->nqf;
  }
  return PDG_OK;
}

int pdg_set_permeability(pdg_context *ctx, const double *K, int is_log) {
  PDG_CHECK_CTX(ctx);
  if (!K) return set_error(PDG_EINVAL, "null permeability");
  double *tmp = nullptr;
  PDG_TRY(upload(ctx, &tmp, K, ctx->ncell));
  k_perm<<<(unsigned)((ctx->ncell + 255) / 256), 256, 0, ctx->stream>>>(ctx->ncell, tmp, is_log,
                                                                        ctx->K64, ctx->K32);
  PDG_CUDA_TRY(cudaGetLastError());
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  cudaFree(tmp);
  // A = K I: a tensor set before is dropped
  free_tensors(ctx);
  ctx->gen_A = 0;
  invalidate(ctx, true);
  return PDG_OK;
}

int pdg_set_permeability_tensor(pdg_context *ctx, const double *A) {
  PDG_CHECK_CTX(ctx);
  if (!A) {
    if (ctx->gen_A == 1 || ctx->gen_A == 3) {
      free_tensors(ctx);
      ctx->gen_A = 0;
      invalidate(ctx, true);
    }
    return PDG_OK;
  }
  free_tensors(ctx);
  const int d = ctx->dim;
  const size_t n = (size_t)ctx->ncell * d * d;
  PDG_TRY(upload_dual(ctx, &ctx->Ac64, &ctx->Ac32, A, n));
  // a diagonal tensor keeps the operator separable: K per direction in the
  // Kronecker records (and the FDM block Jacobi stays exact)
  std::vector<double> h(n);
  PDG_CUDA_TRY(cudaMemcpy(h.data(), ctx->Ac64, sizeof(double) * n, cudaMemcpyDeviceToHost));
  bool diag = true;
  for (long e = 0; e < ctx->ncell && diag; e++)
    for (int i = 0; i < d; i++)
      for (int j = 0; j < d; j++)
        if (i != j && h[(size_t)e * d * d + i * d + j] != 0.0) diag = false;
  if (diag) {
    std::vector<double> kd((size_t)ctx->ncell * 3, 1.0);
    for (long e = 0; e < ctx->ncell; e++)
      for (int i = 0; i < d; i++) kd[(size_t)e * 3 + i] = h[(size_t)e * d * d + i * d + i];
    PDG_TRY(upload_dual(ctx, &ctx->Kd64, &ctx->Kd32, kd.data(), kd.size()));
    ctx->gen_A = 3;
  } else {
    ctx->gen_A = 1;
  }
  invalidate(ctx, true);
  return PDG_OK;
}

int pdg_set_permeability_points(pdg_context *ctx, const double *Avol, const double *Aface) {
  PDG_CHECK_CTX(ctx);
  if (!Avol != !Aface)
    return set_error(PDG_EINVAL, "give both the volume and the face tensors, or neither");
  if (!Avol) {
    if (ctx->gen_A == 2) {
      free_tensors(ctx);
      ctx->gen_A = 0;
      invalidate(ctx, true);
    }
    return PDG_OK;
  }
  free_tensors(ctx);
  const size_t dd = (size_t)ctx->dim * ctx->dim;
  PDG_TRY(upload_dual(ctx, &ctx->Aqv64, &ctx->Aqv32, Avol, (size_t)ctx->ncell * ctx->nqv * dd));
  PDG_TRY(upload_dual(ctx, &ctx->Aqf64, &ctx->Aqf32, Aface,
                      (size_t)ctx->ncell * 2 * ctx->dim * ctx->nqf * dd));
  ctx->gen_A = 2;
  invalidate(ctx, true);
  return PDG_OK;
}

int pdg_set_reaction_points(pdg_context *ctx, const double *cq) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(upload_dual(ctx, &ctx->cq64, &ctx->cq32, cq, (size_t)ctx->ncell * ctx->nqv));
  invalidate(ctx, true);
  return PDG_OK;
}

int pdg_set_velocity_points(pdg_context *ctx, const double *bvol, const double *bface) {
  PDG_CHECK_CTX(ctx);
  if (!bvol != !bface)
    return set_error(PDG_EINVAL, "give both the volume and the face velocities, or neither");
  if (!bvol) {
    if (ctx->vel_points) {
      PDG_TRY(upload(ctx, &ctx->bqv64, nullptr, 0));
      PDG_TRY(upload(ctx, &ctx->bqf64, nullptr, 0));
      ctx->vel_points = 0;
      invalidate(ctx, true);
    }
    return PDG_OK;
  }
  PDG_TRY(upload(ctx, &ctx->bqv64, bvol, (size_t)ctx->ncell * ctx->nqv * 3));
  PDG_TRY(upload(ctx, &ctx->bqf64, bface, (size_t)face_lattice_count(ctx) * ctx->nqf * 3));
  ctx->vel.nmodes = 0;
  ctx->vel_points = 1;
  invalidate(ctx, true);
  const int st = ctx->dim == 3 ? conv_setup(ctx) : check_outflow_2d(ctx);
  if (st != PDG_OK) ctx->vel_points = 0;
  return st;
}

int pdg_set_f64_arithmetic(pdg_context *ctx, int mode) {
  PDG_CHECK_CTX(ctx);
  if (mode != PDG_F64_NATIVE && mode != PDG_F64_FLOAT_PAIR)
    return set_error(PDG_EINVAL, "mode must be PDG_F64_NATIVE or PDG_F64_FLOAT_PAIR");
  if (mode == PDG_F64_FLOAT_PAIR && ctx->dim != 3)
    return set_error(PDG_EUNSUPPORTED, "float-pair arithmetic is implemented for 3D grids");
  ctx->f64_pair = mode == PDG_F64_FLOAT_PAIR;
  ctx->op_gen++;   // cached solver state (block-SOR graphs) follows the operator
  return PDG_OK;
}

int pdg_face_lattice_size(const pdg_context *ctx, long *nfaces) {
  if (!ctx || !nfaces) return set_error(PDG_EINVAL, "null argument");
  *nfaces = face_lattice_count(ctx);
  return PDG_OK;
}

int pdg_face_lattice_points(const pdg_context *ctx, double *xyz) {
  if (!ctx || !xyz) return set_error(PDG_EINVAL, "null argument");
  const RhsTables t = make_rhs_tables(ctx);
  const int d = ctx->dim, N = ctx->N;
  int nc[3] = {ctx->cfg.cells[0], ctx->cfg.cells[1], d == 3 ? ctx->cfg.cells[2] : 1};
  for (int dir = 0; dir < d; dir++) {
    int od[2] = {0, 0}, no = 0;
    for (int j = 0; j < d; j++)
      if (j != dir) od[no++] = j;
    int ix[3] = {0, 0, 0};
    for (int pl = 0; pl <= nc[dir]; pl++)
      for (int b = 0; b < (no > 1 ? nc[od[1]] : 1); b++)
        for (int a = 0; a < nc[od[0]]; a++) {
          ix[od[0]] = a;
          if (no > 1) ix[od[1]] = b;
          const long fi = face_lattice_index(nc, d, dir, pl, ix);
          for (int q = 0; q < ctx->nqf; q++) {
            double *pt = xyz + (fi * ctx->nqf + q) * d;
            pt[dir] = pl * ctx->h[dir];
            pt[od[0]] = (a + t.x[q % N]) * ctx->h[od[0]];
            if (no > 1) pt[od[1]] = (b + t.x[q / N]) * ctx->h[od[1]];
          }
        }
  }
  return PDG_OK;
}

int pdg_cell_face_points(const pdg_context *ctx, double *xyz) {
  if (!ctx || !xyz) return set_error(PDG_EINVAL, "null argument");
  const RhsTables t = make_rhs_tables(ctx);
  const int d = ctx->dim, N = ctx->N;
  for (long e = 0; e < ctx->ncell; e++) {
    int ix[3];
    long r = e;
    for (int j = 0; j < d; j++) { ix[j] = (int)(r % ctx->cfg.cells[j]); r /= ctx->cfg.cells[j]; }
    for (int f = 0; f < 2 * d; f++) {
      const int dir = f >> 1, hi = f & 1;
      int od[2] = {0, 0}, no = 0;
      for (int j = 0; j < d; j++)
        if (j != dir) od[no++] = j;
      for (int q = 0; q < ctx->nqf; q++) {
        double *pt = xyz + ((e * 2 * d + f) * ctx->nqf + q) * d;
        pt[dir] = (ix[dir] + hi) * ctx->h[dir];
        pt[od[0]] = (ix[od[0]] + t.x[q % N]) * ctx->h[od[0]];
        if (no > 1) pt[od[1]] = (ix[od[1]] + t.x[q / N]) * ctx->h[od[1]];
      }
    }
  }
  return PDG_OK;
}

int pdg_set_reaction(pdg_context *ctx, const double *c) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(upload(ctx, &ctx->c64, c, ctx->ncell));
  if (!c) {
    if (ctx->c32) cudaFree(ctx->c32);
    ctx->c32 = nullptr;
  } else {
    if (!ctx->c32) PDG_CUDA_TRY(cudaMalloc(&ctx->c32, sizeof(float) * ctx->ncell));
    PDG_TRY(vec_to_f32(ctx, ctx->ncell, ctx->c64, ctx->c32));
    PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  invalidate(ctx, true);
  return PDG_OK;
}

int pdg_set_velocity_modes(pdg_context *ctx, int nmodes, const double *modes) {
  PDG_CHECK_CTX(ctx);
  if (nmodes < 0 || nmodes > kMaxModes) return set_error(PDG_EINVAL, "nmodes must be 0..16");
  if (nmodes > 0 && !modes) return set_error(PDG_EINVAL, "null modes");
  ctx->vel.nmodes = nmodes;
  if (nmodes > 0 && ctx->vel_points) {
    // modes replace velocity point data
    PDG_TRY(upload(ctx, &ctx->bqv64, nullptr, 0));
    PDG_TRY(upload(ctx, &ctx->bqf64, nullptr, 0));
    ctx->vel_points = 0;
  }
  for (int m = 0; m < nmodes; m++)
    for (int j = 0; j < 7; j++) ctx->vel.m[m][j] = modes[7 * m + j];
  invalidate(ctx, true);
  if (nmodes > 0) {
    // 3D: the convection kernel's records; 2D: the Gauss-point operator
    // evaluates b itself, so only the outflow sides are checked here
    const int st = ctx->dim == 3 ? conv_setup(ctx) : check_outflow_2d(ctx);
    if (st != PDG_OK) {
      ctx->vel.nmodes = 0;
      return st;
    }
  }
  return PDG_OK;
}

int pdg_set_source(pdg_context *ctx, const double *fq, const double *fc) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(upload(ctx, &ctx->fq, fq, (size_t)ctx->ncell * ctx->nqv));
  PDG_TRY(upload(ctx, &ctx->fc, fc, ctx->ncell));
  invalidate(ctx, false);
  return PDG_OK;
}

int pdg_set_boundary_data(pdg_context *ctx, const double *g, const double *j, const double *o) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(upload(ctx, &ctx->gq, g, ctx->nbpts));
  PDG_TRY(upload(ctx, &ctx->jq, j, ctx->nbpts));
  PDG_TRY(upload(ctx, &ctx->oq, o, ctx->nbpts));
  if (!g && ctx->r0K) {
    cudaFree(ctx->r0K);
    ctx->r0K = nullptr;
  }
  invalidate(ctx, false);
  return PDG_OK;
}

static int ensure_stage(pdg_context *ctx) {
  if (!ctx->stage_a) PDG_CUDA_TRY(cudaMalloc(&ctx->stage_a, sizeof(double) * ctx->ndof));
  if (!ctx->stage_b) PDG_CUDA_TRY(cudaMalloc(&ctx->stage_b, sizeof(double) * ctx->ndof));
  return PDG_OK;
}

// ---- host-buffer applies pipelined over slabs of cells --------------------
// Copying x in, applying and copying y out one after another costs the copies
// on top of the kernel.  The grid is cut into slabs of whole planes of the
// slowest direction (contiguous cell and DOF ranges); slab s is applied once
// slabs s and s+1 are on the device (its faces read one neighbour plane) and
// copied out while slab s+1 is applied, so the copies in, the kernels and the
// copies out overlap, ordered by events.  Consecutive slabs are applied on
// two alternating streams: they write disjoint ranges of y, and the last,
// partly filled wave of one slab's grid overlaps the first of the next.
constexpr int kMaxSlabs = kPipeMaxSlabs;
static_assert(sizeof(pdg_context::pipe_ev) / sizeof(cudaEvent_t) == 2 * kMaxSlabs + 3,
              "one event per slab each way, plus start, end and the second stream's");
constexpr long kMinSlabCells = 16384;

static int cuda_status(cudaError_t e) {
  return e == cudaSuccess ? PDG_OK
                          : set_error(PDG_ECUDA, std::string("host-buffer apply: ") +
                                                     cudaGetErrorString(e));
}

static int pipe_ready(pdg_context *ctx) {
  if (ctx->pipe_h2d) return PDG_OK;
  PDG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->pipe_h2d, cudaStreamNonBlocking));
  PDG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->pipe_d2h, cudaStreamNonBlocking));
  PDG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->pipe_k2, cudaStreamNonBlocking));
  for (int i = 0; i < 2 * kMaxSlabs + 3; i++)
    PDG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->pipe_ev[i], cudaEventDisableTiming));
  return PDG_OK;
}

// number of slabs (1: no pipelining) and planes per slab
static int pipe_slabs(const pdg_context *ctx, long *planes_per_slab) {
  const long planes = ctx->cfg.cells[ctx->dim - 1];
  long s = ctx->ncell / kMinSlabCells;
  if (s > kMaxSlabs) s = kMaxSlabs;
  if (s > planes) s = planes;
  if (s < 2) return 1;
  const long pps = (planes + s - 1) / s;
  *planes_per_slab = pps;
  return (int)((planes + pps - 1) / pps);
}

// y = (acc ? y : 0) + alpha J x + add with x and/or y in host memory;
// xdev/ydev: the device copies (staging buffers for host vectors)
static int apply_pipelined(pdg_context *ctx, const double *x, double *y, const double *xdev,
                           double *ydev, bool hx, bool hy, const double *add, double alpha,
                           int acc, int transpose, int nslab, long pps) {
  PDG_TRY(pipe_ready(ctx));
  PDG_TRY(prepare_apply64(ctx, transpose));
  const long plane = ctx->ncell / ctx->cfg.cells[ctx->dim - 1];
  const long nb = ctx->nb;
  cudaEvent_t *ev_in = ctx->pipe_ev, *ev_out = ctx->pipe_ev + kMaxSlabs;
  cudaEvent_t ev_start = ctx->pipe_ev[2 * kMaxSlabs], ev_end = ctx->pipe_ev[2 * kMaxSlabs + 1];
  cudaEvent_t ev_k2 = ctx->pipe_ev[2 * kMaxSlabs + 2];
  // the side streams start after the work already queued on the context stream
  PDG_CUDA_TRY(cudaEventRecord(ev_start, ctx->stream));
  PDG_CUDA_TRY(cudaStreamWaitEvent(ctx->pipe_h2d, ev_start, 0));
  PDG_CUDA_TRY(cudaStreamWaitEvent(ctx->pipe_d2h, ev_start, 0));
  PDG_CUDA_TRY(cudaStreamWaitEvent(ctx->pipe_k2, ev_start, 0));
  cudaStream_t const ctx_stream = ctx->stream;
  auto range = [&](int s, long *c0, long *c1) {
    *c0 = s * pps * plane;
    *c1 = std::min(ctx->ncell, (s + 1) * pps * plane);
  };
  for (int s = 0; s < nslab; s++) {
    long c0, c1;
    range(s, &c0, &c1);
    const size_t off = (size_t)(c0 * nb), bytes = sizeof(double) * (size_t)((c1 - c0) * nb);
    if (hx)
      PDG_CUDA_TRY(cudaMemcpyAsync((double *)xdev + off, x + off, bytes, cudaMemcpyHostToDevice,
                                   ctx->pipe_h2d));
    if (hy && acc)
      PDG_CUDA_TRY(cudaMemcpyAsync(ydev + off, y + off, bytes, cudaMemcpyHostToDevice,
                                   ctx->pipe_h2d));
    PDG_CUDA_TRY(cudaEventRecord(ev_in[s], ctx->pipe_h2d));
  }
  int st = PDG_OK;
  for (int s = 0; s < nslab && st == PDG_OK; s++) {
    long c0, c1;
    range(s, &c0, &c1);
    // the launchers enqueue on ctx->stream: point it at this slab's stream
    ctx->stream = (s & 1) ? ctx->pipe_k2 : ctx_stream;
    if ((st = cuda_status(cudaStreamWaitEvent(ctx->stream, ev_in[std::min(s + 1, nslab - 1)],
                                              0))))
      break;
    ApplyArgs<double> a{xdev, ydev, add, alpha, acc, transpose, 0, nullptr, nullptr,
                        (int)(c1 - c0), (int)c0};
    if ((st = launch_apply<double>(ctx, a, ctx->K64, ctx->c64, ctx->tab64))) break;
    if (hy) {
      const size_t off = (size_t)(c0 * nb), bytes = sizeof(double) * (size_t)((c1 - c0) * nb);
      if ((st = cuda_status(cudaEventRecord(ev_out[s], ctx->stream))) ||
          (st = cuda_status(cudaStreamWaitEvent(ctx->pipe_d2h, ev_out[s], 0))) ||
          (st = cuda_status(cudaMemcpyAsync(y + off, ydev + off, bytes, cudaMemcpyDeviceToHost,
                                            ctx->pipe_d2h))))
        break;
    }
  }
  ctx->stream = ctx_stream;
  PDG_TRY(st);
  PDG_CUDA_TRY(cudaEventRecord(ev_k2, ctx->pipe_k2));
  PDG_CUDA_TRY(cudaEventRecord(ev_end, ctx->pipe_d2h));
  PDG_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_k2, 0));
  PDG_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_end, 0));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

// y = (acc ? y : 0) + alpha J x + (with_r0 ? R(0) : 0), host or device vectors
static int apply_entry(pdg_context *ctx, const double *x, double *y, double alpha, int acc,
                       int transpose, bool with_r0) {
  PDG_CHECK_CTX(ctx);
  if (!x || !y) return set_error(PDG_EINVAL, "null vector");
  if (with_r0) PDG_TRY(ensure_r0(ctx));
  const bool hx = !is_device_ptr(x), hy = !is_device_ptr(y);
  if (hx || hy) PDG_TRY(ensure_stage(ctx));
  long pps = 0;
  const int nslab = (hx || hy) ? pipe_slabs(ctx, &pps) : 1;
  if (nslab > 1 && !ctx->use_matrix && !ctx->ops32 && ctx->nl_deg == 0 &&
      ctx->basis != PDG_BASIS_LEGENDRE)
    return apply_pipelined(ctx, x, y, hx ? ctx->stage_a : x, hy ? ctx->stage_b : y, hx, hy,
                           with_r0 ? ctx->r0 : nullptr, alpha, acc, transpose, nslab, pps);
  Staged<double> sx, sy;
  PDG_TRY(stage_in<double>(ctx, x, ctx->ndof, ctx->stage_a, true, &sx));
  PDG_TRY(stage_in<double>(ctx, y, ctx->ndof, ctx->stage_b, acc != 0, &sy));
  if (with_r0 && ctx->nl_deg > 0) {
    // R(x) = J_lin x + R(0) + int q(u) psi: the linearized term stays out
    ctx->nl_off = 1;
    const int st = op_launch<double>(ctx, sx.dev, sy.dev, ctx->r0, alpha, acc, transpose, nullptr);
    ctx->nl_off = 0;
    PDG_TRY(st);
    PDG_TRY(nl_residual(ctx, sx.dev, sy.dev));
  } else {
    PDG_TRY(op_launch<double>(ctx, sx.dev, sy.dev, with_r0 ? ctx->r0 : nullptr, alpha, acc,
                              transpose, nullptr));
  }
  PDG_TRY(stage_out<double>(ctx, sy));
  return PDG_OK;
}

// r = R(x) on device vectors (overwrites r)
static int residual_dev(pdg_context *ctx, const double *x, double *r) {
  PDG_TRY(ensure_r0(ctx));
  ctx->nl_off = 1;
  const int st = op_launch<double>(ctx, x, r, ctx->r0, 1.0, 0, 0, nullptr);
  ctx->nl_off = 0;
  PDG_TRY(st);
  return nl_residual(ctx, x, r);
}

static int norm_dev(pdg_context *ctx, const double *v, double *out) {
  const RedCtx rc = red_ctx(ctx);
  PDG_TRY(red_dot(ctx, rc, ctx->ndof, v, v, nullptr, nullptr, FIN_NORM, S_DOT, -1, false));
  double scal[S_COUNT];
  PDG_TRY(fetch_state(ctx, scal, nullptr));
  *out = scal[S_DOT];
  return PDG_OK;
}

int pdg_residual(pdg_context *ctx, const double *x, double *r) {
  return apply_entry(ctx, x, r, 1.0, 1, 0, true);
}
int pdg_jacobian_apply(pdg_context *ctx, const double *z, double *y) {
  return apply_entry(ctx, z, y, 1.0, 1, 0, false);
}
int pdg_jacobian_apply_transpose(pdg_context *ctx, const double *z, double *y) {
  return apply_entry(ctx, z, y, 1.0, 1, 1, false);
}
int pdg_apply(pdg_context *ctx, const double *x, double *y) {
  return apply_entry(ctx, x, y, 1.0, 0, 0, false);
}
int pdg_applyscaleadd(pdg_context *ctx, double alpha, const double *x, double *y) {
  return apply_entry(ctx, x, y, alpha, 1, 0, false);
}

int pdg_jacobian_apply_f32(pdg_context *ctx, const float *z, float *y) {
  PDG_CHECK_CTX(ctx);
  if (!z || !y) return set_error(PDG_EINVAL, "null vector");
  if (!is_device_ptr(z) || !is_device_ptr(y))
    return set_error(PDG_EINVAL, "pdg_jacobian_apply_f32 takes device pointers");
  return op_launch<float>(ctx, z, y, nullptr, 1.f, 1, 0, nullptr);
}
int pdg_apply_f32(pdg_context *ctx, const float *x, float *y) {
  PDG_CHECK_CTX(ctx);
  if (!x || !y) return set_error(PDG_EINVAL, "null vector");
  if (!is_device_ptr(x) || !is_device_ptr(y))
    return set_error(PDG_EINVAL, "pdg_apply_f32 takes device pointers");
  return op_launch<float>(ctx, x, y, nullptr, 1.f, 0, 0, nullptr);
}
int pdg_jacobian_apply_transpose_f32(pdg_context *ctx, const float *z, float *y) {
  PDG_CHECK_CTX(ctx);
  if (!z || !y) return set_error(PDG_EINVAL, "null vector");
  if (!is_device_ptr(z) || !is_device_ptr(y))
    return set_error(PDG_EINVAL, "pdg_jacobian_apply_transpose_f32 takes device pointers");
  return op_launch<float>(ctx, z, y, nullptr, 1.f, 1, 1, nullptr);
}

int pdg_prec_setup(pdg_context *ctx, int kind, int precision) {
  PDG_CHECK_CTX(ctx);
  return prec_setup_impl(ctx, kind, precision);
}

static int prec_entry(pdg_context *ctx, const double *d, double *v, int transpose) {
  PDG_CHECK_CTX(ctx);
  if (!d || !v) return set_error(PDG_EINVAL, "null vector");
  const bool hd = !is_device_ptr(d), hv = !is_device_ptr(v);
  if (hd || hv) PDG_TRY(ensure_stage(ctx));
  Staged<double> sd, sv;
  PDG_TRY(stage_in<double>(ctx, d, ctx->ndof, ctx->stage_a, true, &sd));
  PDG_TRY(stage_in<double>(ctx, v, ctx->ndof, ctx->stage_b, false, &sv));
  PDG_TRY(prec_apply_impl<double>(ctx, sd.dev, sv.dev, transpose));
  PDG_TRY(stage_out<double>(ctx, sv));
  return PDG_OK;
}
int pdg_prec_apply(pdg_context *ctx, const double *d, double *v) {
  return prec_entry(ctx, d, v, 0);
}
int pdg_prec_apply_transpose(pdg_context *ctx, const double *d, double *v) {
  return prec_entry(ctx, d, v, 1);
}
int pdg_prec_apply_f32(pdg_context *ctx, const float *d, float *v) {
  PDG_CHECK_CTX(ctx);
  if (!d || !v) return set_error(PDG_EINVAL, "null vector");
  if (!is_device_ptr(d) || !is_device_ptr(v))
    return set_error(PDG_EINVAL, "pdg_prec_apply_f32 takes device pointers");
  return prec_apply_impl<float>(ctx, d, v, 0);
}

static int dot_entry(pdg_context *ctx, const double *a, const double *b, double *out, bool norm) {
  PDG_CHECK_CTX(ctx);
  if (!a || !b || !out) return set_error(PDG_EINVAL, "null argument");
  const bool ha = !is_device_ptr(a), hb = !is_device_ptr(b);
  if (ha || hb) PDG_TRY(ensure_stage(ctx));
  Staged<double> sa, sb;
  PDG_TRY(stage_in<double>(ctx, a, ctx->ndof, ctx->stage_a, true, &sa));
  PDG_TRY(stage_in<double>(ctx, b, ctx->ndof, ctx->stage_b, true, &sb));
  const RedCtx rc = red_ctx(ctx);
  PDG_TRY(red_dot(ctx, rc, ctx->ndof, sa.dev, sb.dev, nullptr, nullptr,
                  norm ? FIN_NORM : FIN_STORE, S_DOT, -1, false));
  double scal[S_COUNT];
  PDG_TRY(fetch_state(ctx, scal, nullptr));
  *out = scal[S_DOT];
  return PDG_OK;
}
int pdg_norm(pdg_context *ctx, const double *v, double *out) {
  return dot_entry(ctx, v, v, out, true);
}
int pdg_dot(pdg_context *ctx, const double *a, const double *b, double *out) {
  return dot_entry(ctx, a, b, out, false);
}

static int check_opts(const pdg_solver_options *o) {
  if (!o) return set_error(PDG_EINVAL, "null options");
  if (o->method != PDG_CG && o->method != PDG_BICGSTAB && o->method != PDG_GMRES)
    return set_error(PDG_EINVAL, "bad method");
  if (o->inner_method < -1 || o->inner_method > PDG_GMRES)
    return set_error(PDG_EINVAL, "bad inner method");
  if ((o->method == PDG_GMRES || o->inner_method != PDG_CG) && (o->restart < 1 || o->restart > 64))
    return set_error(PDG_EINVAL, "GMRES restart length must be 1..64");
  if (o->mixed < 0 || o->mixed > 3) return set_error(PDG_EINVAL, "mixed must be 0..3");
  if (o->assembled != 0 && o->assembled != 1) return set_error(PDG_EINVAL, "bad assembled flag");
  if ((o->preconditioner & ~(PDG_PREC_BLOCK_MASK | PDG_PREC_SOR)) != 0 ||
      (o->preconditioner & PDG_PREC_BLOCK_MASK) > PDG_PREC_BJ_ITERATIVE)
    return set_error(PDG_EINVAL, "bad preconditioner kind");
  if (o->inner_vectors < -1 || o->inner_vectors > PDG_F32)
    return set_error(PDG_EINVAL, "bad inner vector precision");
  if (o->maxit < 1 || (o->mixed && (o->inner_maxit < 1 || o->max_outer < 1)))
    return set_error(PDG_EINVAL, "iteration caps must be >= 1");
  if (!(o->reduction > 0)) return set_error(PDG_EINVAL, "reduction must be > 0");
  return PDG_OK;
}

int pdg_set_nonlinearity(pdg_context *ctx, int degree, const double *coef) {
  PDG_CHECK_CTX(ctx);
  if (coef && (degree < 1 || degree > 4)) return set_error(PDG_EINVAL, "degree must be 1..4");
  if (coef && ctx->basis == PDG_BASIS_LEGENDRE)
    return set_error(PDG_EUNSUPPORTED, "the nonlinear volume term needs a nodal basis");
  ctx->nl_deg = coef ? degree : 0;
  for (int m = 0; m < 5; m++) ctx->nl_coef[m] = (coef && m <= degree) ? coef[m] : 0.0;
  ctx->nl_point = 0;
  invalidate(ctx, true);
  return PDG_OK;
}

int pdg_set_linearization_point(pdg_context *ctx, const double *x) {
  PDG_CHECK_CTX(ctx);
  if (!x) return set_error(PDG_EINVAL, "null vector");
  PDG_TRY(ensure_stage(ctx));
  Staged<double> sx;
  PDG_TRY(stage_in<double>(ctx, x, ctx->ndof, ctx->stage_a, true, &sx));
  PDG_TRY(nl_set_point(ctx, sx.dev));
  ctx->A_valid = 0;
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

int pdg_jacobian_apply_nonlinear(pdg_context *ctx, const double *x, const double *z, double *y) {
  PDG_TRY(pdg_set_linearization_point(ctx, x));
  return apply_entry(ctx, z, y, 1.0, 1, 0, false);
}

void pdg_default_newton_options(pdg_newton_options *o) {
  if (!o) return;
  o->reduction = 1e-8;
  o->absolute_limit = 1e-12;
  o->max_iterations = 40;
  o->force_iteration = 0;
  o->min_linear_reduction = 1e-3;
  o->fixed_linear_reduction = 0;
  o->line_search = 1;
  o->line_search_max_iterations = 10;
  o->line_search_damping = 0.5;
  o->line_search_accept_best = 0;
  o->verbose = 0;
}

// NewtonMethod::apply (solver/newton.hh:177-335) on device vectors.
static int newton_run(pdg_context *ctx, const pdg_newton_options *opt,
                      const pdg_solver_options *lin, double *u, pdg_newton_result *res,
                      double *r, double *z, double *uprev) {
  const long n = ctx->ndof;
  double defect = 0.0;
  // updateDefect (:341-369): r = R(u), defect = |r|
  auto update_defect = [&]() -> int {
    PDG_TRY(residual_dev(ctx, u, r));
    return norm_dev(ctx, r, &defect);
  };
  PDG_TRY(update_defect());
  res->first_defect = defect;
  res->defect = defect;
  double prev = defect;
  int prec_ready = 0;
  for (;;) {
    // DefaultTerminate::terminate (terminate.hh:29-40)
    if (!(opt->force_iteration && res->iterations == 0)) {
      res->converged = defect < opt->absolute_limit || defect < res->first_defect * opt->reduction;
      if (res->converged) break;
      if (res->iterations >= opt->max_iterations)
        return set_error(PDG_ENOTCONVERGED, "Newton: maximum iteration count reached");
    }
    if (!std::isfinite(defect)) return set_error(PDG_ENONFINITE, "Newton: non-finite defect");
    // prepareStep (:99-143): linear reduction
    double linred = opt->min_linear_reduction;
    if (!opt->fixed_linear_reduction &&
        !(res->iterations == 0 && res->first_defect < opt->absolute_limit)) {
      const double stop = std::max(res->first_defect * opt->reduction, opt->absolute_limit);
      linred = std::max(stop / (10 * defect),
                        std::min(opt->min_linear_reduction, defect * defect / (prev * prev)));
    }
    prev = defect;
    // linearSolve (:145-170) at the linearization point u
    PDG_TRY(nl_set_point(ctx, u));
    ctx->A_valid = 0;
    if (!prec_ready) {
      // GridOperatorPreconditioner::pre sets the block preconditioner up
      // once, at the first linearization point (gridoperatorpreconditioner.hh:45-75)
      PDG_TRY(prec_setup_impl(ctx, lin->preconditioner, lin->mixed ? PDG_F32 : PDG_F64));
      prec_ready = 1;
    }
    pdg_solver_options o = *lin;
    o.reduction = linred;
    PDG_TRY(vec_fill<double>(ctx, n, z, 0.0));
    pdg_solver_result lr;
    std::memset(&lr, 0, sizeof(lr));
    const int ls = solve_correction(ctx, &o, z, r, 0, &lr);
    res->linear_solver_iterations += lr.iterations;
    if (ls != PDG_OK && ls != PDG_ENOTCONVERGED) return ls;
    // line search (linesearch.hh:81-165)
    if (!opt->line_search || defect < opt->absolute_limit) {
      PDG_TRY(vec_axpy(ctx, n, -1.0, z, u));
      PDG_TRY(update_defect());
    } else {
      double lambda = 1.0, best_lambda = 0.0, best = defect;
      const double previous = defect;
      bool ok = false;
      PDG_TRY(vec_copy<double>(ctx, n, u, uprev));
      for (int it = 0; it < opt->line_search_max_iterations; it++) {
        PDG_TRY(vec_axpy(ctx, n, -lambda, z, u));
        PDG_TRY(update_defect());
        if (defect <= (1.0 - lambda / 4) * previous) { ok = true; break; }
        if (defect < best) { best = defect; best_lambda = lambda; }
        lambda *= opt->line_search_damping;
        PDG_TRY(vec_copy<double>(ctx, n, uprev, u));
      }
      if (!ok) {
        if (!opt->line_search_accept_best || best_lambda == 0.0) {
          PDG_TRY(vec_copy<double>(ctx, n, uprev, u));
          PDG_TRY(update_defect());
          res->defect = defect;
          return set_error(PDG_ELINESEARCH, "Newton: line search failed");
        }
        if (best_lambda != lambda) {
          PDG_TRY(vec_copy<double>(ctx, n, uprev, u));
          PDG_TRY(vec_axpy(ctx, n, -best_lambda, z, u));
          PDG_TRY(update_defect());
        }
      }
    }
    res->iterations++;
    res->defect = defect;
    res->reduction = res->first_defect > 0 ? defect / res->first_defect : 0.0;
    res->conv_rate = std::pow(res->reduction, 1.0 / res->iterations);
    if (opt->verbose)
      std::fprintf(stderr, "pdg newton: iteration %d defect %.3e (linear %d its, reduction %.2e)\n",
                   res->iterations, defect, lr.iterations, linred);
  }
  res->defect = defect;
  res->reduction = res->first_defect > 0 ? defect / res->first_defect : 0.0;
  return PDG_OK;
}

int pdg_newton_solve(pdg_context *ctx, const pdg_newton_options *opt,
                     const pdg_solver_options *lin, double *u, pdg_newton_result *res) {
  PDG_CHECK_CTX(ctx);
  if (!opt || !lin || !u || !res) return set_error(PDG_EINVAL, "null argument");
  PDG_TRY(check_opts(lin));
  if (opt->max_iterations < 1 || !(opt->line_search_damping > 0 && opt->line_search_damping < 1))
    return set_error(PDG_EINVAL, "bad Newton options");
  std::memset(res, 0, sizeof(*res));
  PDG_TRY(ensure_stage(ctx));
  PDG_TRY(ensure_work(ctx, lin->mixed != 0));
  Staged<double> su;
  PDG_TRY(stage_in<double>(ctx, u, ctx->ndof, ctx->stage_a, true, &su));
  double *buf[3] = {nullptr, nullptr, nullptr};
  for (auto &b : buf)
    if (cudaMalloc(&b, sizeof(double) * ctx->ndof) != cudaSuccess) {
      for (auto &c : buf)
        if (c) cudaFree(c);
      return set_error(PDG_ECUDA, "out of device memory for Newton");
    }
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, ctx->stream);
  const int st = newton_run(ctx, opt, lin, su.dev, res, buf[0], buf[1], buf[2]);
  cudaEventRecord(t1, ctx->stream);
  cudaEventSynchronize(t1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  res->elapsed = ms * 1e-3;
  res->status = st;
  for (auto &b : buf) cudaFree(b);
  const int so = stage_out<double>(ctx, su);
  return st != PDG_OK ? st : so;
}

int pdg_mass_apply(pdg_context *ctx, const double *x, double *y) {
  PDG_CHECK_CTX(ctx);
  if (!x || !y) return set_error(PDG_EINVAL, "null vector");
  PDG_TRY(ensure_stage(ctx));
  Staged<double> sx, sy;
  PDG_TRY(stage_in<double>(ctx, x, ctx->ndof, ctx->stage_a, true, &sx));
  PDG_TRY(stage_in<double>(ctx, y, ctx->ndof, ctx->stage_b, false, &sy));
  PDG_TRY(mass_apply(ctx, sx.dev, sy.dev, 1.0, 0, 0));
  PDG_TRY(stage_out<double>(ctx, sy));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

// Tables of instationary/onestepparameter.hh (the published schemes:
// theta method, Alexander's SDIRK 2 and 3, the fractional-step theta scheme,
// Heun, Shu's SSP RK3, classical RK4), row r-1 = stage r.
int pdg_onestep_table(int method, double theta, int *stages, double *A, double *B, double *D) {
  if (!stages || !A || !B || !D) return set_error(PDG_EINVAL, "null argument");
  double a[4][5] = {}, b[4][5] = {}, d[5] = {};
  int s = 0;
  switch (method) {
    case PDG_ONESTEP_IMPLICIT_EULER: theta = 1.0; [[fallthrough]];
    case PDG_ONESTEP_EXPLICIT_EULER:
      if (method == PDG_ONESTEP_EXPLICIT_EULER) theta = 0.0;
      [[fallthrough]];
    case PDG_ONESTEP_THETA:
      s = 1;
      d[0] = 0.0; d[1] = 1.0;
      a[0][0] = -1.0; a[0][1] = 1.0;
      b[0][0] = 1.0 - theta; b[0][1] = theta;
      break;
    case PDG_ONESTEP_ALEXANDER2: {
      const double al = 1.0 - 0.5 * std::sqrt(2.0);
      s = 2;
      d[0] = 0.0; d[1] = al; d[2] = 1.0;
      a[0][0] = -1.0; a[0][1] = 1.0;
      a[1][0] = -1.0; a[1][2] = 1.0;
      b[0][1] = al;
      b[1][1] = 1.0 - al; b[1][2] = al;
      break;
    }
    case PDG_ONESTEP_ALEXANDER3: {
      // alpha: root of alpha^3 - 3 alpha^2 + 1.5 alpha - 1/6 = 0 near 0.4359 (Newton)
      double al = 0.4358665215;
      for (int i = 0; i < 10; i++)
        al = al - (al * (al * al - 3.0 * (al - 0.5)) - 1.0 / 6.0) / (3.0 * al * (al - 2.0) + 1.5);
      const double tau2 = (1.0 + al) * 0.5;
      const double b1 = -(6.0 * al * al - 16.0 * al + 1.0) * 0.25;
      const double b2 = (6 * al * al - 20.0 * al + 5.0) * 0.25;
      s = 3;
      d[0] = 0.0; d[1] = al; d[2] = tau2; d[3] = 1.0;
      a[0][0] = -1.0; a[0][1] = 1.0;
      a[1][0] = -1.0; a[1][2] = 1.0;
      a[2][0] = -1.0; a[2][3] = 1.0;
      b[0][1] = al;
      b[1][1] = tau2 - al; b[1][2] = al;
      b[2][1] = b1; b[2][2] = b2; b[2][3] = al;
      break;
    }
    case PDG_ONESTEP_FRACTIONAL_STEP: {
      const double th = 1.0 - 0.5 * std::sqrt(2.0), thp = 1.0 - 2.0 * th;
      const double al = 2.0 - std::sqrt(2.0), be = 1.0 - al;
      s = 3;
      d[0] = 0.0; d[1] = th; d[2] = 1.0 - th; d[3] = 1.0;
      a[0][0] = -1.0; a[0][1] = 1.0;
      a[1][1] = -1.0; a[1][2] = 1.0;
      a[2][2] = -1.0; a[2][3] = 1.0;
      b[0][0] = be * th; b[0][1] = al * th;
      b[1][1] = al * thp; b[1][2] = al * th;
      b[2][2] = be * th; b[2][3] = al * th;
      break;
    }
    case PDG_ONESTEP_HEUN:
      s = 2;
      d[0] = 0.0; d[1] = 1.0; d[2] = 1.0;
      a[0][0] = -1.0; a[0][1] = 1.0;
      a[1][0] = -0.5; a[1][1] = -0.5; a[1][2] = 1.0;
      b[0][0] = 1.0;
      b[1][1] = 0.5;
      break;
    case PDG_ONESTEP_SHU3:
      s = 3;
      d[0] = 0.0; d[1] = 1.0; d[2] = 0.5; d[3] = 1.0;
      a[0][0] = -1.0; a[0][1] = 1.0;
      a[1][0] = -0.75; a[1][1] = -0.25; a[1][2] = 1.0;
      a[2][0] = -1.0 / 3.0; a[2][2] = -2.0 / 3.0; a[2][3] = 1.0;
      b[0][0] = 1.0;
      b[1][1] = 0.25;
      b[2][2] = 2.0 / 3.0;
      break;
    case PDG_ONESTEP_RK4:
      s = 4;
      d[0] = 0.0; d[1] = 0.5; d[2] = 0.5; d[3] = 1.0; d[4] = 1.0;
      for (int r = 0; r < 4; r++) { a[r][0] = -1.0; a[r][r + 1] = 1.0; }
      b[0][0] = 0.5;
      b[1][1] = 0.5;
      b[2][2] = 1.0;
      b[3][0] = 1.0 / 6.0; b[3][1] = 1.0 / 3.0; b[3][2] = 1.0 / 3.0; b[3][3] = 1.0 / 6.0;
      break;
    default:
      return set_error(PDG_EINVAL, "unknown one-step method");
  }
  *stages = s;
  for (int r = 0; r < s; r++)
    for (int i = 0; i <= s; i++) {
      A[r * (s + 1) + i] = a[r][i];
      B[r * (s + 1) + i] = b[r][i];
    }
  for (int i = 0; i <= s; i++) D[i] = d[i];
  return PDG_OK;
}

__global__ void k_shift_c(long n, const double *c, double sigma, double *c64, float *c32) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = (c ? c[i] : 0.0) + sigma;
  c64[i] = v;
  c32[i] = (float)v;
}

// Use J + sigma M as the operator: reaction c -> c + sigma (the mass term
// int u psi is the reaction term with unit coefficient).  sigma = 0 with
// `restore` puts the original coefficient back.
static int set_mass_shift(pdg_context *ctx, double sigma, bool restore, double *c_orig64,
                          float *c_orig32) {
  if (restore) {
    ctx->c64 = c_orig64;
    ctx->c32 = c_orig32;
    ctx->mass_shift = 0.0;
    invalidate(ctx, true);
    return PDG_OK;
  }
  if (!ctx->cstage64) {
    PDG_CUDA_TRY(cudaMalloc(&ctx->cstage64, sizeof(double) * ctx->ncell));
    PDG_CUDA_TRY(cudaMalloc(&ctx->cstage32, sizeof(float) * ctx->ncell));
  }
  k_shift_c<<<(unsigned)((ctx->ncell + 255) / 256), 256, 0, ctx->stream>>>(
      ctx->ncell, c_orig64, sigma, ctx->cstage64, ctx->cstage32);
  PDG_CUDA_TRY(cudaGetLastError());
  ctx->c64 = ctx->cstage64;
  ctx->c32 = ctx->cstage32;
  ctx->mass_shift = sigma;
  invalidate(ctx, true);
  return PDG_OK;
}

static int onestep_run(pdg_context *ctx, int s, const double *A, const double *B, double dt,
                       const pdg_solver_options *lin, const double *xold, double *xnew,
                       pdg_onestep_result *res, std::vector<double *> &buf) {
  const long n = ctx->ndof;
  // buf: X[1..s-1] stage values, RX[0..s-1] = R(x_j), MX[0..s-1] = M x_j, C, r, z
  double **X = buf.data();                 // X[0] unused (xold), X[s] = xnew
  double **RX = X + s + 1, **MX = RX + s;
  double *C = buf[3 * s + 1], *r = buf[3 * s + 2], *z = buf[3 * s + 3];
  const double *x0 = xold;
  auto xs = [&](int j) -> const double * { return j == 0 ? x0 : (j == s ? xnew : X[j]); };
  // R(x) = (J + shift M) x - shift M x + R(0) with whatever shift is active
  auto spatial_residual = [&](const double *x, double *out, double *mx) -> int {
    PDG_TRY(mass_apply(ctx, x, mx, 1.0, 0, 0));
    PDG_TRY(ensure_r0(ctx));
    PDG_TRY(op_launch<double>(ctx, x, out, ctx->r0, 1.0, 0, 0, nullptr));
    if (ctx->mass_shift != 0.0) PDG_TRY(vec_axpy(ctx, n, -ctx->mass_shift, mx, out));
    return PDG_OK;
  };
  PDG_TRY(spatial_residual(x0, RX[0], MX[0]));
  for (int rr = 1; rr <= s; rr++) {
    const double *a = A + (rr - 1) * (s + 1), *b = B + (rr - 1) * (s + 1);
    // constant part C = sum_{j<r} [b_rj dt R(x_j) + a_rj M x_j]
    PDG_TRY(vec_fill<double>(ctx, n, C, 0.0));
    for (int j = 0; j < rr; j++) {
      if (b[j] != 0.0) PDG_TRY(vec_axpy(ctx, n, b[j] * dt, RX[j], C));
      if (a[j] != 0.0) PDG_TRY(vec_axpy(ctx, n, a[j], MX[j], C));
    }
    double *xr = const_cast<double *>(xs(rr));
    const double arr = a[rr], brr = b[rr];
    if (brr == 0.0) {
      // explicit stage: a_rr M x_r = -C
      if (arr == 0.0) return set_error(PDG_EINVAL, "singular one-step stage");
      PDG_TRY(mass_apply(ctx, C, xr, -1.0 / arr, 0, 1));
    } else {
      // implicit stage: (J + sigma M) x = -C/(b_rr dt) - R(0), sigma = a_rr/(b_rr dt);
      // residual form from the previous stage value as initial guess
      const double sigma = arr / (brr * dt);
      if (sigma != ctx->mass_shift || !ctx->mass_shift_on) {
        PDG_TRY(set_mass_shift(ctx, sigma, false, ctx->c_orig64, ctx->c_orig32));
        ctx->mass_shift_on = 1;
      }
      PDG_TRY(vec_copy<double>(ctx, n, xs(rr - 1), xr));
      PDG_TRY(ensure_r0(ctx));
      PDG_TRY(op_launch<double>(ctx, xr, r, ctx->r0, 1.0, 0, 0, nullptr));
      PDG_TRY(vec_axpy(ctx, n, 1.0 / (brr * dt), C, r));
      PDG_TRY(vec_fill<double>(ctx, n, z, 0.0));
      pdg_solver_result lr;
      std::memset(&lr, 0, sizeof(lr));
      const int st = solve_correction(ctx, lin, z, r, 0, &lr);
      res->linear_solver_iterations += lr.iterations;
      if (st != PDG_OK) return st;
      PDG_TRY(vec_axpy(ctx, n, -1.0, z, xr));
    }
    if (rr < s) PDG_TRY(spatial_residual(xr, RX[rr], MX[rr]));
  }
  res->stages = s;
  return PDG_OK;
}

int pdg_onestep_apply(pdg_context *ctx, int stages, const double *A, const double *B,
                      const double *D, double dt, const pdg_solver_options *lin,
                      const double *xold, double *xnew, pdg_onestep_result *res) {
  PDG_CHECK_CTX(ctx);
  if (!A || !B || !D || !lin || !xold || !xnew || !res)
    return set_error(PDG_EINVAL, "null argument");
  if (stages < 1 || stages > 4 || !(dt > 0)) return set_error(PDG_EINVAL, "bad stages or dt");
  PDG_TRY(check_opts(lin));
  if (ctx->nl_deg > 0)
    return set_error(PDG_EUNSUPPORTED, "one-step methods with a nonlinear operator");
  std::memset(res, 0, sizeof(*res));
  PDG_TRY(ensure_stage(ctx));
  PDG_TRY(ensure_work(ctx, lin->mixed != 0));
  const long n = ctx->ndof;
  Staged<double> so, sn;
  PDG_TRY(stage_in<double>(ctx, xold, n, ctx->stage_a, true, &so));
  PDG_TRY(stage_in<double>(ctx, xnew, n, ctx->stage_b, false, &sn));
  std::vector<double *> buf(3 * stages + 4, nullptr);
  for (auto &p : buf)
    if (cudaMalloc(&p, sizeof(double) * n) != cudaSuccess) {
      for (auto &q : buf)
        if (q) cudaFree(q);
      return set_error(PDG_ECUDA, "out of device memory for the stages");
    }
  ctx->c_orig64 = ctx->c64;
  ctx->c_orig32 = ctx->c32;
  ctx->mass_shift = 0.0;
  ctx->mass_shift_on = 0;
  cudaEventRecord(ctx->ev0, ctx->stream);
  int st = onestep_run(ctx, stages, A, B, dt, lin, so.dev, sn.dev, res, buf);
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaEventSynchronize(ctx->ev1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  res->elapsed = ms * 1e-3;
  if (ctx->mass_shift_on) set_mass_shift(ctx, 0.0, true, ctx->c_orig64, ctx->c_orig32);
  ctx->mass_shift_on = 0;
  for (auto &p : buf) cudaFree(p);
  res->status = st;
  if (st != PDG_OK) return st;
  PDG_TRY(stage_out<double>(ctx, sn));
  return PDG_OK;
}

int pdg_jacobian_assemble(pdg_context *ctx) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(ensure_work(ctx, false));
  PDG_TRY(assemble_jacobian(ctx));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

int pdg_jacobian_pattern(const pdg_context *ctx, long *nnz_blocks) {
  if (!ctx || !nnz_blocks) return set_error(PDG_EINVAL, "null argument");
  *nnz_blocks = jacobian_nnz_blocks(ctx);
  return PDG_OK;
}

int pdg_jacobian_export(pdg_context *ctx, long *rowptr, long *colind, double *values) {
  PDG_CHECK_CTX(ctx);
  if (!ctx->A_valid) return set_error(PDG_EINVAL, "the Jacobian has not been assembled");
  const long nnzb = jacobian_nnz_blocks(ctx);
  std::vector<long> rp(ctx->ncell + 1), ci(nnzb);
  PDG_TRY(jacobian_rowptr(ctx, rp.data(), ci.data()));
  if (rowptr) std::memcpy(rowptr, rp.data(), sizeof(long) * rp.size());
  if (colind) std::memcpy(colind, ci.data(), sizeof(long) * ci.size());
  if (!values) return PDG_OK;
  const size_t nval = (size_t)nnzb * ctx->nb * ctx->nb;
  long *rp_dev = nullptr;
  double *vdev = nullptr;
  const bool host = !is_device_ptr(values);
  int st = PDG_OK;
  if (cudaMalloc(&rp_dev, sizeof(long) * rp.size()) != cudaSuccess ||
      (host && cudaMalloc(&vdev, sizeof(double) * nval) != cudaSuccess)) {
    st = set_error(PDG_ECUDA, "out of device memory for the export");
  } else {
    cudaMemcpyAsync(rp_dev, rp.data(), sizeof(long) * rp.size(), cudaMemcpyHostToDevice,
                    ctx->stream);
    st = matrix_export(ctx, rp_dev, host ? vdev : values);
    if (st == PDG_OK && host &&
        cudaMemcpyAsync(values, vdev, sizeof(double) * nval, cudaMemcpyDeviceToHost,
                        ctx->stream) != cudaSuccess)
      st = set_error(PDG_ECUDA, "export copy failed");
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && st == PDG_OK)
      st = set_error(PDG_ECUDA, "export failed");
  }
  if (rp_dev) cudaFree(rp_dev);
  if (vdev) cudaFree(vdev);
  return st;
}

int pdg_matrix_apply(pdg_context *ctx, const double *x, double *y) {
  PDG_CHECK_CTX(ctx);
  if (!x || !y) return set_error(PDG_EINVAL, "null vector");
  if (!ctx->A_valid) return set_error(PDG_EINVAL, "the Jacobian has not been assembled");
  UseMatrixScope use_matrix(ctx, 1);
  return apply_entry(ctx, x, y, 1.0, 0, 0, false);
}

int pdg_krylov_solve(pdg_context *ctx, const pdg_solver_options *opt, double *z, double *r,
                     pdg_solver_result *res) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(check_opts(opt));
  if (!z || !r || !res) return set_error(PDG_EINVAL, "null argument");
  std::memset(res, 0, sizeof(*res));
  PDG_TRY(ensure_stage(ctx));
  Staged<double> sz, sr;
  PDG_TRY(stage_in<double>(ctx, z, ctx->ndof, ctx->stage_a, true, &sz));
  PDG_TRY(stage_in<double>(ctx, r, ctx->ndof, ctx->stage_b, true, &sr));
  const int st = solve_correction(ctx, opt, sz.dev, sr.dev, 0, res);
  PDG_TRY(stage_out<double>(ctx, sz));
  PDG_TRY(stage_out<double>(ctx, sr));
  return st;
}

int pdg_solve_linear_problem(pdg_context *ctx, const pdg_solver_options *opt, double *x,
                             pdg_solver_result *res) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(check_opts(opt));
  if (!x || !res) return set_error(PDG_EINVAL, "null argument");
  std::memset(res, 0, sizeof(*res));
  PDG_TRY(ensure_stage(ctx));
  PDG_TRY(ensure_work(ctx, opt->mixed != 0));
  PDG_TRY(ensure_r0(ctx));
  Staged<double> sx;
  PDG_TRY(stage_in<double>(ctx, x, ctx->ndof, ctx->stage_a, true, &sx));
  double *r = ctx->stage_b, *z = ctx->w64[7];
  const long n = ctx->ndof;
  // r = R(x)   (linearproblem.hh:245-246)
  PDG_TRY(op_launch<double>(ctx, sx.dev, r, ctx->r0, 1.0, 0, 0, nullptr));
  double defect = 0.0;
  {
    const RedCtx rc = red_ctx(ctx);
    PDG_TRY(red_dot(ctx, rc, n, r, r, nullptr, nullptr, FIN_NORM, S_DOT, -1, false));
    double scal[S_COUNT];
    PDG_TRY(fetch_state(ctx, scal, nullptr));
    defect = scal[S_DOT];
  }
  // red = max(reduction, min_defect / defect)   (:260)
  pdg_solver_options o = *opt;
  if (defect > 0 && opt->min_defect / defect > o.reduction) o.reduction = opt->min_defect / defect;
  PDG_TRY(vec_fill<double>(ctx, n, z, 0.0));
  const int st = solve_correction(ctx, &o, z, r, 0, res);
  res->first_defect = defect;
  // x -= z   (:294)
  if (st == PDG_OK || st == PDG_ENOTCONVERGED) PDG_TRY(vec_axpy(ctx, n, -1.0, z, sx.dev));
  PDG_TRY(stage_out<double>(ctx, sx));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return st;
}

int pdg_adjoint_solve(pdg_context *ctx, const pdg_solver_options *opt, const double *rhs,
                      double *lambda, pdg_solver_result *res) {
  PDG_CHECK_CTX(ctx);
  PDG_TRY(check_opts(opt));
  if (!rhs || !lambda || !res) return set_error(PDG_EINVAL, "null argument");
  std::memset(res, 0, sizeof(*res));
  PDG_TRY(ensure_stage(ctx));
  PDG_TRY(ensure_work(ctx, opt->mixed != 0));
  Staged<double> sl;
  PDG_TRY(stage_in<double>(ctx, lambda, ctx->ndof, ctx->stage_a, true, &sl));
  double *r = ctx->stage_b;
  if (is_device_ptr(rhs))
    PDG_CUDA_TRY(cudaMemcpyAsync(r, rhs, sizeof(double) * ctx->ndof, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  else
    PDG_CUDA_TRY(cudaMemcpyAsync(r, rhs, sizeof(double) * ctx->ndof, cudaMemcpyHostToDevice,
                                 ctx->stream));
  // SIPG diffusion-reaction with a scalar K is symmetric (J^T = J); NIPG/IIPG,
  // upwind convection and general tensors (which need not be symmetric) are not
  const int transpose =
      (ctx->cfg.method == PDG_SIPG && !convection_on(ctx) && ctx->gen_A == 0) ? 0 : 1;
  pdg_solver_options o = *opt;
  if (transpose && (o.preconditioner & PDG_PREC_BLOCK_MASK) == PDG_PREC_BJ_FDM)
    o.preconditioner = (o.preconditioner & ~PDG_PREC_BLOCK_MASK) | PDG_PREC_BJ_DENSE;
  const int st = solve_correction(ctx, &o, sl.dev, r, transpose, res);
  PDG_TRY(stage_out<double>(ctx, sl));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return st;
}

int pdg_grad_logK(pdg_context *ctx, const double *u, const double *lambda, double *g) {
  PDG_CHECK_CTX(ctx);
  if (!u || !lambda || !g) return set_error(PDG_EINVAL, "null argument");
  if (ctx->cfg.weights != PDG_WEIGHTS_ON)
    return set_error(PDG_EUNSUPPORTED, "log-K gradient needs weightsOn");
  if (ctx->gen_A != 0)
    return set_error(PDG_EUNSUPPORTED, "log-K gradient needs A = K I per cell (no tensor)");
  PDG_TRY(ensure_r0(ctx));
  PDG_TRY(ensure_stage(ctx));
  Staged<double> su, sl;
  PDG_TRY(stage_in<double>(ctx, u, ctx->ndof, ctx->stage_a, true, &su));
  PDG_TRY(stage_in<double>(ctx, lambda, ctx->ndof, ctx->stage_b, true, &sl));
  double *gd = nullptr;
  const bool hg = !is_device_ptr(g);
  if (hg) {
    PDG_TRY(ensure_work(ctx, false));
    gd = ctx->w64[0];
  } else {
    gd = g;
  }
  PDG_TRY(launch_grad_logK(ctx, su.dev, sl.dev, gd));
  if (hg)
    PDG_CUDA_TRY(cudaMemcpyAsync(g, gd, sizeof(double) * ctx->ncell, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

int pdg_grad_source(pdg_context *ctx, const double *lambda, double *g) {
  PDG_CHECK_CTX(ctx);
  if (!lambda || !g) return set_error(PDG_EINVAL, "null argument");
  PDG_TRY(ensure_stage(ctx));
  Staged<double> sl;
  PDG_TRY(stage_in<double>(ctx, lambda, ctx->ndof, ctx->stage_b, true, &sl));
  double *gd = nullptr;
  const bool hg = !is_device_ptr(g);
  if (hg) {
    PDG_TRY(ensure_work(ctx, false));
    gd = ctx->w64[0];
  } else {
    gd = g;
  }
  PDG_TRY(launch_grad_source(ctx, sl.dev, gd));
  if (hg)
    PDG_CUDA_TRY(cudaMemcpyAsync(g, gd, sizeof(double) * ctx->ncell, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return PDG_OK;
}

}  // extern "C"
