// pdg_nonlinear.cu -- the nonlinear volume term of
// NonlinearConvectionDiffusionDG (test/localoperator/
// nonlinearconvectiondiffusiondg.hh:28-307): ConvectionDiffusionDG plus
//   residual:        + int q(u) psi_i                       (alpha_volume, :93-131)
//   jacobian apply:  + int q'(u(x)) z psi_i  at the linearization point x
//                                                          (jacobian_apply_volume, :133-176)
// integrated with the same Gauss rule (order 2k, k+1 points per direction),
// q a polynomial q(u) = sum_m a_m u^m (degree <= 4; the reference's test
// problem uses q = mu u^2, matrix_free_nonlinear.cc:40-50).
//
// Setting the linearization point evaluates once per cell and Gauss point
// W_q = w_q |J| q'(u_x(x_q)); every Jacobian apply then adds the cell-local
// weighted mass  y_e += (B^T)^{(x)d} diag(W) B^{(x)d} z_e, B[q][a] = phi_a(xi_q),
// as three (two) sum-factorised passes forward and back.  The term is
// symmetric and cell-local, so it enters the transposed apply and the
// diagonal blocks unchanged.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pdg_internal.cuh"
#include "pdg_vec.cuh"

namespace pdg {

struct NlTab {
  double B[kMaxN1 * kMaxN1];   // B[q][a]
  double w[kMaxN1];
  double coef[5];
  int deg;
  double detJ;
};

__device__ __forceinline__ double q_eval(const NlTab &t, double u) {
  double s = 0.0;
  for (int m = t.deg; m >= 0; m--) s = s * u + t.coef[m];
  return s;
}
__device__ __forceinline__ double qprime_eval(const NlTab &t, double u) {
  double s = 0.0;
  for (int m = t.deg; m >= 1; m--) s = s * u + m * t.coef[m];
  return s;
}

// One cell per CTA, one thread per node / Gauss point (blockDim >= N^d):
// sum-factorised passes through shared memory.  `fwd`: values at the points
// from nodal coefficients (B); otherwise the transpose (B^T).
template <int D, int N>
__device__ __forceinline__ void tensor_pass(const NlTab &t, double *a, double *b, bool fwd) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  const int i = threadIdx.x;
#pragma unroll
  for (int dir = 0; dir < D; dir++) {
    const int stride = dir == 0 ? 1 : (dir == 1 ? N : N * N);
    if (i < NB) {
      const int c = (i / stride) % N;              // coordinate along dir
      const int base = i - c * stride;
      double s = 0.0;
      for (int j = 0; j < N; j++)
        s += (fwd ? t.B[c * N + j] : t.B[j * N + c]) * a[base + j * stride];
      b[i] = s;
    }
    __syncthreads();
    if (i < NB) a[i] = b[i];
    __syncthreads();
  }
}

__device__ __forceinline__ double point_weight(const NlTab &t, int D, int N, int q) {
  const int qx = q % N, qy = (q / N) % N, qz = D == 3 ? q / (N * N) : 0;
  double w = t.w[qx] * t.w[qy] * t.detJ;
  if (D == 3) w *= t.w[qz];
  return w;
}

// W_q = w_q |J| q'(u_x(x_q)) per cell (FP64 and an FP32 copy)
template <int D, int N>
__global__ void k_nl_weights(long ncell, const NlTab t, const double *__restrict__ x,
                             double *__restrict__ W64, float *__restrict__ W32) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  __shared__ double a[NB], b[NB];
  const long e = blockIdx.x;
  const int i = threadIdx.x;
  if (i < NB) a[i] = x[e * NB + i];
  __syncthreads();
  tensor_pass<D, N>(t, a, b, true);
  if (i < NB) {
    const double v = point_weight(t, D, N, i) * qprime_eval(t, a[i]);
    W64[e * NB + i] = v;
    W32[e * NB + i] = (float)v;
  }
}

// r_e += int q(u) psi   (residual part)
template <int D, int N>
__global__ void k_nl_residual(long ncell, const NlTab t, const double *__restrict__ x,
                              double *__restrict__ r) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  __shared__ double a[NB], b[NB];
  const long e = blockIdx.x;
  const int i = threadIdx.x;
  if (i < NB) a[i] = x[e * NB + i];
  __syncthreads();
  tensor_pass<D, N>(t, a, b, true);
  if (i < NB) a[i] = point_weight(t, D, N, i) * q_eval(t, a[i]);
  __syncthreads();
  tensor_pass<D, N>(t, a, b, false);
  if (i < NB) r[e * NB + i] += a[i];
}

// y_e += alpha (B^T)^d diag(W_e) B^d z_e on the listed cells (all if null).
// N^(d-1) threads per cell, each owning a line along the last direction in
// registers; the other directions go through shared memory.
template <typename T, int D, int N>
__global__ void __launch_bounds__(128)
    k_nl_apply(long ncell, const T *__restrict__ W, const T *__restrict__ Bt,
               const T *__restrict__ z, T *__restrict__ y, T alpha, const int *__restrict__ cells,
               int ncells, const int *__restrict__ skip) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  constexpr int TPC = D == 3 ? N * N : N;
  constexpr int CPB = 128 / TPC > 0 ? 128 / TPC : 1;
  if (skip && *skip) return;
  __shared__ T B[N * N];
  __shared__ T S[CPB][NB];
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) B[i] = Bt[i];
  const int cs = threadIdx.x / TPC, l = threadIdx.x - cs * TPC;
  const long li = (long)blockIdx.x * CPB + cs;
  const bool active = cs < CPB && (cells ? li < ncells : li < ncell);
  const long e = active ? (cells ? (long)cells[li] : li) : 0;
  T col[N];
  // own line along the last direction: offsets l + m * TPC
  if (cs < CPB) {
#pragma unroll
    for (int m = 0; m < N; m++) col[m] = active ? z[e * NB + m * TPC + l] : T(0);
  }
  __syncthreads();
  T *s = cs < CPB ? S[cs] : S[0];
  // forward along the last direction (registers)
  T a[N];
#pragma unroll
  for (int q = 0; q < N; q++) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < N; j++) acc += B[q * N + j] * col[j];
    a[q] = acc;
  }
  if (cs < CPB) {
#pragma unroll
    for (int q = 0; q < N; q++) s[q * TPC + l] = a[q];
  }
  __syncthreads();
  // forward along the other directions (shared memory), then scale by W
  if (D == 3) {
    const int tx = l % N, ty = l / N;
    T b[N];
#pragma unroll
    for (int q = 0; q < N; q++) {   // q: index along the last direction (z)
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < N; j++) acc += B[ty * N + j] * s[q * TPC + j * N + tx];
      b[q] = acc;
    }
    __syncthreads();
    if (cs < CPB) {
#pragma unroll
      for (int q = 0; q < N; q++) s[q * TPC + l] = b[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; q++) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < N; j++) acc += B[tx * N + j] * s[q * TPC + ty * N + j];
      a[q] = acc * (active ? W[e * NB + q * TPC + l] : T(0));
    }
    __syncthreads();
    if (cs < CPB) {
#pragma unroll
      for (int q = 0; q < N; q++) s[q * TPC + l] = a[q];
    }
    __syncthreads();
    // back along x, then y (shared memory)
#pragma unroll
    for (int q = 0; q < N; q++) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < N; j++) acc += B[j * N + tx] * s[q * TPC + ty * N + j];
      b[q] = acc;
    }
    __syncthreads();
    if (cs < CPB) {
#pragma unroll
      for (int q = 0; q < N; q++) s[q * TPC + l] = b[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; q++) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < N; j++) acc += B[j * N + ty] * s[q * TPC + j * N + tx];
      a[q] = acc;
    }
  } else {
    const int tx = l;
#pragma unroll
    for (int q = 0; q < N; q++) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < N; j++) acc += B[tx * N + j] * s[q * TPC + j];
      a[q] = acc * (active ? W[e * NB + q * TPC + l] : T(0));
    }
    __syncthreads();
    if (cs < CPB) {
#pragma unroll
      for (int q = 0; q < N; q++) s[q * TPC + l] = a[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; q++) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < N; j++) acc += B[j * N + tx] * s[q * TPC + j];
      a[q] = acc;
    }
  }
  // back along the last direction (registers) and accumulate
  if (active) {
#pragma unroll
    for (int m = 0; m < N; m++) {
      T acc = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) acc += B[q * N + m] * a[q];
      y[e * NB + m * TPC + l] += alpha * acc;
    }
  }
}

static NlTab nl_tab(const pdg_context *ctx) {
  NlTab t{};
  const RhsTables r = make_rhs_tables(ctx);
  const int N = ctx->N;
  for (int i = 0; i < N * N; i++) t.B[i] = r.B[i];
  for (int i = 0; i < N; i++) t.w[i] = r.w[i];
  for (int m = 0; m < 5; m++) t.coef[m] = ctx->nl_coef[m];
  t.deg = ctx->nl_deg;
  t.detJ = 1.0;
  for (int j = 0; j < ctx->dim; j++) t.detJ *= ctx->h[j];
  return t;
}

template <int D, int N>
static int nl_weights_dn(pdg_context *ctx, const double *x) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  const NlTab t = nl_tab(ctx);
  k_nl_weights<D, N><<<(unsigned)ctx->ncell, ((NB + 31) / 32) * 32, 0, ctx->stream>>>(
      ctx->ncell, t, x, ctx->nlW64, ctx->nlW32);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <int D, int N>
static int nl_residual_dn(pdg_context *ctx, const double *x, double *r) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  const NlTab t = nl_tab(ctx);
  k_nl_residual<D, N><<<(unsigned)ctx->ncell, ((NB + 31) / 32) * 32, 0, ctx->stream>>>(
      ctx->ncell, t, x, r);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

#define PDG_DN_SWITCH(FN, ...)                                        \
  switch (ctx->dim * 10 + ctx->k) {                                   \
    case 21: return FN<2, 2>(__VA_ARGS__);                            \
    case 22: return FN<2, 3>(__VA_ARGS__);                            \
    case 23: return FN<2, 4>(__VA_ARGS__);                            \
    case 24: return FN<2, 5>(__VA_ARGS__);                            \
    case 31: return FN<3, 2>(__VA_ARGS__);                            \
    case 32: return FN<3, 3>(__VA_ARGS__);                            \
    case 33: return FN<3, 4>(__VA_ARGS__);                            \
    case 34: return FN<3, 5>(__VA_ARGS__);                            \
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in"); \
  }

static int nl_weights_dispatch(pdg_context *ctx, const double *x) {
  PDG_DN_SWITCH(nl_weights_dn, ctx, x)
}

int nl_set_point(pdg_context *ctx, const double *x) {
  if (ctx->nl_deg <= 0) return PDG_OK;
  if (!ctx->nlW64) PDG_CUDA_TRY(cudaMalloc(&ctx->nlW64, sizeof(double) * ctx->ndof));
  if (!ctx->nlW32) PDG_CUDA_TRY(cudaMalloc(&ctx->nlW32, sizeof(float) * ctx->ndof));
  if (!ctx->nlB32) {
    const RhsTables r = make_rhs_tables(ctx);
    float b32[kMaxN1 * kMaxN1];
    for (int i = 0; i < ctx->N * ctx->N; i++) b32[i] = (float)r.B[i];
    PDG_CUDA_TRY(cudaMalloc(&ctx->nlB32, sizeof(float) * ctx->N * ctx->N));
    PDG_CUDA_TRY(cudaMalloc(&ctx->nlB64, sizeof(double) * ctx->N * ctx->N));
    PDG_CUDA_TRY(cudaMemcpy(ctx->nlB32, b32, sizeof(float) * ctx->N * ctx->N,
                            cudaMemcpyHostToDevice));
    PDG_CUDA_TRY(cudaMemcpy(ctx->nlB64, r.B, sizeof(double) * ctx->N * ctx->N,
                            cudaMemcpyHostToDevice));
  }
  PDG_TRY(nl_weights_dispatch(ctx, x));
  ctx->nl_point = 1;
  return PDG_OK;
}

int nl_residual(pdg_context *ctx, const double *x, double *r) {
  if (ctx->nl_deg <= 0) return PDG_OK;
  PDG_DN_SWITCH(nl_residual_dn, ctx, x, r)
}

template <typename T, int D, int N>
static int weighted_apply_dn(pdg_context *ctx, const T *W, const T *B, const ApplyArgs<T> &a) {
  constexpr int TPC = D == 3 ? N * N : N;
  constexpr int CPB = 128 / TPC > 0 ? 128 / TPC : 1;
  const long work = a.cells ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  k_nl_apply<T, D, N><<<(unsigned)((work + CPB - 1) / CPB), 128, 0, ctx->stream>>>(
      ctx->ncell, W, B, a.x, a.y, a.alpha, a.cells, a.ncells, a.skip);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// y += alpha (X^T)^d diag(W) X^d x per cell, X an N x N table on the device
template <typename T>
int weighted_apply(pdg_context *ctx, const T *W, const T *X, const ApplyArgs<T> &a) {
  switch (ctx->dim * 10 + ctx->k) {
    case 21: return weighted_apply_dn<T, 2, 2>(ctx, W, X, a);
    case 22: return weighted_apply_dn<T, 2, 3>(ctx, W, X, a);
    case 23: return weighted_apply_dn<T, 2, 4>(ctx, W, X, a);
    case 24: return weighted_apply_dn<T, 2, 5>(ctx, W, X, a);
    case 31: return weighted_apply_dn<T, 3, 2>(ctx, W, X, a);
    case 32: return weighted_apply_dn<T, 3, 3>(ctx, W, X, a);
    case 33: return weighted_apply_dn<T, 3, 4>(ctx, W, X, a);
    case 34: return weighted_apply_dn<T, 3, 5>(ctx, W, X, a);
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
}
template int weighted_apply<double>(pdg_context *, const double *, const double *,
                                    const ApplyArgs<double> &);

// The DG mass matrix (the temporal operator of one-step methods, int u psi)
// and its inverse per cell, both through the weighted tensor kernel:
//   M = (B^T)^d diag(w |J|) B^d,   M^{-1} = (B^{-1})^d diag(1/(w |J|)) (B^{-T})^d,
// B[q][a] = phi_a(xi_q) (square, invertible: k+1 Gauss points, k+1 nodes).
static int ensure_mass(pdg_context *ctx) {
  if (ctx->massW) return PDG_OK;
  const RhsTables r = make_rhs_tables(ctx);
  const int N = ctx->N, D = ctx->dim;
  const int NB = D == 3 ? N * N * N : N * N;
  double detJ = 1.0;
  for (int j = 0; j < D; j++) detJ *= ctx->h[j];
  std::vector<double> w(NB), wi(NB);
  for (int q = 0; q < NB; q++) {
    const int qx = q % N, qy = (q / N) % N, qz = D == 3 ? q / (N * N) : 0;
    w[q] = r.w[qx] * r.w[qy] * (D == 3 ? r.w[qz] : 1.0) * detJ;
    wi[q] = 1.0 / w[q];
  }
  // B^{-T}: invert B (Gauss-Jordan with partial pivoting, N <= 5), transpose
  double a[kMaxN1][2 * kMaxN1];
  for (int i = 0; i < N; i++)
    for (int j = 0; j < 2 * N; j++) a[i][j] = j < N ? r.B[i * N + j] : (j - N == i ? 1.0 : 0.0);
  for (int c = 0; c < N; c++) {
    int p = c;
    for (int i = c + 1; i < N; i++)
      if (std::fabs(a[i][c]) > std::fabs(a[p][c])) p = i;
    for (int j = 0; j < 2 * N; j++) std::swap(a[c][j], a[p][j]);
    const double inv = 1.0 / a[c][c];
    for (int j = 0; j < 2 * N; j++) a[c][j] *= inv;
    for (int i = 0; i < N; i++)
      if (i != c) {
        const double f = a[i][c];
        for (int j = 0; j < 2 * N; j++) a[i][j] -= f * a[c][j];
      }
  }
  std::vector<double> BinvT(N * N), Bt(N * N);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      BinvT[i * N + j] = a[j][N + i];   // (B^{-1})^T
      Bt[i * N + j] = r.B[i * N + j];
    }
  std::vector<double> W(ctx->ndof), Wi(ctx->ndof);
  for (long e = 0; e < ctx->ncell; e++)
    for (int q = 0; q < NB; q++) {
      W[e * NB + q] = w[q];
      Wi[e * NB + q] = wi[q];
    }
  PDG_CUDA_TRY(cudaMalloc(&ctx->massW, sizeof(double) * ctx->ndof));
  PDG_CUDA_TRY(cudaMalloc(&ctx->massWi, sizeof(double) * ctx->ndof));
  PDG_CUDA_TRY(cudaMalloc(&ctx->massB, sizeof(double) * N * N));
  PDG_CUDA_TRY(cudaMalloc(&ctx->massBiT, sizeof(double) * N * N));
  PDG_CUDA_TRY(cudaMemcpy(ctx->massW, W.data(), sizeof(double) * ctx->ndof, cudaMemcpyHostToDevice));
  PDG_CUDA_TRY(cudaMemcpy(ctx->massWi, Wi.data(), sizeof(double) * ctx->ndof, cudaMemcpyHostToDevice));
  PDG_CUDA_TRY(cudaMemcpy(ctx->massB, Bt.data(), sizeof(double) * N * N, cudaMemcpyHostToDevice));
  PDG_CUDA_TRY(cudaMemcpy(ctx->massBiT, BinvT.data(), sizeof(double) * N * N, cudaMemcpyHostToDevice));
  return PDG_OK;
}

// y = (accumulate ? y : 0) + alpha M x   (M^{-1} with `inverse`)
int mass_apply(pdg_context *ctx, const double *x, double *y, double alpha, int accumulate,
               int inverse) {
  PDG_TRY(ensure_mass(ctx));
  if (ctx->basis == PDG_BASIS_LEGENDRE) {
    // M_L = T^T M T and M_L^{-1} = T^{-1} M^{-1} T^{-T} (pdg_basis.cu)
    double *w0 = ctx->legw64[0], *w1 = ctx->legw64[1];
    PDG_TRY(basis_change<double>(ctx, inverse, inverse, x, w0, 1.0, 0, nullptr, nullptr));
    PDG_TRY(vec_fill<double>(ctx, ctx->ndof, w1, 0.0));
    ApplyArgs<double> a{w0, w1, nullptr, 1.0, 1, 0, 0, nullptr};
    PDG_TRY(inverse ? weighted_apply<double>(ctx, ctx->massWi, ctx->massBiT, a)
                    : weighted_apply<double>(ctx, ctx->massW, ctx->massB, a));
    return basis_change<double>(ctx, inverse, !inverse, w1, y, alpha, accumulate, nullptr,
                                nullptr);
  }
  if (!accumulate) PDG_TRY(vec_fill<double>(ctx, ctx->ndof, y, 0.0));
  ApplyArgs<double> a{x, y, nullptr, alpha, 1, 0, 0, nullptr};
  return inverse ? weighted_apply<double>(ctx, ctx->massWi, ctx->massBiT, a)
                 : weighted_apply<double>(ctx, ctx->massW, ctx->massB, a);
}

template <typename T>
int nl_apply(pdg_context *ctx, const ApplyArgs<T> &a) {
  if (ctx->nl_deg <= 0 || !ctx->nl_point || ctx->nl_off) return PDG_OK;
  const bool dbl = std::is_same<T, double>::value;
  const T *W = dbl ? (const T *)ctx->nlW64 : (const T *)ctx->nlW32;
  const T *B = dbl ? (const T *)ctx->nlB64 : (const T *)ctx->nlB32;
  return weighted_apply<T>(ctx, W, B, a);
}
template int weighted_apply<float>(pdg_context *, const float *, const float *,
                                   const ApplyArgs<float> &);

template int nl_apply<double>(pdg_context *, const ApplyArgs<double> &);
template int nl_apply<float>(pdg_context *, const ApplyArgs<float> &);

}  // namespace pdg
