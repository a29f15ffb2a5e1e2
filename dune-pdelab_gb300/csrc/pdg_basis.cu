// pdg_basis.cu -- the modal (Legendre) QkDG basis on top of the nodal kernels.
//
// DGLegendreLocalBasis (finiteelement/qkdglegendre.hh:236-328) spans the same
// space Q_k as the equidistant Lagrange basis the kernels work in, so with
// the 1D change of basis T[j][i] = P_i(j/k) (Legendre polynomial i at node j)
// the Legendre coefficients c of a function and its nodal values u are
// related per cell by u = (T (x) T (x) T) c, and every local form of the
// operator transforms by congruence:
//   residual / jacobian_apply:  r_L = (T (x) T (x) T)^T r_nodal(u),
//   diagonal blocks:            D_L = T^T D_nodal T  (tensorised),
//   inverse blocks:             D_L^{-1} = T^{-1} D_nodal^{-1} T^{-T}.
// Gauss order 2k integrates all these products exactly in either basis, so
// the Legendre operator of the reference and the transformed nodal one agree
// to rounding.  The change of basis is one HBM-bound kernel per vector.
#include "pdg_internal.cuh"

namespace pdg {

// out_e = acc ? out_e : 0  +  alpha (M (x) M [(x) M]) in_e  +  add_e  per cell,
// M = mat or mat^T (N x N, row-major).  One thread per local DOF, CPB cells
// per CTA staged in shared memory, one contraction per direction.
template <typename T, int D, int N>
__global__ void __launch_bounds__(128)
    k_basis_change(long ncell, const T *__restrict__ mat, int transpose,
                   const T *__restrict__ in, T *__restrict__ out, T alpha, int acc,
                   const T *__restrict__ add, const int *__restrict__ skip) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  constexpr int CPB = 128 / NB > 0 ? 128 / NB : 1;
  __shared__ T M[N * N];
  __shared__ T s0[CPB * NB], s1[CPB * NB];
  if (skip && *skip) return;
  const int t = threadIdx.x, cs = t / NB, l = t - cs * NB;
  if (t < N * N) {
    const int a = t / N, q = t - a * N;
    M[t] = transpose ? mat[q * N + a] : mat[a * N + q];
  }
  const long e = (long)blockIdx.x * CPB + cs;
  const bool active = cs < CPB && e < ncell;
  if (active) s0[cs * NB + l] = in[e * NB + l];
  __syncthreads();
  const int x = l % N, y = (l / N) % N, z = l / (N * N);
  T r = T(0);
  if (cs < CPB) {
    const T *c0 = s0 + cs * NB;
    T *c1 = s1 + cs * NB;
#pragma unroll
    for (int q = 0; q < N; q++) r += M[x * N + q] * c0[l - x + q];
    c1[l] = r;
  }
  __syncthreads();
  if (cs < CPB) {
    const T *c1 = s1 + cs * NB;
    r = T(0);
#pragma unroll
    for (int q = 0; q < N; q++) r += M[y * N + q] * c1[l + (q - y) * N];
  }
  if (D == 3) {
    __syncthreads();
    if (cs < CPB) s0[cs * NB + l] = r;
    __syncthreads();
    if (cs < CPB) {
      const T *c0 = s0 + cs * NB;
      r = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) r += M[z * N + q] * c0[l + (q - z) * N * N];
    }
  }
  if (active) {
    const long i = e * NB + l;
    T v = alpha * r;
    if (acc) v += out[i];
    if (add) v += add[i];
    out[i] = v;
  }
}

template <typename T, int D, int N>
static int basis_launch(pdg_context *ctx, const T *mat, int transpose, const T *in, T *out,
                        T alpha, int acc, const T *add, const int *skip) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  constexpr int CPB = 128 / NB > 0 ? 128 / NB : 1;
  const unsigned blocks = (unsigned)((ctx->ncell + CPB - 1) / CPB);
  k_basis_change<T, D, N><<<blocks, CPB * NB, 0, ctx->stream>>>(ctx->ncell, mat, transpose, in,
                                                                out, alpha, acc, add, skip);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <typename T>
int basis_change(pdg_context *ctx, int which, int transpose, const T *in, T *out, T alpha,
                 int acc, const T *add, const int *skip) {
  const bool dbl = std::is_same<T, double>::value;
  const T *mat = (dbl ? (const T *)ctx->leg64 : (const T *)ctx->leg32) +
                 (which ? ctx->N * ctx->N : 0);
  switch (ctx->dim * 10 + ctx->N) {
    case 22: return basis_launch<T, 2, 2>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 23: return basis_launch<T, 2, 3>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 24: return basis_launch<T, 2, 4>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 25: return basis_launch<T, 2, 5>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 32: return basis_launch<T, 3, 2>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 33: return basis_launch<T, 3, 3>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 34: return basis_launch<T, 3, 4>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    case 35: return basis_launch<T, 3, 5>(ctx, mat, transpose, in, out, alpha, acc, add, skip);
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
}

template int basis_change<double>(pdg_context *, int, int, const double *, double *, double,
                                  int, const double *, const int *);
template int basis_change<float>(pdg_context *, int, int, const float *, float *, float, int,
                                 const float *, const int *);

}  // namespace pdg
