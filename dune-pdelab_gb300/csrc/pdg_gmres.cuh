// pdg_gmres.cuh -- restarted, right-preconditioned GMRES(m) on the device,
// with a fixed preconditioner (cell-block Jacobi) or a flexible one (FGMRES,
// Saad 1993: the preconditioner may change from step to step and the
// preconditioned directions Z_j are kept).
//
// No reference counterpart (PDELab's matrix-free backends use dune-istl's
// CG/BiCGStab).  Used
//  * as an outer FP64 method on request (PDG_GMRES), and
//  * as the FP64 outer loop of the mixed-precision solve for non-symmetric
//    operators, whose variable preconditioner is a short inner Krylov solve
//    with the FP32 operator and FP32 block Jacobi: a Krylov-accelerated
//    defect correction (flexible GMRES-based iterative refinement).  Plain
//    defect correction with an FP32 BiCGStab inner solve diverges on the
//    48^3 Q4 convection problem (the FP32 operator agrees with the FP64 one
//    to 2e-7, but BiCGStab's intermediate residual growth amplifies that
//    perturbation); the outer FGMRES minimises the true FP64 residual over
//    all inner corrections, so a poor inner solve only slows convergence.
//
// Arnoldi with classical Gram-Schmidt applied twice (CGS2: one fused
// multi-dot and one fused multi-axpy per pass); Givens rotations and the
// small least-squares problem on the host (one device-to-host copy per
// Arnoldi step).  Dot products accumulate per thread in T and across threads
// in FP64 in a fixed order (deterministic).
//
// Included by pdg_abi.cu only.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pdg_internal.cuh"
#include "pdg_vec.cuh"

namespace pdg {

constexpr int kGmThreads = 256;
constexpr int kGmMaxBlocks = 512;
constexpr int kGmMaxM = 64;

// partial[blk * k + i] = sum over this block's elements of w . V_i
template <typename T, int KMAX>
__global__ void __launch_bounds__(kGmThreads)
    k_multidot(long n, const T *__restrict__ w, const T *__restrict__ V, long ld, int k,
               double *__restrict__ partial) {
  T acc[KMAX];
#pragma unroll
  for (int i = 0; i < KMAX; i++) acc[i] = T(0);
  const long stride = (long)gridDim.x * blockDim.x;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    const T we = w[e];
#pragma unroll
    for (int i = 0; i < KMAX; i++)
      if (i < k) acc[i] += we * V[i * ld + e];
  }
  __shared__ double sm[kGmThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = 0; i < k; i++) {
    double v = (double)acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int j = 0; j < (int)(blockDim.x >> 5); j++) s += sm[j];
      partial[blockIdx.x * k + i] = s;
    }
    __syncthreads();
  }
}

// out[i] = sum_blk partial[blk * k + i]  (fixed order)
__global__ void k_multidot_sum(int nblk, int k, const double *__restrict__ partial,
                               double *__restrict__ out) {
  const int i = threadIdx.x;
  if (i >= k) return;
  double s = 0.0;
  for (int b = 0; b < nblk; b++) s += partial[b * k + i];
  out[i] = s;
}

// w += sign * sum_i c[i] V_i   (coefficients on the device)
template <typename T>
__global__ void k_multiaxpy(long n, T *__restrict__ w, const T *__restrict__ V, long ld, int k,
                            const double *__restrict__ c, double sign) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double s = 0.0;
    for (int i = 0; i < k; i++) s += c[i] * (double)V[i * ld + e];
    w[e] = (T)((double)w[e] + sign * s);
  }
}

// v = w / sqrt(nrm2[0])
template <typename T>
__global__ void k_scale_by(long n, T *__restrict__ v, const T *__restrict__ w,
                           const double *__restrict__ nrm2) {
  const double s = 1.0 / sqrt(*nrm2);
  const long stride = (long)gridDim.x * blockDim.x;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    v[e] = (T)((double)w[e] * s);
}

inline unsigned gm_grid(long n) {
  long g = (n + kGmThreads * 4 - 1) / (kGmThreads * 4);
  if (g > kGmMaxBlocks) g = kGmMaxBlocks;
  return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
int gm_multidot(pdg_context *ctx, long n, const T *w, const T *V, long ld, int k, double *out) {
  const unsigned g = gm_grid(n);
  if (k <= 8)
    k_multidot<T, 8><<<g, kGmThreads, 0, ctx->stream>>>(n, w, V, ld, k, ctx->gm_partial);
  else if (k <= 16)
    k_multidot<T, 16><<<g, kGmThreads, 0, ctx->stream>>>(n, w, V, ld, k, ctx->gm_partial);
  else if (k <= 32)
    k_multidot<T, 32><<<g, kGmThreads, 0, ctx->stream>>>(n, w, V, ld, k, ctx->gm_partial);
  else
    k_multidot<T, 64><<<g, kGmThreads, 0, ctx->stream>>>(n, w, V, ld, k, ctx->gm_partial);
  k_multidot_sum<<<1, 64, 0, ctx->stream>>>((int)g, k, ctx->gm_partial, out);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

struct GmresOut {
  int iterations = 0;
  int state = 0;   // 0 maxit, 1 converged, 2 non-finite
  double def0 = 0.0, def = 0.0;
};

// Solve A x = b from the initial guess x.  Op(const T* in, T* out): out = A in.
// Prec(const T* in, T* out): out = M^{-1} in.  With `flexible` the directions
// Z_j = M_j^{-1} v_j are stored (FGMRES) and the preconditioner may differ
// between steps.  b is overwritten by the final residual.
//
// zt, q: two work vectors of length ndof; Vbuf / Vm: the basis storage and its
// capacity in vectors (grown on demand).  The preconditioner may use any
// storage but these (it runs only between uses of zt / q that do not span it).
template <typename T, typename Op, typename Prec>
int gmres_core(pdg_context *ctx, T *x, T *b, T *zt, T *q, void *&Vbuf, int &Vm, double reduction,
               int maxit, int m, bool flexible, bool verbose, Op &&op, Prec &&prec,
               GmresOut *out) {
  if (m < 1 || m > kGmMaxM) return set_error(PDG_EINVAL, "GMRES restart length must be 1..64");
  const long n = ctx->ndof;
  const int nvec = flexible ? 2 * m + 1 : m + 1;
  if (Vbuf && Vm < nvec) {
    cudaFree(Vbuf);
    Vbuf = nullptr;
  }
  if (!Vbuf) {
    PDG_CUDA_TRY(cudaMalloc(&Vbuf, sizeof(T) * (size_t)nvec * n));
    Vm = nvec;
  }
  if (!ctx->gm_partial)
    PDG_CUDA_TRY(cudaMalloc(&ctx->gm_partial, sizeof(double) * kGmMaxBlocks * (kGmMaxM + 1)));
  if (!ctx->gm_coef) PDG_CUDA_TRY(cudaMalloc(&ctx->gm_coef, sizeof(double) * 4 * (kGmMaxM + 8)));
  T *V = static_cast<T *>(Vbuf);
  T *Z = flexible ? V + (size_t)(m + 1) * n : nullptr;
  T *r = b;
  double *h1 = ctx->gm_coef;          // first CGS pass
  double *h2 = h1 + (kGmMaxM + 1);    // second CGS pass
  double *nd = h2 + (kGmMaxM + 1);    // |w|^2
  double *yd = nd + 8;                // least-squares solution
  const unsigned eg = gm_grid(n);
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hcol(m + 2);
  double hbuf[2 * (kGmMaxM + 1) + 1];

  auto norm2 = [&](const T *v, double *dst) -> int { return gm_multidot<T>(ctx, n, v, v, n, 1, dst); };
  auto fetch1 = [&](double *dst) -> int {
    PDG_CUDA_TRY(cudaMemcpyAsync(dst, nd, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PDG_OK;
  };
  // r = b - A x
  PDG_TRY(op(x, q));
  {
    const double minus1 = -1.0;
    PDG_CUDA_TRY(cudaMemcpyAsync(yd, &minus1, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    k_multiaxpy<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, r, q, n, 1, yd, 1.0);
  }
  double beta2 = 0.0;
  PDG_TRY(norm2(r, nd));
  PDG_TRY(fetch1(&beta2));
  double beta = std::sqrt(beta2);
  const double def0 = beta;
  out->def0 = def0;
  out->state = 0;
  int total = 0;
  if (!std::isfinite(beta)) { out->state = 2; out->def = beta; return PDG_OK; }
  if (beta < def0 * reduction || beta < 1e-30) { out->state = 1; out->def = beta; return PDG_OK; }
  double resid = beta;
  while (total < maxit) {
    k_scale_by<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, V, r, nd);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && total < maxit; j++) {
      T *vj = V + (size_t)j * n, *vn = V + (size_t)(j + 1) * n;
      T *zj = flexible ? Z + (size_t)j * n : zt;
      PDG_TRY(prec(vj, zj));
      PDG_TRY(op(zj, vn));
      for (int pass = 0; pass < 2; pass++) {
        double *hp = pass == 0 ? h1 : h2;
        PDG_TRY(gm_multidot<T>(ctx, n, vn, V, n, j + 1, hp));
        k_multiaxpy<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, vn, V, n, j + 1, hp, -1.0);
      }
      PDG_TRY(norm2(vn, nd));
      k_scale_by<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, vn, vn, nd);
      PDG_CUDA_TRY(cudaMemcpyAsync(hbuf, h1, sizeof(double) * (2 * (kGmMaxM + 1) + 1),
                                   cudaMemcpyDeviceToHost, ctx->stream));
      PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
      total++;
      for (int i = 0; i <= j; i++) hcol[i] = hbuf[i] + hbuf[(kGmMaxM + 1) + i];
      hcol[j + 1] = std::sqrt(hbuf[2 * (kGmMaxM + 1)]);
      for (int i = 0; i < j; i++) {
        const double t0 = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
        hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
        hcol[i] = t0;
      }
      const double den = std::hypot(hcol[j], hcol[j + 1]);
      cs[j] = den > 0 ? hcol[j] / den : 1.0;
      sn[j] = den > 0 ? hcol[j + 1] / den : 0.0;
      hcol[j] = den;
      hcol[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = hcol[i];
      resid = std::fabs(g[j + 1]);
      if (verbose)
        std::fprintf(stderr, "pdg %sgmres: step %d residual %.3e (reduction %.3e)\n",
                     flexible ? "f" : "", total, resid, resid / def0);
      if (!std::isfinite(resid)) { out->state = 2; break; }
      if (resid < def0 * reduction || resid < 1e-30) { j++; break; }
    }
    if (out->state == 2) break;
    const int k = j;
    std::vector<double> y(k);
    for (int i = k - 1; i >= 0; i--) {
      double s = g[i];
      for (int l = i + 1; l < k; l++) s -= H[(size_t)i * m + l] * y[l];
      y[i] = H[(size_t)i * m + i] != 0.0 ? s / H[(size_t)i * m + i] : 0.0;
    }
    PDG_CUDA_TRY(cudaMemcpyAsync(yd, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice,
                                 ctx->stream));
    // correction: flexible x += Z y ; fixed x += M^{-1} V y
    T *corr = zt;
    if (flexible) {
      PDG_TRY(vec_fill<T>(ctx, n, corr, T(0)));
      k_multiaxpy<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, corr, Z, n, k, yd, 1.0);
    } else {
      PDG_TRY(vec_fill<T>(ctx, n, q, T(0)));
      k_multiaxpy<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, q, V, n, k, yd, 1.0);
      PDG_TRY(prec(q, corr));
    }
    {
      const double one = 1.0;
      PDG_CUDA_TRY(cudaMemcpyAsync(yd, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      k_multiaxpy<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, x, corr, n, 1, yd, 1.0);
      // r_new = r_cycle - A corr
      PDG_TRY(op(corr, q));
      const double minus1 = -1.0;
      PDG_CUDA_TRY(cudaMemcpyAsync(yd, &minus1, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      k_multiaxpy<T><<<eg, kGmThreads, 0, ctx->stream>>>(n, r, q, n, 1, yd, 1.0);
    }
    PDG_TRY(norm2(r, nd));
    PDG_TRY(fetch1(&beta2));
    beta = std::sqrt(beta2);
    resid = beta;
    if (!std::isfinite(beta)) { out->state = 2; break; }
    if (beta < def0 * reduction || beta < 1e-30) { out->state = 1; break; }
  }
  out->iterations = total;
  out->def = resid;
  return PDG_OK;
}

}  // namespace pdg
