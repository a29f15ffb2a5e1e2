// pdg_vec.cu -- deterministic reductions with device-side Krylov scalars,
// fused Krylov vector updates (dune-istl CGSolver / BiCGSTABSolver
// recurrences), and precision conversions for defect correction.
#include <cmath>
#include <cstdint>

#include "pdg_vec.cuh"

namespace pdg {

constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of two values, result valid in thread 0.
__device__ __forceinline__ void block_sum2(double &a, double &b) {
  __shared__ double sa[kRedThreads / 32], sb[kRedThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  if (lane == 0) { sa[w] = a; sb[w] = b; }
  __syncthreads();
  if (w == 0) {
    a = lane < (int)(blockDim.x >> 5) ? sa[lane] : 0.0;
    b = lane < (int)(blockDim.x >> 5) ? sb[lane] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
  }
}

// Shared tail of every reducing kernel: publish the block partial, let the
// last block add all partials in block order and run the finisher.
__device__ __forceinline__ void reduce_tail(const RedCtx &rc, double s0, double s1, int fin,
                                            int slot0, int slot1) {
  __shared__ bool is_last;
  block_sum2(s0, s1);
  if (threadIdx.x == 0) {
    rc.partials[2 * blockIdx.x] = s0;
    rc.partials[2 * blockIdx.x + 1] = s1;
    __threadfence();
    const int ticket = atomicAdd(&rc.flags[F_COUNTER], 1);
    is_last = ticket == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // fixed-order final sum: thread t adds partials t, t+blockDim, ... then tree
  double a = 0.0, b = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
    a += ((volatile double *)rc.partials)[2 * i];
    b += ((volatile double *)rc.partials)[2 * i + 1];
  }
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    run_finisher(rc, fin, slot0, slot1, a, b);
    rc.flags[F_COUNTER] = 0;
  }
}

// 16-byte vector of T and the sum of its lane products, in lane order
template <typename T> struct Vec16;
template <> struct Vec16<double> {
  using type = double2;
  static __device__ __forceinline__ double dot(double s, double2 x, double2 y) {
    s = fma(x.x, y.x, s);
    return fma(x.y, y.y, s);
  }
};
template <> struct Vec16<float> {
  using type = float4;
  static __device__ __forceinline__ float dot(float s, float4 x, float4 y) {
    s = fmaf(x.x, y.x, s);
    s = fmaf(x.y, y.y, s);
    s = fmaf(x.z, y.z, s);
    return fmaf(x.w, y.w, s);
  }
};

// <a, b> (and <c, d> when c is given).  With vec set (every pointer 16-byte
// aligned) the first n - n % W elements are read as 16-byte vectors, W per
// load, the rest one by one.  The order of the sums is fixed by n, the grid
// and vec, so results repeat bit for bit.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_dot(long n, const T *__restrict__ a, const T *__restrict__ b, const T *__restrict__ c,
          const T *__restrict__ d, RedCtx rc, int fin, int slot0, int slot1, int respect,
          int vec) {
  if (respect && rc.flags[F_STATE]) return;
  using V = typename Vec16<T>::type;
  constexpr int W = 16 / sizeof(T);
  T s0 = T(0), s1 = T(0);
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long stride = (long)gridDim.x * blockDim.x;
  long i0 = 0;
  if (vec) {
    const long nv = n / W;
    const V *av = reinterpret_cast<const V *>(a), *bv = reinterpret_cast<const V *>(b);
    if (c) {
      const V *cv = reinterpret_cast<const V *>(c), *dv = reinterpret_cast<const V *>(d);
#pragma unroll 4
      for (long j = tid; j < nv; j += stride) {
        s0 = Vec16<T>::dot(s0, av[j], bv[j]);
        s1 = Vec16<T>::dot(s1, cv[j], dv[j]);
      }
    } else {
#pragma unroll 4
      for (long j = tid; j < nv; j += stride) s0 = Vec16<T>::dot(s0, av[j], bv[j]);
    }
    i0 = nv * W;
  }
  for (long i = i0 + tid; i < n; i += stride) {
    s0 += a[i] * b[i];
    if (c) s1 += c[i] * d[i];
  }
  reduce_tail(rc, (double)s0, (double)s1, fin, slot0, slot1);
}

static unsigned red_grid(long n) {
  long g = (n + kRedThreads * 8 - 1) / (kRedThreads * 8);
  if (g < 1) g = 1;
  if (g > kRedBlocks) g = kRedBlocks;
  return (unsigned)g;
}

static int aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

template <typename T>
static int launch_dot(pdg_context *ctx, const RedCtx &rc, long n, const T *a, const T *b,
                      const T *c, const T *d, int fin, int slot0, int slot1, bool respect_flag) {
  const int vec = aligned16(a) && aligned16(b) && (!c || (aligned16(c) && aligned16(d)));
  k_dot<T><<<red_grid(n), kRedThreads, 0, ctx->stream>>>(n, a, b, c, d, rc, fin, slot0, slot1,
                                                          respect_flag, vec);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int red_dot(pdg_context *ctx, const RedCtx &rc, long n, const double *a, const double *b,
            const double *c, const double *d, int fin, int slot0, int slot1,
            bool respect_flag) {
  return launch_dot<double>(ctx, rc, n, a, b, c, d, fin, slot0, slot1, respect_flag);
}

int red_dot_f32(pdg_context *ctx, const RedCtx &rc, long n, const float *a, const float *b,
                const float *c, const float *d, int fin, int slot0, int slot1,
                bool respect_flag) {
  return launch_dot<float>(ctx, rc, n, a, b, c, d, fin, slot0, slot1, respect_flag);
}

// ---- fused Krylov updates ------------------------------------------------

// x += lambda p ; r -= lambda q ; |r|^2 -> defect check   (CGSolver)
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_cg_xr(long n, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
            const T *__restrict__ q, RedCtx rc) {
  if (rc.flags[F_STATE]) return;
  const T lambda = (T)rc.scal[S_ALPHA];
  T s = T(0);
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] += lambda * p[i];
    const T ri = r[i] - lambda * q[i];
    r[i] = ri;
    s += ri * ri;
  }
  reduce_tail(rc, (double)s, 0.0, FIN_DEF, -1, -1);
}

// p = z + beta p   (CGSolver: p *= beta; p += q)
template <typename T>
__global__ void k_cg_p(long n, T *__restrict__ p, const T *__restrict__ z, RedCtx rc) {
  if (rc.flags[F_STATE]) return;
  const T beta = (T)rc.scal[S_BETA];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = beta * p[i] + z[i];
}

// fused CG: x += lambda p ; p = z + beta p
template <typename T>
__global__ void k_cg_px(long n, T *__restrict__ x, T *__restrict__ p, const T *__restrict__ z,
                        RedCtx rc) {
  if (rc.flags[F_STATE]) return;
  const T lambda = (T)rc.scal[S_ALPHA], beta = (T)rc.scal[S_BETA];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T pi = p[i];
    x[i] += lambda * pi;
    p[i] = beta * pi + z[i];
  }
}

// x += lambda p for the iteration that stopped the fused CG (its px launch
// was skipped)
template <typename T>
__global__ void k_cg_xfin(long n, T *__restrict__ x, const T *__restrict__ p, RedCtx rc) {
  if (!rc.flags[F_XPEND]) return;
  const T lambda = (T)rc.scal[S_ALPHA];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    x[i] += lambda * p[i];
}

// BiCGSTABSolver: p = r (first half step) or p = beta (p - omega v) + r
template <typename T>
__global__ void k_bi_p(long n, T *__restrict__ p, const T *__restrict__ r,
                       const T *__restrict__ v, RedCtx rc, int first) {
  if (rc.flags[F_STATE]) return;
  const T beta = (T)rc.scal[S_BETA], omega = (T)rc.scal[S_OMEGA];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = first ? r[i] : beta * (p[i] - omega * v[i]) + r[i];
}

// x += a y ; r -= a v ; defect check   (a = alpha or omega)
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_bi_xr(long n, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ y,
            const T *__restrict__ v, RedCtx rc, int slot, int rho_update) {
  if (rc.flags[F_STATE]) return;
  const T aa = (T)rc.scal[slot];
  T s = T(0);
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] += aa * y[i];
    const T ri = r[i] - aa * v[i];
    r[i] = ri;
    s += ri * ri;
  }
  reduce_tail(rc, (double)s, 0.0, FIN_DEF, rho_update ? S_RHO : -1, -1);
}

__global__ void k_set_iter(RedCtx rc, double it) {
  if (rc.flags[F_STATE]) return;
  rc.scal[S_ITER] = it;
}
// the same, counting on the device (launches replayed from a graph)
__global__ void k_inc_iter(RedCtx rc, double step) {
  if (rc.flags[F_STATE]) return;
  rc.scal[S_ITER] += step;
}

static unsigned ew_grid(long n) {
  long g = (n + 255) / 256;
  if (g > 152 * 64) g = 152 * 64;
  return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
int cg_update_xr(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *r, const T *p,
                 const T *q) {
  k_cg_xr<T><<<red_grid(n), kRedThreads, 0, ctx->stream>>>(n, x, r, p, q, rc);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template <typename T>
int cg_update_p(pdg_context *ctx, const RedCtx &rc, long n, T *p, const T *z) {
  k_cg_p<T><<<ew_grid(n), 256, 0, ctx->stream>>>(n, p, z, rc);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
// FP32 vectors, 16-byte accesses (n4 = n / 4 float4 elements)
__global__ void k_cg_px4(long n4, float4 *__restrict__ x, float4 *__restrict__ p,
                         const float4 *__restrict__ z, RedCtx rc) {
  if (rc.flags[F_STATE]) return;
  const float lambda = (float)rc.scal[S_ALPHA], beta = (float)rc.scal[S_BETA];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    const float4 pi = p[i], zi = z[i];
    float4 xi = x[i];
    xi.x += lambda * pi.x; xi.y += lambda * pi.y; xi.z += lambda * pi.z; xi.w += lambda * pi.w;
    x[i] = xi;
    p[i] = make_float4(beta * pi.x + zi.x, beta * pi.y + zi.y, beta * pi.z + zi.z,
                       beta * pi.w + zi.w);
  }
}

template <typename T>
int cg_update_px(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *p, const T *z) {
  const bool vec = std::is_same<T, float>::value && n % 4 == 0 &&
                   ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(p) |
                     reinterpret_cast<uintptr_t>(z)) & 15) == 0;
  if (vec) {
    long g = (n / 4 + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_cg_px4<<<(unsigned)g, 256, 0, ctx->stream>>>(n / 4, reinterpret_cast<float4 *>(x),
                                                   reinterpret_cast<float4 *>(p),
                                                   reinterpret_cast<const float4 *>(z), rc);
  } else {
    k_cg_px<T><<<ew_grid(n), 256, 0, ctx->stream>>>(n, x, p, z, rc);
  }
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template <typename T>
int cg_finish_x(pdg_context *ctx, const RedCtx &rc, long n, T *x, const T *p) {
  k_cg_xfin<T><<<ew_grid(n), 256, 0, ctx->stream>>>(n, x, p, rc);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template <typename T>
int bi_update_p(pdg_context *ctx, const RedCtx &rc, long n, T *p, const T *r, const T *v,
                int first) {
  k_bi_p<T><<<ew_grid(n), 256, 0, ctx->stream>>>(n, p, r, v, rc, first);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template <typename T>
int bi_update_half(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *r, const T *y,
                   const T *v) {
  k_bi_xr<T><<<red_grid(n), kRedThreads, 0, ctx->stream>>>(n, x, r, y, v, rc, S_ALPHA, 0);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template <typename T>
int bi_update_full(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *r, const T *y,
                   const T *t) {
  k_bi_xr<T><<<red_grid(n), kRedThreads, 0, ctx->stream>>>(n, x, r, y, t, rc, S_OMEGA, 1);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
int set_iter(pdg_context *ctx, const RedCtx &rc, double it) {
  k_set_iter<<<1, 1, 0, ctx->stream>>>(rc, it);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
int inc_iter(pdg_context *ctx, const RedCtx &rc, double step) {
  k_inc_iter<<<1, 1, 0, ctx->stream>>>(rc, step);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

#define PDG_INST_UPD(T)                                                                     \
  template int cg_update_xr<T>(pdg_context *, const RedCtx &, long, T *, T *, const T *,    \
                               const T *);                                                  \
  template int cg_update_p<T>(pdg_context *, const RedCtx &, long, T *, const T *);         \
  template int cg_update_px<T>(pdg_context *, const RedCtx &, long, T *, T *, const T *);   \
  template int cg_finish_x<T>(pdg_context *, const RedCtx &, long, T *, const T *);         \
  template int bi_update_p<T>(pdg_context *, const RedCtx &, long, T *, const T *,          \
                              const T *, int);                                              \
  template int bi_update_half<T>(pdg_context *, const RedCtx &, long, T *, T *, const T *,  \
                                 const T *);                                                \
  template int bi_update_full<T>(pdg_context *, const RedCtx &, long, T *, T *, const T *,  \
                                 const T *);
PDG_INST_UPD(double)
PDG_INST_UPD(float)

// ---- plain vector kernels -------------------------------------------------

template <typename T>
__global__ void k_copy(long n, const T *__restrict__ s, T *__restrict__ d) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) d[i] = s[i];
}
template <typename T>
__global__ void k_fill(long n, T *__restrict__ d, T v) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) d[i] = v;
}
__global__ void k_axpy(long n, double a, const double *__restrict__ x, double *__restrict__ y) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] += a * x[i];
}
__global__ void k_to_f32_scaled(long n, const double *__restrict__ x, float *__restrict__ y,
                                const double *__restrict__ scal) {
  const double s = 1.0 / scal[S_SCALE];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = (float)(x[i] * s);
}
__global__ void k_add_f32_scaled(long n, const float *__restrict__ x, double *__restrict__ y,
                                 const double *__restrict__ scal, double sign) {
  const double s = sign * scal[S_SCALE];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] += s * (double)x[i];
}
__global__ void k_to_f32(long n, const double *__restrict__ x, float *__restrict__ y) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = (float)x[i];
}

template <typename T>
int vec_copy(pdg_context *ctx, long n, const T *src, T *dst) {
  k_copy<T><<<ew_grid(n), 256, 0, ctx->stream>>>(n, src, dst);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template <typename T>
int vec_fill(pdg_context *ctx, long n, T *dst, T v) {
  k_fill<T><<<ew_grid(n), 256, 0, ctx->stream>>>(n, dst, v);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
template int vec_copy<double>(pdg_context *, long, const double *, double *);
template int vec_copy<float>(pdg_context *, long, const float *, float *);
template int vec_fill<double>(pdg_context *, long, double *, double);
template int vec_fill<float>(pdg_context *, long, float *, float);

int vec_axpy(pdg_context *ctx, long n, double alpha, const double *x, double *y) {
  k_axpy<<<ew_grid(n), 256, 0, ctx->stream>>>(n, alpha, x, y);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
int vec_to_f32_scaled(pdg_context *ctx, long n, const double *x, float *y, const double *scal) {
  k_to_f32_scaled<<<ew_grid(n), 256, 0, ctx->stream>>>(n, x, y, scal);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
int vec_add_f32_scaled(pdg_context *ctx, long n, const float *x, double *y, const double *scal,
                       double sign) {
  k_add_f32_scaled<<<ew_grid(n), 256, 0, ctx->stream>>>(n, x, y, scal, sign);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
__global__ void k_to_f32_skip(long n, const double *__restrict__ x, float *__restrict__ y,
                              const int *__restrict__ skip) {
  if (skip && *skip) return;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = (float)x[i];
}
__global__ void k_from_f32_combine(long n, const float *__restrict__ s, double *__restrict__ y,
                                   const double *__restrict__ add, double alpha, int acc,
                                   const int *__restrict__ skip) {
  if (skip && *skip) return;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double v = alpha * (double)s[i];
    if (acc) v += y[i];
    if (add) v += add[i];
    y[i] = v;
  }
}
int vec_to_f32_skip(pdg_context *ctx, long n, const double *x, float *y, const int *skip) {
  k_to_f32_skip<<<ew_grid(n), 256, 0, ctx->stream>>>(n, x, y, skip);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}
int vec_from_f32_combine(pdg_context *ctx, long n, const float *s32, double *y, const double *add,
                         double alpha, int acc, const int *skip) {
  k_from_f32_combine<<<ew_grid(n), 256, 0, ctx->stream>>>(n, s32, y, add, alpha, acc, skip);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int vec_to_f32(pdg_context *ctx, long n, const double *x, float *y) {
  k_to_f32<<<ew_grid(n), 256, 0, ctx->stream>>>(n, x, y);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

}  // namespace pdg
