// pdg_vec.cuh -- device-resident Krylov scalars and fused vector kernels.
//
// The Krylov recurrences of dune-istl's CGSolver / BiCGSTABSolver keep a
// handful of scalars (rho, alpha, omega, defect ...).  Here they live in a
// small device array so that one iteration is a fixed sequence of kernel
// launches with no host round trip; the convergence test
// (IterativeSolver::Iteration::step: def < def0 * reduction or def < 1e-30,
// non-finite defects abort) is evaluated on the device and raises a flag
// that every later kernel of the solve checks before doing any work.
//
// Dot products are deterministic: each block writes one partial sum (fixed
// grid-stride order, fixed tree), the last block to finish adds the
// partials in block order and runs the "finisher" for the scalars.
#pragma once

#include "pdg_internal.cuh"

namespace pdg {

// scalar slots
enum Slot {
  S_DEF0 = 0,     // first defect
  S_DEF = 1,      // current defect (two-norm)
  S_RED = 2,      // requested reduction
  S_RHO = 3,      // CG rholast / BiCGStab rho
  S_RHONEW = 4,   // BiCGStab rho_new
  S_ALPHA = 5,    // CG lambda / BiCGStab alpha
  S_BETA = 6,
  S_OMEGA = 7,
  S_H = 8,        // BiCGStab h = <rt, v>
  S_TR = 9,       // BiCGStab <t, r>
  S_TT = 10,      // BiCGStab <t, t>
  S_ITER = 11,    // iteration count (as double; BiCGStab counts halves)
  S_DOT = 12,     // generic dot result
  S_DOT2 = 13,
  S_SCALE = 14,   // mixed precision: scaling of the inner right-hand side
  S_GUARD = 15,   // relative breakdown threshold (0: dune-istl's absolute tests only)
  S_COUNT = 16
};

// flag words (int): [0] state (0 running, 1 converged, 2 non-finite,
// 3 breakdown), [1] reduction counter (last-block detection), [2] the CG
// x update of the stopping iteration is still to be applied, [3] a kernel's
// TMA staging did not complete within its poll limit (sticky)
enum { F_STATE = 0, F_COUNTER = 1, F_XPEND = 2, F_TMA = 3, F_COUNT = 4 };

enum Finisher {
  FIN_STORE = 0,        // scal[slot0] = d0 ; scal[slot1] = d1
  FIN_DEF0 = 1,         // def0 = def = sqrt(d0); iteration 0 check
  FIN_DEF = 2,          // def = sqrt(d0); convergence check at scal[S_ITER]
  FIN_CG_LAMBDA = 3,    // lambda = rholast / d0
  FIN_CG_BETA = 4,      // beta = d0 / rholast; rholast = d0
  FIN_BI_RHONEW = 5,    // rho_new = d0; breakdown checks
  FIN_BI_ALPHA = 6,     // h = d0; alpha = rho_new / h
  FIN_BI_OMEGA = 7,     // omega = d0 / d1
  FIN_NORM = 8,         // scal[slot0] = sqrt(d0)
  FIN_CG_DEF_BETA = 9   // def = sqrt(d0) + convergence check; beta = d1 / rholast;
                        // rholast = d1; a stop marks the iteration's x update pending
};

struct RedCtx {
  double *partials;   // [kRedBlocks * 2]
  double *scal;       // [S_COUNT]
  int *flags;         // [F_COUNT]
};

// Finisher of a reduction: updates the Krylov scalars (dune-istl's
// CGSolver / BiCGSTABSolver recurrences and breakdown tests) from the two
// reduced sums d0, d1.
__device__ inline void run_finisher(const RedCtx &rc, int fin, int slot0, int slot1, double d0,
                             double d1) {
  double *s = rc.scal;
  int *fl = rc.flags;
  switch (fin) {
    case FIN_STORE:
      if (slot0 >= 0) s[slot0] = d0;
      if (slot1 >= 0) s[slot1] = d1;
      break;
    case FIN_NORM:
      s[slot0] = sqrt(d0);
      break;
    case FIN_DEF0: {
      const double def = sqrt(d0);
      s[S_DEF0] = def;
      s[S_DEF] = def;
      if (!isfinite(def)) fl[F_STATE] = 2;
      else if (def < def * s[S_RED] || def < 1e-30) fl[F_STATE] = 1;
      break;
    }
    case FIN_DEF: {
      const double def = sqrt(d0);
      s[S_DEF] = def;
      if (!isfinite(def)) fl[F_STATE] = 2;
      else if (def < s[S_DEF0] * s[S_RED] || def < 1e-30) fl[F_STATE] = 1;
      if (slot0 == S_RHO) s[S_RHO] = s[S_RHONEW];   // BiCGStab: rho = rho_new
      break;
    }
    case FIN_CG_LAMBDA:
      s[S_ALPHA] = s[S_RHO] / d0;
      break;
    case FIN_CG_BETA:
      s[S_BETA] = d0 / s[S_RHO];
      s[S_RHO] = d0;
      break;
    case FIN_CG_DEF_BETA: {
      // CGSolver: the defect check after b -= lambda q, then (when it goes
      // on) rho = <M^{-1} b, b>, beta = rho / rholast
      const double def = sqrt(d0);
      s[S_DEF] = def;
      if (!isfinite(def)) fl[F_STATE] = 2;
      else if (def < s[S_DEF0] * s[S_RED] || def < 1e-30) fl[F_STATE] = 1;
      if (fl[F_STATE]) fl[F_XPEND] = 1;
      s[S_BETA] = d1 / s[S_RHO];
      s[S_RHO] = d1;
      break;
    }
    // BiCGSTABSolver breakdown tests are absolute (rho, omega <= 1e-80,
    // |h| < 1e-80).  With S_GUARD > 0 (FP32 inner solves, whose dot products
    // carry ~1e-7 relative noise) a relative test is added:
    // |<rt, r>| or |<rt, v>| below S_GUARD |rt| |r| (|rt| |v|) is treated as a
    // breakdown, and the solve stops with the last finite iterate.
    case FIN_BI_RHONEW:
      s[S_RHONEW] = d0;
      if (fabs(s[S_RHO]) <= 1e-80 || fabs(s[S_OMEGA]) <= 1e-80 || !isfinite(d0) ||
          (s[S_GUARD] > 0 && fabs(d0) < s[S_GUARD] * s[S_DEF0] * s[S_DEF]))
        fl[F_STATE] = 3;
      else
        s[S_BETA] = (d0 / s[S_RHO]) * (s[S_ALPHA] / s[S_OMEGA]);
      break;
    case FIN_BI_ALPHA:
      s[S_H] = d0;
      if (fabs(d0) < 1e-80 || !isfinite(d0) ||
          (s[S_GUARD] > 0 && fabs(d0) < s[S_GUARD] * s[S_DEF0] * sqrt(d1)))
        fl[F_STATE] = 3;
      else
        s[S_ALPHA] = s[S_RHONEW] / d0;
      break;
    case FIN_BI_OMEGA:
      s[S_TR] = d0;
      s[S_TT] = d1;
      if (!(d1 > 0.0) || !isfinite(d0 / d1)) fl[F_STATE] = 3;
      else s[S_OMEGA] = d0 / d1;
      break;
    default:
      break;
  }
}


// ---- reductions fused into other kernels ----------------------------------
// A kernel that produces one operand of a dot product (the operator writing
// q = A p, the block preconditioner writing z = M^{-1} r) adds the product of
// its own output with the other operand per block.  Same determinism as the
// dot kernels: block partials in a per-kernel array, the last block adds
// them in block order and runs the finisher.  Blocks of any size <= MAXT.
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int MAXT>
__device__ __forceinline__ void block_sum2_with(double &a, double &b, double *sa, double *sb) {
  __syncthreads();   // the arrays may still be read by a previous call
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = 0.0, y = 0.0;
    for (unsigned i = threadIdx.x; i < blockDim.x; i += 32) {
      x += sa[i];
      y += sb[i];
    }
    a = warp_sum_d(x);
    b = warp_sum_d(y);
  }
}

template <int MAXT>
__device__ __forceinline__ void block_sum2_any(double &a, double &b) {
  __shared__ double sa[MAXT], sb[MAXT];
  block_sum2_with<MAXT>(a, b, sa, sb);
}

// block sums through a caller-provided scratch of 2 * MAXT doubles (the
// kernel's dynamic shared memory) or static arrays
template <int MAXT, bool kScratch>
__device__ __forceinline__ void block_sum2_sel(double &a, double &b, double *scratch) {
  if constexpr (kScratch) block_sum2_with<MAXT>(a, b, scratch, scratch + MAXT);
  else block_sum2_any<MAXT>(a, b);
}

// Two-level tail for grids of many blocks: the last block of each group of
// kFuseGroup blocks adds the group's partials in block order into a group
// partial; the last group to finish adds the group partials in group order
// and runs the finisher.  The order of every sum is fixed, so the result does
// not depend on which block finishes last.  Layout of `part`: 2 doubles per
// block, then 2 per group from offset 2 * max_blocks; `cnt`: one int per
// group, zero between launches (each group's last block resets its own).
constexpr int kFuseGroup = 256;

template <int MAXT, bool kScratch = false>
__device__ __forceinline__ void reduce_tail_grouped(double *part, long max_blocks, int *cnt,
                                                    const RedCtx &rc, double s0, double s1,
                                                    int fin, int slot0, int slot1,
                                                    double *scratch = nullptr) {
  __shared__ bool last;
  block_sum2_sel<MAXT, kScratch>(s0, s1, scratch);
  const int b = (int)blockIdx.x, g = b / kFuseGroup;
  const int ngroups = (int)((gridDim.x + kFuseGroup - 1) / kFuseGroup);
  const int gsize = min(kFuseGroup, (int)gridDim.x - g * kFuseGroup);
  if (threadIdx.x == 0) {
    part[2 * b] = s0;
    part[2 * b + 1] = s1;
    __threadfence();
    last = atomicAdd(&cnt[g], 1) == gsize - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < gsize; i += blockDim.x) {
    a += __ldcg(part + 2 * (g * kFuseGroup + i));
    c += __ldcg(part + 2 * (g * kFuseGroup + i) + 1);
  }
  block_sum2_sel<MAXT, kScratch>(a, c, scratch);
  double *gpart = part + 2 * max_blocks;
  if (threadIdx.x == 0) {
    gpart[2 * g] = a;
    gpart[2 * g + 1] = c;
    cnt[g] = 0;
    __threadfence();
    last = atomicAdd(&rc.flags[F_COUNTER], 1) == ngroups - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  a = 0.0;
  c = 0.0;
  for (int i = threadIdx.x; i < ngroups; i += blockDim.x) {
    a += __ldcg(gpart + 2 * i);
    c += __ldcg(gpart + 2 * i + 1);
  }
  block_sum2_sel<MAXT, kScratch>(a, c, scratch);
  if (threadIdx.x == 0) {
    run_finisher(rc, fin, slot0, slot1, a, c);
    rc.flags[F_COUNTER] = 0;
  }
}

int red_dot(pdg_context *ctx, const RedCtx &rc, long n, const double *a, const double *b,
            const double *c, const double *d, int fin, int slot0, int slot1, bool respect_flag);
int red_dot_f32(pdg_context *ctx, const RedCtx &rc, long n, const float *a, const float *b,
                const float *c, const float *d, int fin, int slot0, int slot1,
                bool respect_flag);

// fused updates (skip when the flag is raised)
template <typename T>
int cg_update_xr(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *r, const T *p,
                 const T *q);   // x += lambda p; r -= lambda q; def check
template <typename T>
int cg_update_p(pdg_context *ctx, const RedCtx &rc, long n, T *p, const T *z);  // p = z + beta p
// fused CG: x += lambda p ; p = z + beta p (the residual update and defect
// check ran in the preconditioner kernel) and, after the loop, the x update of
// the stopping iteration
template <typename T>
int cg_update_px(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *p, const T *z);
template <typename T>
int cg_finish_x(pdg_context *ctx, const RedCtx &rc, long n, T *x, const T *p);
template <typename T>
int bi_update_p(pdg_context *ctx, const RedCtx &rc, long n, T *p, const T *r, const T *v,
                int first);   // p = r (first) or p = beta (p - omega v) + r
template <typename T>
int bi_update_half(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *r, const T *y,
                   const T *v);   // x += alpha y; r -= alpha v; def check
template <typename T>
int bi_update_full(pdg_context *ctx, const RedCtx &rc, long n, T *x, T *r, const T *y,
                   const T *t);   // x += omega y; r -= omega t; def check; rho = rho_new
int set_iter(pdg_context *ctx, const RedCtx &rc, double it);
int inc_iter(pdg_context *ctx, const RedCtx &rc, double step);

// plain vector kernels
template <typename T>
int vec_copy(pdg_context *ctx, long n, const T *src, T *dst);
template <typename T>
int vec_fill(pdg_context *ctx, long n, T *dst, T v);
int vec_axpy(pdg_context *ctx, long n, double alpha, const double *x, double *y);
// y32 = (float)(x64 * s) with s = 1/scal[S_SCALE]
int vec_to_f32_scaled(pdg_context *ctx, long n, const double *x, float *y, const double *scal);
// y64 += scal[S_SCALE] * sign * (double)x32
int vec_add_f32_scaled(pdg_context *ctx, long n, const float *x, double *y, const double *scal,
                       double sign);
int vec_to_f32(pdg_context *ctx, long n, const double *x, float *y);
// skip-aware conversions around an FP32 operator inside an FP64 Krylov solve:
// y32 = (float)x ;  y = (acc ? y : 0) + alpha (double)s32 + (add ? add : 0)
int vec_to_f32_skip(pdg_context *ctx, long n, const double *x, float *y, const int *skip);
int vec_from_f32_combine(pdg_context *ctx, long n, const float *s32, double *y, const double *add,
                         double alpha, int acc, const int *skip);

}  // namespace pdg
