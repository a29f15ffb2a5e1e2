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
// 3 breakdown), [1] reduction counter (last-block detection)
enum { F_STATE = 0, F_COUNTER = 1, F_COUNT = 4 };

enum Finisher {
  FIN_STORE = 0,        // scal[slot0] = d0 ; scal[slot1] = d1
  FIN_DEF0 = 1,         // def0 = def = sqrt(d0); iteration 0 check
  FIN_DEF = 2,          // def = sqrt(d0); convergence check at scal[S_ITER]
  FIN_CG_LAMBDA = 3,    // lambda = rholast / d0
  FIN_CG_BETA = 4,      // beta = d0 / rholast; rholast = d0
  FIN_BI_RHONEW = 5,    // rho_new = d0; breakdown checks
  FIN_BI_ALPHA = 6,     // h = d0; alpha = rho_new / h
  FIN_BI_OMEGA = 7,     // omega = d0 / d1
  FIN_NORM = 8          // scal[slot0] = sqrt(d0)
};

struct RedCtx {
  double *partials;   // [kRedBlocks * 2]
  double *scal;       // [S_COUNT]
  int *flags;         // [F_COUNT]
};

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
