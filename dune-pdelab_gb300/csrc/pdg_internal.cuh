// pdg_internal.cuh -- shared definitions of the GB300 matrix-free SIPG DG
// library (context, kernel parameter blocks, launch helpers).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <type_traits>

#include "../../include/pdg.h"

namespace pdg {

constexpr int kMaxDim = 3;
constexpr int kMaxDeg = 4;
constexpr int kMaxN1 = kMaxDeg + 1;
// most slabs a host-vector apply is pipelined over (sizes the context's events)
constexpr int kPipeMaxSlabs = 16;
constexpr int kMaxModes = 16;

// Records a message for pdg_last_error() and returns the status code.
int set_error(int status, const std::string &msg);

#define PDG_CUDA_TRY(call)                                                      \
  do {                                                                          \
    cudaError_t _e = (call);                                                    \
    if (_e != cudaSuccess)                                                      \
      return ::pdg::set_error(PDG_ECUDA, std::string(#call) + ": " +            \
                                             cudaGetErrorString(_e));           \
  } while (0)

#define PDG_TRY(call)                                                           \
  do {                                                                          \
    int _s = (call);                                                            \
    if (_s != PDG_OK) return _s;                                                \
  } while (0)

// Velocity b(x) = sum_m coef_m sin(2 pi kv_m . x + phase_m).
struct Velocity {
  int nmodes;
  double m[kMaxModes][7];
};

// Unsigned division by a runtime constant d >= 1 via a 32x32 high multiply
// (round-up method): q = (umulhi(n, m) + n) >> s ... computed as
// t = umulhi(n, m); q = (t + ((n - t) >> 1)) >> (s - 1) for s >= 1.
struct FastDiv {
  unsigned d, m, s;
  void init(unsigned dd) {
    d = dd;
    if (dd == 1) { m = 0; s = 0; return; }
    unsigned l = 0;
    while ((1ull << l) < dd) l++;
    m = (unsigned)(((1ull << 32) * ((1ull << l) - dd)) / dd + 1);
    s = l;
  }
  __host__ __device__ __forceinline__ unsigned div(unsigned n) const {
    if (d == 1) return n;
#ifdef __CUDA_ARCH__
    const unsigned t = __umulhi(n, m);
#else
    const unsigned t = (unsigned)(((unsigned long long)n * m) >> 32);
#endif
    return (t + ((n - t) >> 1)) >> (s - 1);
  }
};

// Everything an operator kernel needs besides the vectors.  Passed by value.
template <typename T>
struct OpParams {
  int nc[3];
  FastDiv div0, div1;   // division by nc[0], nc[1]
  long ncell;
  T h[3];
  T inv_h[3];
  T theta;        // SIPG -1, NIPG +1, IIPG 0
  T pen_fac;      // alpha * k * (k + d - 1)
  int weights;    // PDG_WEIGHTS_ON / OFF
  int bc[6];
  const T *K;     // per cell
  const T *Kd;    // diagonal tensor per cell [ncell][3] (K per direction), or null
  const T *c;     // per cell or nullptr
  const T *tab;   // 1D tables: Mhat[N*N], Shat[N*N], d0[N], d1[N]
};

// One launch of the cell operator:
//   y = (accumulate ? y : 0) + alpha * J x + (add ? add : 0)
template <typename T>
struct ApplyArgs {
  const T *x;
  T *y;
  const T *add;
  T alpha;
  int accumulate;
  int transpose;   // J^T instead of J
  int diag_only;   // drop the neighbour coupling (cell-block diagonal)
  const int *skip; // if non-null and *skip != 0 the launch does nothing
  const int *cells; // if non-null: only these cells (ncells of them) are computed
  int ncells;
  int cell0;        // cells null and ncells > 0: the cell range [cell0, cell0 + ncells)
  // fused dot product <x, y_out> (staged FP32 operator): block partials into
  // dot_part, finisher dot_fin on the Krylov scalars dot_scal / dot_flags
  double *dot_part;
  long dot_max_blocks;
  int *dot_cnt;
  double *dot_scal;
  int *dot_flags;
  int dot_fin;
};

// One cell-block Jacobi preconditioner instance (per precision).
struct PrecData {
  int kind, ready;
  void *Q, *L;     // FDM factors [ncell][d][N*N], [ncell][d][N]
  void *inv;       // dense inverses, column-major per block [ncell][nb*nb]
  void *blk;       // iterative block Jacobi: diagonal blocks, column-major [ncell][nb*nb]
  void *invdiag;   // and the inverses of their diagonals [ncell][nb]
  int *iters;      // block-solve iteration counts of the last apply [ncell]
  void *inv16;     // FP16 dense inverses (dense_fp16), scaled by invscale [ncell]
  float *invscale;
  double *Lsum_inv;  // FP64 FDM: 1 / (sum of the directions' eigenvalues) per DOF [ncell][N^d]
};

}  // namespace pdg

struct pdg_context {
  pdg_config cfg;
  int dim, k, N, nb, nqv, nqf;
  long ncell, ndof, nbpts;
  double h[3];
  double theta, pen_fac;
  cudaStream_t stream;
  cudaStream_t own_stream;
  int device;

  // coefficients on the device
  double *K64;
  float *K32;
  double *c64;
  float *c32;
  double *tab64;
  float *tab32;
  pdg::Velocity vel;

  // source and boundary data on the device
  double *fq, *fc, *gq, *jq, *oq;
  double *r0;          // R(0): source and boundary-data part of the residual
  int r0_valid;
  double *rec64;       // FP64 per-cell operator records (scaled A'_dir + face coefficients)
  int rec_valid;
  double *rec64m;      // 3D: Mhat^-1 A'_dir and the operator's line coefficients (k_apply_m)
  int rec64m_valid;
  double *rec64mT;     // 3D: Mhat^-1 A'_dir^T and the transpose's line coefficients
  int rec64mT_valid;
  double *tabm64;      // 3D: Mhat, Mhat^-1 e0, Mhat^-1 e_{N-1}, Mhat^-1 d0, Mhat^-1 d1, Mhat^-1
  float *rec32;        // the same records rounded to FP32 (3D FP32 operator)
  int rec32_valid;
  float *rec32q;       // Q3: the FP32 records padded to 84 floats, couplings of
  int rec32q_valid;    // faces without a neighbour zeroed (k_apply32_q3t)
  // parameter fields beyond A = K I (pdg_set_permeability_tensor / _points,
  // pdg_set_reaction_points): the diffusion and reaction terms then run in
  // the Gauss-point operator (pdg_general.cu).  gen_A: 0 = scalar K per cell,
  // 1 = tensor per cell Ac [ncell][d*d], 2 = tensor per point Aqv
  // [ncell][nqv][d*d] and Aqf [ncell][2d][nqf][d*d]; cq [ncell][nqv] a
  // per-point reaction added to c.
  // gen_A = 3: a diagonal tensor per cell, kept in Kronecker form with K per
  // direction Kd [ncell][3] (the records, the FDM block Jacobi and R(0) take
  // K_dir for the terms of direction dir; no Gauss-point operator)
  int gen_A;
  double *Ac64, *Aqv64, *Aqf64, *cq64, *Kd64;
  float *Ac32, *Aqv32, *Aqf32, *cq32, *Kd32;
  // FP64 operator applies in float-pair arithmetic (pdg_set_f64_arithmetic):
  // float-pair copies of rec64 and of the 1D tables
  int f64_pair;
  void *recfp, *tabfp;
  int recfp_valid;
  // velocity from point data (pdg_set_velocity_points) instead of Fourier
  // modes: volume points [ncell][nqv][3], face lattice [faces][nqf][3]
  int vel_points;
  double *bqv64, *bqf64;
  double *conv64;      // per-cell weighted velocity at volume and face points (FP64)
  float *conv32;       // the same in FP32
  double *convtab64;   // B and D (basis values / derivatives at Gauss points)
  float *convtab32;
  // GMRES Krylov bases (m+1 vectors), the FP64 flexible-GMRES basis of the
  // mixed solve (2m+1 vectors: V and the preconditioned directions Z), and
  // coefficient scratch
  void *gm_V32, *gm_V64, *gm_F64;
  int gm_m32, gm_m64, gm_mF;
  double *gm_partial, *gm_coef;

  // nonlinear volume term q(u) = sum_m nl_coef[m] u^m (nl_deg 0 = none) and
  // its weights w_q |J| q'(u_x) at the linearization point x
  int nl_deg;
  double nl_coef[5];
  double *nlW64, *nlB64;
  float *nlW32, *nlB32;
  int nl_point;            // weights valid for the current linearization point
  // DG mass matrix (temporal operator): point weights, their inverses, B, B^{-T}
  double *massW, *massWi, *massB, *massBiT;
  // one-step stages: reaction shifted by sigma = a_rr / (b_rr dt)
  double *cstage64, *c_orig64;
  float *cstage32, *c_orig32;
  double mass_shift;
  int mass_shift_on;
  int nl_off;              // temporarily exclude the term (residual evaluation)

  // assembled Jacobian: [ncell][2d+1][nb][nb], column-major blocks
  double *A64;
  int A_valid;
  int use_matrix;          // Krylov operator = assembled Jacobian (matrix-based path)

  // preconditioner, one instance per precision (index PDG_F64 / PDG_F32)
  pdg::PrecData prec[2];
  pdg_prec_options popt;
  // block SOR: cells grouped by hyperplane ix+iy+iz = s (grid order within
  // each), hp_off[s] .. hp_off[s+1] on the host; the sweep's scratch vectors
  int *hp_cells;
  long *hp_off;
  int hp_n;
  double *sor_a64, *sor_d64, *sor_v64;
  float *sor_a32, *sor_d32, *sor_v32;
  // the sweep captured as a CUDA graph on fixed buffers, per
  // [precision][transpose][with skip flag], valid for generation op_gen
  cudaGraphExec_t sor_graph[2][2][2];
  unsigned sor_graph_gen[2][2][2];
  unsigned op_gen;         // bumped whenever the operator or a preconditioner changes
  double *r0K;             // K-proportional Dirichlet-data part of R(0)

  // reduction scratch (deterministic two-stage reductions)
  double *red_partials;    // [kRedBlocks * 4]
  double *red_out;         // [16] device results
  double *h_red;           // pinned host mirror [16]

  // local basis (PDG_BASIS_*).  Nodal bases: the k+1 nodes on [0,1].  The
  // modal (Legendre) basis runs the nodal kernels between changes of basis:
  // leg64/leg32 hold T[j][i] = P_i(j/k) and T^{-1} (2 N*N values); legw*
  // are nodal work vectors; leg_nodal marks a launch already in nodal form.
  int basis;
  double nodes[8];
  double *leg64;
  float *leg32;
  double *legw64[2];
  float *legw32[2];
  int leg_nodal;

  // dot products fused into the FP32 operator / FDM block Jacobi of the
  // inner CG: fuse_fin != 0 asks the next such launch for <in, out> with that
  // finisher; block and group partials in fuse_part, group counters in
  // fuse_cnt (reduce_tail_grouped)
  double *fuse_part;
  long fuse_max_blocks;
  int *fuse_cnt;
  int fuse_fin;
  void *fuse_q;            // FIN_CG_DEF_BETA: the FDM launch first does b -= lambda q

  // staging buffers for host pointers
  double *stage_a, *stage_b;
  // host-buffer applies pipelined over slabs: copy streams and their events
  cudaStream_t pipe_h2d, pipe_d2h, pipe_k2;
  cudaEvent_t pipe_ev[2 * pdg::kPipeMaxSlabs + 3];   // per slab in / out, start, end, k2

  // solver work vectors (lazily allocated)
  double *w64[10];
  float *w32[8];
  int ops32;               // FP64 Krylov vectors with FP32 operator / preconditioner
  int *d_flag;             // device-side convergence flag / counters
  cudaEvent_t ev0, ev1;
};

namespace pdg {

constexpr int kRedBlocks = 1024;   // partials per reduction (grid size cap)

// kernels / launchers implemented in the .cu files
template <typename T>
int launch_apply(pdg_context *ctx, const ApplyArgs<T> &a, const T *K, const T *c,
                 const T *tab);
int launch_rhs(pdg_context *ctx);
int prepare_apply64(pdg_context *ctx, int transpose);
// per-cell change of basis out = acc*out + alpha (M (x) M (x) M) in + add with
// M = T (which 0) or T^{-1} (which 1), transposed if `transpose`
template <typename T>
int basis_change(pdg_context *ctx, int which, int transpose, const T *in, T *out, T alpha,
                 int acc, const T *add, const int *skip);
// 3D FP32 operator with staged neighbour runs (all cells, coupled or diag_only)
int launch_apply32_3d(pdg_context *ctx, const ApplyArgs<float> &a, const OpParams<float> &p,
                      const float *rec);
int launch_grad_logK(pdg_context *ctx, const double *u, const double *lam, double *g);
int launch_grad_source(pdg_context *ctx, const double *lam, double *g);

template <typename T>
OpParams<T> make_params(const pdg_context *ctx, const T *K, const T *c, const T *tab);

// preconditioner
int prec_setup_impl(pdg_context *ctx, int kind, int precision);
template <typename T>
int prec_apply_impl(pdg_context *ctx, const T *d, T *v, int transpose);
template <typename T>
int prec_apply_skip(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip);
void prec_free(pdg_context *ctx, int precision);
// v_e = scale * D_e^{-1} d_e on a cell list (all cells if null)
template <typename T>
int block_solve(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip,
                const int *cells, int ncells, T scale);
int diag_blocks(pdg_context *ctx, double **D);   // row-major FP64 diagonal blocks
int bj_iterative_setup(pdg_context *ctx, int precision);
template <typename T>
int bj_iterative_apply(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip,
                       const int *cells, int ncells, T scale);
int sor_setup(pdg_context *ctx);
template <typename T>
int sor_apply(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip);
void sor_free(pdg_context *ctx);

// 1D tables on the Gauss points (host-built, passed by value to kernels)
struct RhsTables {
  double B[kMaxN1 * kMaxN1];   // B[q][a] = phi_a(xi_q)
  double w[kMaxN1];            // Gauss weights on [0,1]
  double x[kMaxN1];            // Gauss points on [0,1]
  double d0[kMaxN1], d1[kMaxN1];
};
RhsTables make_rhs_tables(const pdg_context *ctx);
double *rhs_r0K(pdg_context *ctx, bool alloc);
double lagrange_derivative(const pdg_context *ctx, int i, double x);

// nonlinear volume term: linearization point, residual part, Jacobian part
int nl_set_point(pdg_context *ctx, const double *x);
int nl_residual(pdg_context *ctx, const double *x, double *r);
template <typename T>
int nl_apply(pdg_context *ctx, const ApplyArgs<T> &a);
// y = (accumulate ? y : 0) + alpha M x, or M^{-1} x (block-diagonal DG mass)
int mass_apply(pdg_context *ctx, const double *x, double *y, double alpha, int accumulate,
               int inverse);

// assembled Jacobian (probing the matrix-free operator) and its block product
int assemble_jacobian(pdg_context *ctx);
long jacobian_nnz_blocks(const pdg_context *ctx);
int jacobian_rowptr(const pdg_context *ctx, long *rowptr, long *colind);
int matrix_apply(pdg_context *ctx, const double *x, double *y, const double *add, double alpha,
                 int accumulate, int transpose, const int *skip);
int matrix_export(pdg_context *ctx, const long *rowptr_dev, double *values_dev);

// Index of the face normal to `dir` in plane `plane` (0..nc[dir]) whose other
// coordinates are those of ix, on the face lattice: faces normal to x first,
// then y, then z; planes in order; faces of a plane lexicographic over the
// other directions, x fastest.
__host__ __device__ inline long face_lattice_index(const int *nc, int dim, int dir, int plane,
                                                   const int *ix) {
  long off = 0;
  for (int j = 0; j < dir; j++) {
    long n = nc[j] + 1;
    for (int m = 0; m < dim; m++)
      if (m != j) n *= nc[m];
    off += n;
  }
  long inplane = 1, idx = 0;
  for (int m = 0; m < dim; m++)
    if (m != dir) inplane *= nc[m];
  for (int j = dim - 1; j >= 0; j--) {
    if (j == dir) continue;
    idx = idx * nc[j] + ix[j];
  }
  return off + (long)plane * inplane + idx;
}

// the 3D FP64 operator in float-pair arithmetic (pdg_apply_fp.cu); rec64 must
// be valid
int launch_apply_float_pair(pdg_context *ctx, const ApplyArgs<double> &a);
int prepare_float_pair(pdg_context *ctx);
// the 3D FP64 operator with the mass matrix factored out (pdg_apply_m.cu;
// the operator or its transpose, coupled, all cells or a cell range); rec64
// must be valid
int launch_apply_m(pdg_context *ctx, const ApplyArgs<double> &a, const OpParams<double> &p);
int prepare_apply_m(pdg_context *ctx, int transpose);

// parameter fields beyond A = K I: true when the Gauss-point operator replaces
// the Kronecker kernels; its launch (diffusion and reaction terms only)
bool general_coefficients(const pdg_context *ctx);
template <typename T>
int launch_apply_general(pdg_context *ctx, const ApplyArgs<T> &a);
// R(0)'s Dirichlet-data diffusion terms with the tensor (added to ctx->r0)
int launch_rhs_general(pdg_context *ctx);
// the face lattice (every face once: x-normal faces, then y, then z; planes
// in order, faces in a plane lexicographic over the other directions)
long face_lattice_count(const pdg_context *ctx);
// true when convection terms are present (Fourier modes or point data)
inline bool convection_on(const pdg_context *ctx) {
  return ctx->vel.nmodes > 0 || ctx->vel_points;
}

// convection (3D): set-up of the per-cell velocity records, and the launch
// that adds alpha * C x (or C^T x) to y after the diffusion operator
int conv_setup(pdg_context *ctx);
template <typename T>
int launch_convection(pdg_context *ctx, const ApplyArgs<T> &a);

}  // namespace pdg
