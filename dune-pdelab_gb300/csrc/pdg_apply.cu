// pdg_apply.cu -- the fused cell operator of ConvectionDiffusionDG (SIPG /
// NIPG / IIPG, scalar cellwise permeability) on a structured grid:
// volume + interior faces + boundary faces in one kernel.
//
// Reference: jacobian_apply_volume / _skeleton / _boundary
// (dune/pdelab/localoperator/convectiondiffusiondg.hh:191-195, 474-481,
// 892-899; bodies :105-188, :270-471, :683-879), driven by
// GridOperator::jacobian_apply (gridoperator/gridoperator.hh:192-197).
//
// Formulation.  On an axis-parallel cell with A = K I, Gauss order 2k and
// Lagrange Q_k, every term of the operator is a Kronecker product of 1D
// matrices (the Gauss rule with k+1 points integrates all 1D products of
// degree <= 2k exactly).  The block row of cell e is
//
//   y_e = sum_dir  (A'_dir (x) M (x) M)_dir u_e
//       + sum_faces (B'_face (x) M (x) M)_dir u_neighbour
//
// with Mhat the 1D mass matrix, A'_dir = hperp_dir [ (K_e/h) Shat
// + (c h Mhat if dir = x) + the self terms of the two faces normal to dir ]
// (hperp = product of the tangential cell sizes) and B'_face the rank-2
// coupling through the neighbour's face value and normal derivative.
// Face coefficients reproduce the reference exactly: kappa_e = omega_e K_e
// (omega_e = K_o/(K_e+K_o+1e-20), :326-332), penalty =
// alpha/h_F * harmonic_average * k(k+d-1) (:346, :734), Dirichlet faces
// with K_e and h_F = |T|/|F| (:717-727), theta = -1/+1/0 (:99-101).
//
// Per-cell data (A'_dir and five scaled coefficients per face) is either
// read from a record precomputed once per coefficient field or formed on
// the fly (2D FP32).  The FP64 operator is bound by its FP64 pipe: the
// record removes all divisions and matrix assembly from the apply, and in
// 3D it carries per face the coefficients of the neighbour line (see
// k_cell_record) so that each face point costs N + 1 FP64 operations.
//
// Thread mapping (d = 3): N*N threads per cell, thread (tx,ty) holds the
// z-column u[.,ty,tx] in registers; x/y contractions go through shared
// memory.  d = 2: N threads per cell holding y-columns.  All neighbour
// lines are loaded before any arithmetic so that 2dN loads are in flight.
#include "pdg_ops.cuh"
#include "pdg_vec.cuh"

namespace pdg {

template <int D, int N>
struct Cfg {
  static constexpr int N2 = N * N;
  static constexpr int NB = D == 3 ? N * N * N : N * N;   // DOFs per cell
  static constexpr int TPC = D == 3 ? N * N : N;          // threads per cell
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;  // cells per block
  static constexpr int THREADS = CPB * TPC;
  static constexpr int NF = 2 * D;
  static constexpr int REC = D * N2 + 5 * NF;             // per-cell record
  // 3D FP64 record: A'_dir, then per face the coefficients W_f[0..N] of the
  // neighbour line (see k_cell_record), for the operator and for its transpose
  static constexpr int NW = NF * (N + 1);
  static constexpr int RECW = D * N2 + 2 * NW;
  // shared memory per cell (elements): ue, Xs, Ys, Zs, face data, record, raw coefs
  static constexpr int PER_CELL = (D == 3 ? 4 * NB : 2 * NB) + 4 * D * TPC + REC + 3 * NF;
  static constexpr int TAB = 2 * N2 + 2 * N;
};

// Padding (elements) added to the per-cell shared region of k_apply so that
// the cells that share a warp fall on different shared-memory banks; chosen
// by counting the wavefronts of the kernel's shared accesses per padding
// (e.g. 3D Q3 FP32: 544 floats per cell put both cells of a warp on the same
// banks, 16 more halve the wavefronts).
template <typename T, int D, int N>
constexpr int cell_pad() {
  if (D != 3) return 0;
  if (sizeof(T) == 4) return N == 3 ? 6 : N == 4 ? 16 : N == 5 ? 30 : 0;
  return N == 3 ? 2 : N == 5 ? 14 : 0;
}

// tangential face scale of direction dir (product of the other cell sizes)
template <typename T, int D>
__device__ __forceinline__ T hperp(const OpParams<T> &p, int dir) {
  T s = T(1);
#pragma unroll
  for (int j = 0; j < D; j++)
    if (j != dir) s *= p.h[j];
  return s;
}

// Scaled face coefficients of face f from the raw {kappa_e/h, kappa_o/h, pen}:
// {hp ke, hp ko, hp pen, theta hp ke, theta hp ko}
template <typename T, int D>
__device__ __forceinline__ void scale_face(const OpParams<T> &p, int f, const T *raw, T *c5) {
  const T hp = hperp<T, D>(p, f >> 1);
  c5[0] = hp * raw[0];
  c5[1] = hp * raw[1];
  c5[2] = hp * raw[2];
  c5[3] = p.theta * c5[0];
  c5[4] = p.theta * c5[1];
}

// lexicographic cell coordinates (x fastest) by multiply-high division
template <typename T>
__device__ __forceinline__ void cell_coords(const OpParams<T> &p, unsigned e, int *ix) {
  const unsigned q0 = p.div0.div(e);
  const unsigned q1 = p.div1.div(q0);
  ix[0] = (int)(e - q0 * (unsigned)p.nc[0]);
  ix[1] = (int)(q0 - q1 * (unsigned)p.nc[1]);
  ix[2] = (int)q1;
}

// True where the record carries per-face line coefficients instead of the
// five scaled face coefficients: the 3D FP64 operator, bound by its FP64 pipe.
template <typename T, int D>
constexpr bool face_vectors() { return sizeof(T) == 8 && D == 3; }

// Record of one cell (computed in FP64, stored in T): A'_dir row-major, then
// five scaled coefficients per face {hp ke, hp ko, hp pen, th hp ke, th hp ko},
// or, for the 3D FP64 operator, per face f the coefficients of the neighbour
// line v (its N values along the face normal): the face terms of this cell are
// s1 = sum_q W_f[q] v[q] and s2 = W_f[N] v[qv], with qv = N-1 for the
// neighbour below and 0 above,
//   W_f[q] = sg ko' td[q] - [q = qv] pen,   W_f[N] = sg ke'
// (td: the derivative of the 1D basis at the shared face; ko', ke' = hp ko,
// th hp ke for the operator and th hp ko, hp ke for its transpose; sg = +-1
// by side and form).  The neighbour's normal derivative and face value are
// folded into these coefficients, which takes 2 FP64 operations per face
// point out of the apply.
template <typename T, int D, int N>
__global__ void k_cell_record(const OpParams<double> p, T *__restrict__ rec) {
  using C = Cfg<D, N>;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  const double *tM = p.tab, *tS = p.tab + N * N, *td0 = tS + N * N, *td1 = td0 + N;
  int ix[3];
  cell_coords(p, (unsigned)e, ix);
  const long stride[3] = {1, (long)p.nc[0], (long)p.nc[0] * p.nc[1]};
  const double cc = p.c ? p.c[e] : 0.0;
  double raw[3 * 2 * D];
#pragma unroll
  for (int f = 0; f < 2 * D; f++) {
    const int dir = f >> 1;
    long nb;
    if (f & 1) nb = ix[dir] + 1 < p.nc[dir] ? e + stride[dir] : -1;
    else nb = ix[dir] > 0 ? e - stride[dir] : -1;
    face_coefficients(p, f, kdir(p, e, dir), nb, raw + 3 * f);
  }
  T *r = rec + e * (face_vectors<T, D>() ? C::RECW : C::REC);
#pragma unroll
  for (int dir = 0; dir < D; dir++) {
    const double hp = hperp<double, D>(p, dir);
    for (int i = 0; i < N; i++)
      for (int a = 0; a < N; a++)
        r[dir * N * N + i * N + a] =
            (T)(hp * a_entry<double, N>(p, dir, i, a, kdir(p, e, dir), cc, raw, tM, tS, td0,
                                        td1));
  }
#pragma unroll
  for (int f = 0; f < 2 * D; f++) {
    double c5[5];
    scale_face<double, D>(p, f, raw + 3 * f, c5);
    if constexpr (face_vectors<T, D>()) {
      const int hi = f & 1, qv = hi ? 0 : N - 1;
      const double *td = hi ? td0 : td1;
      for (int tr = 0; tr < 2; tr++) {
        const double sg = (hi ^ tr) ? -1.0 : 1.0;
        const double ko = tr ? c5[4] : c5[1];
        T *w = r + D * N * N + tr * C::NW + f * (N + 1);
        for (int q = 0; q < N; q++) w[q] = (T)(sg * ko * td[q] - (q == qv ? c5[2] : 0.0));
        w[N] = (T)(sg * (tr ? c5[0] : c5[3]));
      }
    } else {
      for (int j = 0; j < 5; j++) r[D * N * N + 5 * f + j] = (T)c5[j];
    }
  }
}

template <typename T, int D, int N>
__global__ void __launch_bounds__(Cfg<D, N>::THREADS)
    k_apply(const OpParams<T> p, const ApplyArgs<T> a, const T *__restrict__ rec) {
  using C = Cfg<D, N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB, NF = C::NF;
  constexpr int PER_CELL = C::PER_CELL + cell_pad<T, D, N>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *tM = reinterpret_cast<T *>(smem_raw);
  T *tS = tM + N2;
  T *td0 = tS + N2;
  T *td1 = td0 + N;
  const int t = threadIdx.x;
  const int cs = t / TPC;
  const int l = t - cs * TPC;
  T *cellmem = tM + C::TAB + cs * PER_CELL;
  T *ue = cellmem;
  T *Xs = ue + NB;
  T *Ys = Xs + (D == 3 ? NB : 0);
  T *Zs = Ys + NB;
  T *fa = (D == 3 ? Zs + NB : Ys + NB);     // [2D][2][TPC]
  T *Am = fa + 4 * D * TPC;                 // record: [D][N2] then [2D][5]
  T *c5 = Am + D * N2;
  T *raw = c5 + 5 * NF;                     // [2D][3] (on-the-fly path)

  if (a.skip && *a.skip) return;
  for (int i = t; i < C::TAB; i += blockDim.x) tM[i] = p.tab[i];

  const int li = blockIdx.x * CPB + cs;         // cell counts fit 31 bits
  const bool ranged = !a.cells && a.ncells > 0;
  const bool active = (a.cells || ranged) ? li < a.ncells : li < p.ncell;
  const int e = a.cells ? (active ? a.cells[li] : 0) : (ranged ? a.cell0 + li : li);
  const int ee = active ? e : 0;
  int ix[3];
  cell_coords(p, (unsigned)ee, ix);
  const int stride[3] = {1, p.nc[0], p.nc[0] * p.nc[1]};
  int nbr[NF];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    if (f & 1) nbr[f] = ix[dir] + 1 < p.nc[dir] ? ee + stride[dir] : -1;
    else nbr[f] = ix[dir] > 0 ? ee - stride[dir] : -1;
  }

  // ---- all global loads first: own column, neighbour lines, record ----
  T col[N];
  const T *xe = a.x + (size_t)ee * NB;
#pragma unroll
  for (int z = 0; z < N; z++) col[z] = xe[z * TPC + l];
  T v[NF][N];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    const int nb = (nbr[f] >= 0 && !a.diag_only) ? nbr[f] : ee;
    const T *xn = a.x + (size_t)nb * NB;
#pragma unroll
    for (int q = 0; q < N; q++) {
      int off;
      if (D == 3)
        off = dir == 0 ? l * N + q : (dir == 1 ? (l / N) * N2 + q * N + (l % N) : q * N2 + l);
      else
        off = dir == 0 ? l * N + q : q * N + l;
      v[f][q] = xn[off];
    }
  }
  if (rec) {
    if constexpr (face_vectors<T, D>()) {
      // A'_dir and the line coefficients of this launch's form (into the
      // face-coefficient region: NW <= 5 NF + 3 NF)
      const T *r = rec + (size_t)ee * C::RECW;
      const int woff = a.transpose ? C::NW : 0;
      for (int i = l; i < D * N2 + C::NW; i += TPC) Am[i] = r[i < D * N2 ? i : i + woff];
    } else {
      const T *r = rec + (size_t)ee * C::REC;
      for (int i = l; i < C::REC; i += TPC) Am[i] = r[i];
    }
  }
#pragma unroll
  for (int z = 0; z < N; z++) ue[z * TPC + l] = col[z];
  if (!rec) {
#pragma unroll
    for (int f = 0; f < NF; f++)
      if (f % TPC == l) {
        face_coefficients(p, f, kdir(p, ee, f >> 1), nbr[f], raw + 3 * f);
        scale_face<T, D>(p, f, raw + 3 * f, c5 + 5 * f);
      }
    __syncthreads();
    const T cc = p.c ? p.c[ee] : T(0);
    if (D == 3) {
      const int i = l / N, aa = l % N;
#pragma unroll
      for (int dir = 0; dir < D; dir++)
        Am[dir * N2 + l] = hperp<T, D>(p, dir) *
                           a_entry<T, N>(p, dir, i, aa, kdir(p, ee, dir), cc, raw, tM, tS, td0,
                                         td1);
    } else {
#pragma unroll
      for (int dir = 0; dir < D; dir++)
#pragma unroll
        for (int aa = 0; aa < N; aa++)
          Am[dir * N2 + l * N + aa] =
              hperp<T, D>(p, dir) *
              a_entry<T, N>(p, dir, l, aa, kdir(p, ee, dir), cc, raw, tM, tS, td0, td1);
    }
  }
  __syncthreads();

  // ---- neighbour face data: one line per thread per face ----
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int hi = f & 1;
    T s1 = T(0), s2 = T(0);
    if constexpr (face_vectors<T, D>()) {
      if (nbr[f] >= 0 && !a.diag_only) {
        const T *w = c5 + f * (N + 1);
#pragma unroll
        for (int q = 0; q < N; q++) s1 += w[q] * v[f][q];
        s2 = w[N] * v[f][hi ? 0 : N - 1];
      }
    } else if (nbr[f] >= 0 && !a.diag_only) {
      const T *cf = c5 + 5 * f;   // hp ke, hp ko, hp pen, th hp ke, th hp ko
      T dv = T(0);
      if (!hi) {
        // neighbour below: its upper face touches this cell's lower face
#pragma unroll
        for (int q = 0; q < N; q++) dv += td1[q] * v[f][q];
        const T val = v[f][N - 1];
        if (!a.transpose) {
          s1 = cf[1] * dv - cf[2] * val;
          s2 = cf[3] * val;
        } else {
          s1 = -cf[2] * val - cf[4] * dv;
          s2 = -cf[0] * val;
        }
      } else {
#pragma unroll
        for (int q = 0; q < N; q++) dv += td0[q] * v[f][q];
        const T val = v[f][0];
        if (!a.transpose) {
          s1 = -cf[1] * dv - cf[2] * val;
          s2 = -cf[3] * val;
        } else {
          s1 = -cf[2] * val + cf[4] * dv;
          s2 = cf[0] * val;
        }
      }
    }
    fa[(2 * f) * TPC + l] = s1;
    fa[(2 * f + 1) * TPC + l] = s2;
  }
  __syncthreads();

  // A'_dir rows (transposed operator: columns) needed by this thread, and
  // the tangential mass rows, in registers
  const int tr = a.transpose;
  auto Aat = [&](int dir, int i, int q) -> T {
    return Am[dir * N2 + (tr ? q * N + i : i * N + q)];
  };

  T out[N];
  if constexpr (D == 3) {
    const int tx = l % N, ty = l / N;
    T Arx[N], Ary[N], Mtx[N], Mty[N];
#pragma unroll
    for (int q = 0; q < N; q++) {
      Arx[q] = Aat(0, tx, q);
      Ary[q] = Aat(1, ty, q);
      Mtx[q] = tM[tx * N + q];
      Mty[q] = tM[ty * N + q];
    }
    const T d0x = td0[tx], d1x = td1[tx], d0y = td0[ty], d1y = td1[ty];
    const T zf0 = fa[8 * TPC + l], zf1 = fa[9 * TPC + l];
    const T zf2 = fa[10 * TPC + l], zf3 = fa[11 * TPC + l];
    T X[N], Y[N], Z[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T sx = T(0), sy = T(0), sz = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        sx += Arx[q] * ue[z * N2 + ty * N + q];
        sy += Ary[q] * ue[z * N2 + q * N + tx];
        sz += Aat(2, z, q) * col[q];
      }
      const int lx = z * N + ty, ly = z * N + tx;
      if (tx == 0) sx += fa[0 * TPC + lx];
      sx += d0x * fa[1 * TPC + lx];
      if (tx == N - 1) sx += fa[2 * TPC + lx];
      sx += d1x * fa[3 * TPC + lx];
      if (ty == 0) sy += fa[4 * TPC + ly];
      sy += d0y * fa[5 * TPC + ly];
      if (ty == N - 1) sy += fa[6 * TPC + ly];
      sy += d1y * fa[7 * TPC + ly];
      if (z == 0) sz += zf0;
      sz += td0[z] * zf1;
      if (z == N - 1) sz += zf2;
      sz += td1[z] * zf3;
      X[z] = sx;
      Y[z] = sy;
      Z[z] = sz;
    }
#pragma unroll
    for (int z = 0; z < N; z++) {
      Xs[z * N2 + l] = X[z];
      Ys[z * N2 + l] = Y[z];
      Zs[z * N2 + l] = Z[z];
    }
    __syncthreads();
    // W = M_y X + M_x Y ; T1 = M_x Z   (tangential masses; scales are in A')
    T W[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T w = T(0), t1 = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        w += Mty[q] * Xs[z * N2 + q * N + tx];
        w += Mtx[q] * Ys[z * N2 + ty * N + q];
        t1 += Mtx[q] * Zs[z * N2 + ty * N + q];
      }
      W[z] = w;
      ue[z * N2 + l] = t1;   // ue is free: all reads finished before the sync
    }
    __syncthreads();
    // out = M_z W + M_y T1
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        s += tM[z * N + q] * W[q];
        s += Mty[q] * ue[z * N2 + q * N + tx];
      }
      out[z] = s;
    }
  } else {
    const int tx = l;
    T Arx[N], Mtx[N];
#pragma unroll
    for (int q = 0; q < N; q++) {
      Arx[q] = Aat(0, tx, q);
      Mtx[q] = tM[tx * N + q];
    }
    const T d0x = td0[tx], d1x = td1[tx];
    const T yf0 = fa[4 * TPC + tx], yf1 = fa[5 * TPC + tx];
    const T yf2 = fa[6 * TPC + tx], yf3 = fa[7 * TPC + tx];
    T X[N];
#pragma unroll
    for (int y = 0; y < N; y++) {
      T sx = T(0), sy = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        sx += Arx[q] * ue[y * N + q];
        sy += Aat(1, y, q) * col[q];
      }
      if (tx == 0) sx += fa[0 * TPC + y];
      sx += d0x * fa[1 * TPC + y];
      if (tx == N - 1) sx += fa[2 * TPC + y];
      sx += d1x * fa[3 * TPC + y];
      if (y == 0) sy += yf0;
      sy += td0[y] * yf1;
      if (y == N - 1) sy += yf2;
      sy += td1[y] * yf3;
      X[y] = sx;
      Ys[y * N + tx] = sy;
    }
    __syncthreads();
    // out = M_y X + M_x Y
#pragma unroll
    for (int y = 0; y < N; y++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        s += tM[y * N + q] * X[q];
        s += Mtx[q] * Ys[y * N + q];
      }
      out[y] = s;
    }
  }

  double part = 0.0;   // <x, y_out> of this thread's entries (fused CG dot)
  if (active) {
    T *ye = a.y + (size_t)e * NB;
    const T *ad = a.add ? a.add + (size_t)e * NB : nullptr;
    const bool scale = a.alpha != T(1);
#pragma unroll
    for (int z = 0; z < N; z++) {
      const int idx = z * TPC + l;
      T r = scale ? a.alpha * out[z] : out[z];
      if (a.accumulate) r += ye[idx];
      if (ad) r += ad[idx];
      ye[idx] = r;
      part += (double)col[z] * (double)r;
    }
  }
  // (compiled for the 2D FP64 operator only, the one fused CG that uses it)
  if constexpr (D == 2 && sizeof(T) == 8) if (a.dot_part) {
    // block sums in the cell memory, free once every thread is past its reads
    __syncthreads();
    reduce_tail_grouped<C::THREADS, true>(a.dot_part, a.dot_max_blocks, a.dot_cnt,
                                          RedCtx{nullptr, a.dot_scal, a.dot_flags}, part, 0.0,
                                          a.dot_fin, -1, -1,
                                          reinterpret_cast<double *>(smem_raw));
  }
}

template <typename T>
OpParams<T> make_params(const pdg_context *ctx, const T *K, const T *c, const T *tab) {
  OpParams<T> p;
  for (int j = 0; j < 3; j++) {
    p.nc[j] = j < ctx->dim ? ctx->cfg.cells[j] : 1;
    p.h[j] = (T)ctx->h[j];
    p.inv_h[j] = (T)(1.0 / ctx->h[j]);
  }
  p.div0.init((unsigned)p.nc[0]);
  p.div1.init((unsigned)p.nc[1]);
  p.ncell = ctx->ncell;
  p.theta = (T)ctx->theta;
  p.pen_fac = (T)ctx->pen_fac;
  p.weights = ctx->cfg.weights;
  for (int j = 0; j < 6; j++) p.bc[j] = ctx->cfg.bctype[j];
  p.K = K;
  p.Kd = nullptr;
  if (ctx->gen_A == 3)
    p.Kd = std::is_same<T, double>::value ? (const T *)ctx->Kd64 : (const T *)ctx->Kd32;
  p.c = c;
  p.tab = tab;
  return p;
}
template OpParams<double> make_params<double>(const pdg_context *, const double *,
                                              const double *, const double *);
template OpParams<float> make_params<float>(const pdg_context *, const float *,
                                            const float *, const float *);

template <typename T, int D, int N>
static int launch_apply_dn(pdg_context *ctx, const ApplyArgs<T> &a, const OpParams<T> &p,
                           const T *rec) {
  using C = Cfg<D, N>;
  const size_t smem = sizeof(T) * (C::TAB + C::CPB * (C::PER_CELL + cell_pad<T, D, N>()));
  static int attr_done = -1;
  if (attr_done != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply<T, D, N>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_done = ctx->device;
  }
  if (face_vectors<T, D>() && !rec)
    return set_error(PDG_EUNSUPPORTED, "the 3D FP64 operator runs from its cell records");
  const long work = (a.cells || a.ncells > 0) ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const long blocks = (work + C::CPB - 1) / C::CPB;
  ApplyArgs<T> af = a;
  if (ctx->fuse_fin && !a.cells && a.ncells == 0) {
    // the fused CG: <p, A p> -> lambda in the same launch
    af.dot_part = ctx->fuse_part;
    af.dot_max_blocks = ctx->fuse_max_blocks;
    af.dot_cnt = ctx->fuse_cnt;
    af.dot_scal = ctx->red_out;
    af.dot_flags = ctx->d_flag;
    af.dot_fin = ctx->fuse_fin;
  }
  k_apply<T, D, N><<<(unsigned)blocks, C::THREADS, smem, ctx->stream>>>(p, af, rec);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <int D, int N>
static int record_dn(pdg_context *ctx) {
  using C = Cfg<D, N>;
  if (!ctx->rec64)
    PDG_CUDA_TRY(cudaMalloc(&ctx->rec64, sizeof(double) * (face_vectors<double, D>() ? C::RECW : C::REC) *
                                             ctx->ncell));
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  const unsigned blocks = (unsigned)((ctx->ncell + 127) / 128);
  k_cell_record<double, D, N><<<blocks, 128, 0, ctx->stream>>>(p, ctx->rec64);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <int N>
static int record32_n(pdg_context *ctx) {
  using C = Cfg<3, N>;
  // 16 floats of slack: bulk copies of a record run round their size up to
  // 16 bytes
  if (!ctx->rec32)
    PDG_CUDA_TRY(cudaMalloc(&ctx->rec32, sizeof(float) * (C::REC * ctx->ncell + 16)));
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  const unsigned blocks = (unsigned)((ctx->ncell + 127) / 128);
  k_cell_record<float, 3, N><<<blocks, 128, 0, ctx->stream>>>(p, ctx->rec32);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// FP32 records of the 3D FP32 operator (computed in FP64, rounded)
static int ensure_record32(pdg_context *ctx) {
  if (ctx->rec32_valid) return PDG_OK;
  int st;
  switch (ctx->N) {
    case 2: st = record32_n<2>(ctx); break;
    case 3: st = record32_n<3>(ctx); break;
    case 4: st = record32_n<4>(ctx); break;
    case 5: st = record32_n<5>(ctx); break;
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
  if (st == PDG_OK) ctx->rec32_valid = 1;
  return st;
}

// FP64 cell records (rebuilt after the coefficients change)
static int ensure_record(pdg_context *ctx) {
  if (ctx->rec_valid) return PDG_OK;
  int st;
  switch (ctx->dim * 10 + ctx->k) {
    case 21: st = record_dn<2, 2>(ctx); break;
    case 22: st = record_dn<2, 3>(ctx); break;
    case 23: st = record_dn<2, 4>(ctx); break;
    case 24: st = record_dn<2, 5>(ctx); break;
    case 31: st = record_dn<3, 2>(ctx); break;
    case 32: st = record_dn<3, 3>(ctx); break;
    case 33: st = record_dn<3, 4>(ctx); break;
    case 34: st = record_dn<3, 5>(ctx); break;
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
  if (st == PDG_OK) ctx->rec_valid = 1;
  return st;
}

// the FP64 operator's lazily built per-cell records, built now (before
// launches are spread over several streams)
int prepare_apply64(pdg_context *ctx, int transpose) {
  PDG_TRY(ensure_record(ctx));
  if (ctx->dim == 3 && ctx->tabm64 && !general_coefficients(ctx))
    PDG_TRY(prepare_apply_m(ctx, transpose));
  if (ctx->f64_pair && ctx->dim == 3 && !general_coefficients(ctx))
    PDG_TRY(prepare_float_pair(ctx));
  return PDG_OK;
}

// Legendre basis: y = acc*y + alpha T^T J_nodal T x + add (pdg_basis.cu)
template <typename T>
static int launch_apply_modal(pdg_context *ctx, const ApplyArgs<T> &a, const T *K, const T *c,
                              const T *tab) {
  if (a.cells || a.ncells > 0)
    return set_error(PDG_EUNSUPPORTED, "cell subsets of the operator (block SOR) need a nodal basis");
  const bool dbl = std::is_same<T, double>::value;
  T *w0 = dbl ? (T *)ctx->legw64[0] : (T *)ctx->legw32[0];
  T *w1 = dbl ? (T *)ctx->legw64[1] : (T *)ctx->legw32[1];
  PDG_TRY(basis_change<T>(ctx, 0, 0, a.x, w0, T(1), 0, nullptr, a.skip));
  ApplyArgs<T> b = a;
  b.x = w0;
  b.y = w1;
  b.add = nullptr;
  b.alpha = T(1);
  b.accumulate = 0;
  ctx->leg_nodal = 1;
  const int st = launch_apply<T>(ctx, b, K, c, tab);
  ctx->leg_nodal = 0;
  PDG_TRY(st);
  return basis_change<T>(ctx, 0, 1, w1, a.y, a.alpha, a.accumulate, a.add, a.skip);
}

template <typename T>
int launch_apply(pdg_context *ctx, const ApplyArgs<T> &a, const T *K, const T *c,
                 const T *tab) {
  if (ctx->basis == PDG_BASIS_LEGENDRE && !ctx->leg_nodal)
    return launch_apply_modal<T>(ctx, a, K, c, tab);
  if (general_coefficients(ctx)) {
    // tensor or per-point coefficients, or 2D convection: the Gauss-point
    // operator (3D convection stays in its own kernel)
    PDG_TRY(launch_apply_general<T>(ctx, a));
    if (convection_on(ctx) && ctx->dim == 3) PDG_TRY(launch_convection<T>(ctx, a));
    return nl_apply<T>(ctx, a);
  }
  OpParams<T> p = make_params<T>(ctx, K, c, tab);
  if constexpr (std::is_same<T, float>::value) {
    // the staged kernels (plane per thread) win for N <= 4: Q1, Q2 (78 vs
    // 126 us at 64^3 Q2) and the Q3 variant with swizzled 16-byte rows; at
    // N = 5 the generic kernel is used
    if (ctx->dim == 3 && ctx->N <= 4 && !a.cells && a.ncells == 0 && K == ctx->K32) {
      PDG_TRY(ensure_record32(ctx));
      PDG_TRY(launch_apply32_3d(ctx, a, p, ctx->rec32));
      if (convection_on(ctx)) PDG_TRY(launch_convection<T>(ctx, a));
      return nl_apply<T>(ctx, a);
    }
  }
  const T *rec = nullptr;
  if (std::is_same<T, double>::value && K == (const T *)ctx->K64) {
    PDG_TRY(ensure_record(ctx));
    rec = (const T *)ctx->rec64;
  } else if (std::is_same<T, float>::value && ctx->dim == 3 && K == (const T *)ctx->K32) {
    // FP32 records (rounded from the FP64 arithmetic): no coefficient
    // assembly or division in the apply
    PDG_TRY(ensure_record32(ctx));
    rec = (const T *)ctx->rec32;
  }
  if constexpr (std::is_same<T, double>::value) {
    if (!ctx->f64_pair && ctx->dim == 3 && rec && ctx->tabm64 && !a.diag_only && !a.cells) {
      // the mass-factored form (fewer FP64 operations), the operator or its
      // transpose
      PDG_TRY(launch_apply_m(ctx, a, p));
      if (convection_on(ctx)) PDG_TRY(launch_convection<T>(ctx, a));
      return nl_apply<T>(ctx, a);
    }
    if (ctx->f64_pair && ctx->dim == 3 && rec) {
      // FP64 applies in float-pair arithmetic on the FP32 pipe
      PDG_TRY(launch_apply_float_pair(ctx, a));
      if (convection_on(ctx)) PDG_TRY(launch_convection<T>(ctx, a));
      return nl_apply<T>(ctx, a);
    }
  }
  const int key = ctx->dim * 10 + ctx->k;
  int st;
  switch (key) {
    case 21: st = launch_apply_dn<T, 2, 2>(ctx, a, p, rec); break;
    case 22: st = launch_apply_dn<T, 2, 3>(ctx, a, p, rec); break;
    case 23: st = launch_apply_dn<T, 2, 4>(ctx, a, p, rec); break;
    case 24: st = launch_apply_dn<T, 2, 5>(ctx, a, p, rec); break;
    case 31: st = launch_apply_dn<T, 3, 2>(ctx, a, p, rec); break;
    case 32: st = launch_apply_dn<T, 3, 3>(ctx, a, p, rec); break;
    case 33: st = launch_apply_dn<T, 3, 4>(ctx, a, p, rec); break;
    case 34: st = launch_apply_dn<T, 3, 5>(ctx, a, p, rec); break;
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
  if (st == PDG_OK && convection_on(ctx)) st = launch_convection<T>(ctx, a);
  if (st == PDG_OK) st = nl_apply<T>(ctx, a);
  return st;
}

template int launch_apply<double>(pdg_context *, const ApplyArgs<double> &, const double *,
                                  const double *, const double *);
template int launch_apply<float>(pdg_context *, const ApplyArgs<float> &, const float *,
                                 const float *, const float *);

}  // namespace pdg
