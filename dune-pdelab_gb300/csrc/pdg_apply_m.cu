// pdg_apply_m.cu -- the 3D FP64 cell operator with the mass matrix factored
// out (the form of the coupled applies, of the operator and of its transpose).
//
// Same operator as k_apply<double, 3, N> (pdg_apply.cu; reference:
// ConvectionDiffusionDG::jacobian_apply_volume / _skeleton / _boundary,
// localoperator/convectiondiffusiondg.hh:191-195, 474-481, 892-899).  With
// Mhat the 1D mass matrix, the block row of cell e
//
//   y_e = sum_dir (A'_dir (x) Mhat (x) Mhat)_dir u_e + face couplings
//
// is evaluated as
//
//   y_e = (Mhat (x) Mhat (x) Mhat) S,
//   S   = sum_dir (B_dir)_dir u_e + the face couplings lifted by Mhat^-1,
//   B_dir = Mhat^-1 A'_dir   (per cell, in the record, computed in FP64).
//
// A face coupling enters y as (e0 s1 + d0 s2)(x) (x) Mhat (x) Mhat (for the
// lower x face; e0 the unit vector of the face node, d0 the derivative of the
// basis at the face, s1 s2 the neighbour-line terms), so in S it is
// (m0 s1 + md0 s2)(x) with m0 = Mhat^-1 e0, md0 = Mhat^-1 d0: the tangential
// masses cancel.  Per thread (one z-column of N values, N*N threads per
// cell) the volume costs 6 N^2 FP64 multiply-adds instead of the 8 N^2 of the
// three-operator form (three directional applies, then three mass
// contractions instead of three applies and five masses), and the exchanges
// through shared memory halve (two arrays instead of four).  The operator is
// bound by its FP64 pipe, so the time follows the count.
#include "pdg_ops.cuh"

namespace pdg {

template <int N>
struct MCfg {
  static constexpr int N2 = N * N, NB = N * N * N, TPC = N * N, NF = 6;
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  static constexpr int NW = NF * (N + 1);            // neighbour-line coefficients
  static constexpr int RECW = 3 * N2 + 2 * NW;       // the FP64 record (both forms)
  static constexpr int RECM = 3 * N2 + NW;           // B_dir and the operator's lines
  static constexpr int TAB = N2 + 4 * N;             // Mhat, m0, m1, md0, md1
  // ue, S, face data (12 TPC), record; one element of padding per cell
  static constexpr int PER_CELL = 2 * NB + 12 * TPC + RECM + 1;
};

// B_dir = Mhat^-1 A'_dir from the FP64 record, with the operator's line
// coefficients.  For the transposed operator the kernel below runs unchanged
// on B_dir = Mhat^-1 A'_dir^T and the transpose's line coefficients: the
// transposed block row of a cell has the same form (directional matrices
// A'_dir^T, face couplings (e0 s1 + d0 s2) (x) Mhat (x) Mhat with the
// transpose's neighbour-line terms).
template <int N>
__global__ void k_record_m(long ncell, const double *__restrict__ rec,
                           const double *__restrict__ minv, double *__restrict__ out,
                           int transpose) {
  using C = MCfg<N>;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ncell) return;
  const double *r = rec + e * C::RECW;
  double *o = out + e * C::RECM;
  // A'_dir[k][q] at r[k * N + q]; its transpose's entry [k][q] at r[q * N + k]
  const int sk = transpose ? 1 : N, sq = transpose ? N : 1;
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < N; i++)
      for (int q = 0; q < N; q++) {
        double s = 0.0;
        for (int k = 0; k < N; k++) s += minv[i * N + k] * r[d * C::N2 + k * sk + q * sq];
        o[d * C::N2 + i * N + q] = s;
      }
  const double *w = r + 3 * C::N2 + (transpose ? C::NW : 0);
  for (int j = 0; j < C::NW; j++) o[3 * C::N2 + j] = w[j];
}

template <int N>
__global__ void __launch_bounds__(MCfg<N>::THREADS)
    k_apply_m(const OpParams<double> p, const ApplyArgs<double> a, const double *__restrict__ rec,
              const double *__restrict__ tab) {
  using C = MCfg<N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB, NF = C::NF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *tM = reinterpret_cast<double *>(smem_raw);
  double *tm0 = tM + N2, *tm1 = tm0 + N, *tmd0 = tm1 + N, *tmd1 = tmd0 + N;
  const int t = threadIdx.x;
  const int cs = t / TPC;
  const int l = t - cs * TPC;
  double *ue = tM + C::TAB + cs * C::PER_CELL;
  double *Ss = ue + NB;
  double *fa = Ss + NB;              // [2 NF][TPC]
  double *Bm = fa + 2 * NF * TPC;    // B_dir [3][N2], then the line coefficients [NF][N+1]
  double *W = Bm + 3 * N2;

  if (a.skip && *a.skip) return;
  for (int i = t; i < C::TAB; i += blockDim.x) tM[i] = tab[i];

  const int li = blockIdx.x * CPB + cs;
  const bool ranged = a.ncells > 0;
  const bool active = ranged ? li < a.ncells : li < p.ncell;
  const int e = ranged ? a.cell0 + li : li;
  const int ee = active ? e : 0;
  int ix[3];
  {
    const unsigned q0 = p.div0.div((unsigned)ee);
    const unsigned q1 = p.div1.div(q0);
    ix[0] = (int)((unsigned)ee - q0 * (unsigned)p.nc[0]);
    ix[1] = (int)(q0 - q1 * (unsigned)p.nc[1]);
    ix[2] = (int)q1;
  }
  const int stride[3] = {1, p.nc[0], p.nc[0] * p.nc[1]};
  int nbr[NF];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    if (f & 1) nbr[f] = ix[dir] + 1 < p.nc[dir] ? ee + stride[dir] : -1;
    else nbr[f] = ix[dir] > 0 ? ee - stride[dir] : -1;
  }

  // ---- all global loads first: own column, neighbour lines, record ----
  double col[N];
  const double *xe = a.x + (size_t)ee * NB;
#pragma unroll
  for (int z = 0; z < N; z++) col[z] = xe[z * TPC + l];
  double v[NF][N];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    const int nb = nbr[f] >= 0 ? nbr[f] : ee;
    const double *xn = a.x + (size_t)nb * NB;
#pragma unroll
    for (int q = 0; q < N; q++) {
      const int off =
          dir == 0 ? l * N + q : (dir == 1 ? (l / N) * N2 + q * N + (l % N) : q * N2 + l);
      v[f][q] = xn[off];
    }
  }
  {
    const double *r = rec + (size_t)ee * C::RECM;
    for (int i = l; i < C::RECM; i += TPC) Bm[i] = r[i];
  }
#pragma unroll
  for (int z = 0; z < N; z++) ue[z * TPC + l] = col[z];
  __syncthreads();

  // ---- neighbour face data: one line per thread per face ----
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int hi = f & 1;
    double s1 = 0.0, s2 = 0.0;
    if (nbr[f] >= 0) {
      const double *w = W + f * (N + 1);
#pragma unroll
      for (int q = 0; q < N; q++) s1 += w[q] * v[f][q];
      s2 = w[N] * v[f][hi ? 0 : N - 1];
    }
    fa[(2 * f) * TPC + l] = s1;
    fa[(2 * f + 1) * TPC + l] = s2;
  }
  __syncthreads();

  const int tx = l % N, ty = l / N;
  // S = sum_dir B_dir u + lifted face terms (own column)
  {
    double Bx[N], By[N];
#pragma unroll
    for (int q = 0; q < N; q++) {
      Bx[q] = Bm[tx * N + q];
      By[q] = Bm[N2 + ty * N + q];
    }
    const double m0x = tm0[tx], m1x = tm1[tx], md0x = tmd0[tx], md1x = tmd1[tx];
    const double m0y = tm0[ty], m1y = tm1[ty], md0y = tmd0[ty], md1y = tmd1[ty];
    const double zf0 = fa[8 * TPC + l], zf1 = fa[9 * TPC + l];
    const double zf2 = fa[10 * TPC + l], zf3 = fa[11 * TPC + l];
#pragma unroll
    for (int z = 0; z < N; z++) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < N; q++) {
        s += Bx[q] * ue[z * N2 + ty * N + q];
        s += By[q] * ue[z * N2 + q * N + tx];
        s += Bm[2 * N2 + z * N + q] * col[q];
      }
      const int lx = z * N + ty, ly = z * N + tx;
      s += m0x * fa[0 * TPC + lx];
      s += md0x * fa[1 * TPC + lx];
      s += m1x * fa[2 * TPC + lx];
      s += md1x * fa[3 * TPC + lx];
      s += m0y * fa[4 * TPC + ly];
      s += md0y * fa[5 * TPC + ly];
      s += m1y * fa[6 * TPC + ly];
      s += md1y * fa[7 * TPC + ly];
      s += tm0[z] * zf0;
      s += tmd0[z] * zf1;
      s += tm1[z] * zf2;
      s += tmd1[z] * zf3;
      Ss[z * N2 + l] = s;
    }
  }
  __syncthreads();
  // S1 = Mhat_x S (into ue: all reads of ue finished before the sync)
  double Mtx[N], Mty[N];
#pragma unroll
  for (int q = 0; q < N; q++) {
    Mtx[q] = tM[tx * N + q];
    Mty[q] = tM[ty * N + q];
  }
#pragma unroll
  for (int z = 0; z < N; z++) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < N; q++) s += Mtx[q] * Ss[z * N2 + ty * N + q];
    ue[z * N2 + l] = s;
  }
  __syncthreads();
  // S2 = Mhat_y S1 (own column), out = Mhat_z S2
  double s2c[N];
#pragma unroll
  for (int z = 0; z < N; z++) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < N; q++) s += Mty[q] * ue[z * N2 + q * N + tx];
    s2c[z] = s;
  }
  if (active) {
    double *ye = a.y + (size_t)e * NB;
    const double *ad = a.add ? a.add + (size_t)e * NB : nullptr;
    const bool scale = a.alpha != 1.0;
#pragma unroll
    for (int z = 0; z < N; z++) {
      double r = 0.0;
#pragma unroll
      for (int q = 0; q < N; q++) r += tM[z * N + q] * s2c[q];
      if (scale) r *= a.alpha;
      const int idx = z * TPC + l;
      if (a.accumulate) r += ye[idx];
      if (ad) r += ad[idx];
      ye[idx] = r;
    }
  }
}

template <int N>
static int record_m_n(pdg_context *ctx, int transpose) {
  using C = MCfg<N>;
  double *&out = transpose ? ctx->rec64mT : ctx->rec64m;
  if (!out) PDG_CUDA_TRY(cudaMalloc(&out, sizeof(double) * C::RECM * ctx->ncell));
  const unsigned blocks = (unsigned)((ctx->ncell + 127) / 128);
  k_record_m<N><<<blocks, 128, 0, ctx->stream>>>(ctx->ncell, ctx->rec64, ctx->tabm64 + C::TAB,
                                                 out, transpose);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// the records of the operator (transpose 0) or of its transpose (1), built
// once per coefficient field
int prepare_apply_m(pdg_context *ctx, int transpose) {
  int &valid = transpose ? ctx->rec64mT_valid : ctx->rec64m_valid;
  if (valid) return PDG_OK;
  if (!ctx->rec_valid || !ctx->tabm64)
    return set_error(PDG_EINVAL, "mass-factored records need the FP64 records and tables");
  int st;
  switch (ctx->N) {
    case 2: st = record_m_n<2>(ctx, transpose); break;
    case 3: st = record_m_n<3>(ctx, transpose); break;
    case 4: st = record_m_n<4>(ctx, transpose); break;
    case 5: st = record_m_n<5>(ctx, transpose); break;
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
  if (st == PDG_OK) valid = 1;
  return st;
}

template <int N>
static int launch_m_n(pdg_context *ctx, const ApplyArgs<double> &a, const OpParams<double> &p) {
  using C = MCfg<N>;
  const size_t smem = sizeof(double) * (C::TAB + C::CPB * C::PER_CELL);
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply_m<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_dev = ctx->device;
  }
  const long work = a.ncells > 0 ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  k_apply_m<N><<<blocks, C::THREADS, smem, ctx->stream>>>(
      p, a, a.transpose ? ctx->rec64mT : ctx->rec64m, ctx->tabm64);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int launch_apply_m(pdg_context *ctx, const ApplyArgs<double> &a, const OpParams<double> &p) {
  PDG_TRY(prepare_apply_m(ctx, a.transpose));
  switch (ctx->N) {
    case 2: return launch_m_n<2>(ctx, a, p);
    case 3: return launch_m_n<3>(ctx, a, p);
    case 4: return launch_m_n<4>(ctx, a, p);
    case 5: return launch_m_n<5>(ctx, a, p);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

}  // namespace pdg
