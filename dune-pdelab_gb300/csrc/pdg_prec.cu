// pdg_prec.cu -- cell-block Jacobi preconditioner.
//
// Reference: AssembledBlockJacobiPreconditionerLocalOperator
// (backend/istl/matrixfree/assembledblockjacobipreconditioner.hh:162-233):
// per cell, assemble the diagonal block D_e (volume + self part of every
// face + boundary faces, localoperator/blockdiagonalwrapper.hh:225-257),
// factor it (Eigen PartialPivLU) and apply D_e^{-1} per Krylov iteration.
//
// Two GPU forms:
//  * FDM (fast diagonalisation).  With A = K I, no convection and
//    axis-parallel cells, D_e is the Kronecker sum
//      D_e = A_x (x) M_y (x) M_z + M_x (x) A_y (x) M_z + M_x (x) M_y (x) A_z
//    (M_dir = h_dir Mhat; A_dir as in the operator kernel).  For symmetric
//    A_dir (SIPG) the generalised eigenproblems A_dir q = lambda M_dir q give
//    D_e^{-1} = (Qx (x) Qy (x) Qz) diag(1/(lx+ly+lz)) (Qx (x) Qy (x) Qz)^T,
//    exactly the inverse of the reference's block, at d(N^2+N) values per
//    cell instead of N^{2d}.
//  * DENSE.  The block D_e is built column by column with the operator
//    kernel restricted to the cell (neighbour coupling dropped, as
//    BlockDiagonalLocalOperatorWrapper::jacobian_apply_skeleton does with a
//    zero neighbour vector, blockdiagonalwrapper.hh:179-192) and inverted
//    with partial pivoting; the apply is a dense per-cell matvec.  Exact for
//    every block (non-symmetric methods, reaction, convection).
#include <cmath>
#include <cstdint>
#include <cuda_fp16.h>
#include <vector>

#include "pdg_ops.cuh"
#include "pdg_tma.cuh"
#include "pdg_vec.cuh"

namespace pdg {

// ---------------------------------------------------------------------------
// FDM setup: one thread per (cell, direction), FP64.
// ---------------------------------------------------------------------------
template <int N>
__global__ void k_fdm_setup(const OpParams<double> p, int dim, const double *__restrict__ Lhinv,
                            double *__restrict__ Qout, double *__restrict__ Lout,
                            float *__restrict__ Qout32, float *__restrict__ Lout32) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= p.ncell * dim) return;
  const long e = gid / dim;
  const int dir = (int)(gid - e * dim);
  const double *tM = p.tab, *tS = p.tab + N * N, *td0 = tS + N * N, *td1 = td0 + N;
  int ix[3];
  {
    long r = e;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  const long stride[3] = {1, (long)p.nc[0], (long)p.nc[0] * p.nc[1]};
  const double Ke = kdir(p, e, dir);
  const double cc = p.c ? p.c[e] : 0.0;
  double cf[18];
  for (int f = 2 * dir; f < 2 * dir + 2; f++) {
    const int d = f >> 1;
    long nb;
    if (f & 1) nb = ix[d] + 1 < p.nc[d] ? e + stride[d] : -1;
    else nb = ix[d] > 0 ? e - stride[d] : -1;
    face_coefficients(p, f, Ke, nb, cf + 3 * f);
  }
  double A[N][N];
  for (int i = 0; i < N; i++)
    for (int a = 0; a < N; a++) A[i][a] = a_entry<double, N>(p, dir, i, a, Ke, cc, cf, tM, tS, td0, td1);
  // C = (1/h) Lhinv A Lhinv^T
  const double h = p.h[dir];
  double Tm[N][N], C[N][N];
  for (int i = 0; i < N; i++)
    for (int a = 0; a < N; a++) {
      double s = 0.0;
      for (int q = 0; q < N; q++) s += Lhinv[i * N + q] * A[q][a];
      Tm[i][a] = s;
    }
  for (int i = 0; i < N; i++)
    for (int a = 0; a < N; a++) {
      double s = 0.0;
      for (int q = 0; q < N; q++) s += Tm[i][q] * Lhinv[a * N + q];
      C[i][a] = s / h;
    }
  // symmetrise (A is symmetric for SIPG; rounding only)
  for (int i = 0; i < N; i++)
    for (int a = i + 1; a < N; a++) {
      const double m = 0.5 * (C[i][a] + C[a][i]);
      C[i][a] = C[a][i] = m;
    }
  // cyclic Jacobi eigenvalue iteration: C = V diag V^T
  double V[N][N];
  for (int i = 0; i < N; i++)
    for (int a = 0; a < N; a++) V[i][a] = i == a ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < N; i++)
      for (int a = 0; a < N; a++) {
        tot += C[i][a] * C[i][a];
        if (i != a) off += C[i][a] * C[i][a];
      }
    if (off <= 1e-32 * tot) break;
    for (int pp = 0; pp < N - 1; pp++)
      for (int qq = pp + 1; qq < N; qq++) {
        const double apq = C[pp][qq];
        if (fabs(apq) < 1e-300) continue;
        const double theta = (C[qq][qq] - C[pp][pp]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < N; k++) {
          const double ckp = C[k][pp], ckq = C[k][qq];
          C[k][pp] = c * ckp - s * ckq;
          C[k][qq] = s * ckp + c * ckq;
        }
        for (int k = 0; k < N; k++) {
          const double cpk = C[pp][k], cqk = C[qq][k];
          C[pp][k] = c * cpk - s * cqk;
          C[qq][k] = s * cpk + c * cqk;
        }
        for (int k = 0; k < N; k++) {
          const double vkp = V[k][pp], vkq = V[k][qq];
          V[k][pp] = c * vkp - s * vkq;
          V[k][qq] = s * vkp + c * vkq;
        }
      }
  }
  // Q = (1/sqrt(h)) Lhinv^T V  (columns = M-orthonormal eigenvectors)
  const double rs = 1.0 / sqrt(h);
  const long qo = (e * dim + dir) * N * N, lo = (e * dim + dir) * N;
  for (int i = 0; i < N; i++)
    for (int a = 0; a < N; a++) {
      double s = 0.0;
      for (int q = 0; q < N; q++) s += Lhinv[q * N + i] * V[q][a];
      s *= rs;
      if (Qout) Qout[qo + i * N + a] = s;
      if (Qout32) Qout32[qo + i * N + a] = (float)s;
    }
  for (int a = 0; a < N; a++) {
    if (Lout) Lout[lo + a] = C[a][a];
    if (Lout32) Lout32[lo + a] = (float)C[a][a];
  }
}

// ---------------------------------------------------------------------------
// FDM apply: v = (Qx (x) Qy (x) Qz) diag(1/(lx+ly+lz)) (Qx (x) Qy (x) Qz)^T d
// ---------------------------------------------------------------------------
template <int D, int N>
struct PCfg {
  static constexpr int N2 = N * N;
  static constexpr int NB = D == 3 ? N * N * N : N * N;
  static constexpr int TPC = D == 3 ? N * N : N;
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  static constexpr int PER_CELL = 2 * NB + D * N2 + D * N;
};

// Padding (elements) of the per-cell shared region of k_fdm_apply that puts
// the cells sharing a warp on different shared-memory banks (chosen by
// counting the wavefronts of the kernel's shared accesses per padding).
template <typename T, int D, int N>
constexpr int fdm_pad() {
  if (D != 3) return 0;
  if (sizeof(T) == 4) return N == 2 ? 2 : N == 3 ? 15 : N == 4 ? 20 : N == 5 ? 5 : 0;
  return N == 2 ? 2 : N == 3 ? 2 : N == 5 ? 5 : 0;
}

// 1 / (Lx[x] + Ly[y] (+ Lz[z])) per DOF (local index x fastest), FP64
__global__ void k_fdm_lsum_inv(long ndof, int dim, int N, const double *__restrict__ L,
                               double *__restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ndof) return;
  const int nb = dim == 3 ? N * N * N : N * N;
  const long e = i / nb;
  const int k = (int)(i - e * nb);
  const double *l = L + e * dim * N;
  double s = l[k % N] + l[N + (k / N) % N];
  if (dim == 3) s += l[2 * N + k / (N * N)];
  out[i] = 1.0 / s;
}

template <typename T, int D, int N>
__global__ void __launch_bounds__(PCfg<D, N>::THREADS)
    k_fdm_apply(long ncell, const T *__restrict__ Q, const T *__restrict__ L, T *d, T *v,
                const int *__restrict__ skip, const int *__restrict__ cells, int ncells, T scale,
                double *dot_part, long dot_max_blocks, int *dot_cnt, double *dot_scal,
                int *dot_flags, int dot_fin, const T *rq, const T *__restrict__ Linv) {
  // rq != null (fused CG): first d -= lambda rq (lambda = dot_scal[S_ALPHA]),
  // written back; the fused dot then carries |d|^2 and <d, v>.  d, v and rq
  // may alias element-wise: every entry is read and written by one thread.
  using C = PCfg<D, N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB;
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, cs = t / TPC, l = t - cs * TPC;
  T *S0 = reinterpret_cast<T *>(smem_raw) + cs * (C::PER_CELL + fdm_pad<T, D, N>());
  T *S1 = S0 + NB;
  T *Qs = S1 + NB;       // [D][N2]
  T *Ls = Qs + D * N2;   // [D][N]
  const int li = blockIdx.x * CPB + cs;
  const bool active = cells ? li < ncells : li < ncell;
  const int e = cells ? (active ? cells[li] : 0) : li;
  const int ee = active ? e : 0;
  for (int i = l; i < D * N2; i += TPC) Qs[i] = Q[(size_t)ee * D * N2 + i];
  for (int i = l; i < D * N; i += TPC) Ls[i] = L[(size_t)ee * D * N + i];
  T col[N];
#pragma unroll
  for (int z = 0; z < N; z++) col[z] = d[(size_t)ee * NB + z * TPC + l];
  T part = T(0), part2 = T(0);   // <d, v> (and |d|^2) of this thread's entries
  if (rq) {
    const T lambda = (T)dot_scal[S_ALPHA];
#pragma unroll
    for (int z = 0; z < N; z++) {
      const size_t i = (size_t)ee * NB + z * TPC + l;
      col[z] -= lambda * rq[i];
      if (active) d[i] = col[z];
      part2 += col[z] * col[z];
    }
    if (!active) part2 = T(0);
  }
  __syncthreads();
  if constexpr (D == 3) {
    const int tx = l % N, ty = l / N;
    const T *Qx = Qs, *Qy = Qs + N2, *Qz = Qs + 2 * N2;
    // z (registers): a[z'] = sum_z Qz[z][z'] col[z]
    T a[N];
#pragma unroll
    for (int zp = 0; zp < N; zp++) {
      T s = T(0);
#pragma unroll
      for (int z = 0; z < N; z++) s += Qz[z * N + zp] * col[z];
      a[zp] = s;
    }
#pragma unroll
    for (int z = 0; z < N; z++) S0[z * N2 + l] = a[z];
    __syncthreads();
    // y: b[z][ty'] = sum_y Qy[y][ty'] a[z][y][tx]
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int y = 0; y < N; y++) s += Qy[y * N + ty] * S0[z * N2 + y * N + tx];
      S1[z * N2 + l] = s;
    }
    __syncthreads();
    // x + scaling: c[z][ty][tx'] = sum_x Qx[x][tx'] b[z][ty][x] / (lx+ly+lz)
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int x = 0; x < N; x++) s += Qx[x * N + tx] * S1[z * N2 + ty * N + x];
      a[z] = Linv ? s * Linv[(size_t)ee * NB + z * N2 + l]
                  : qdiv(s, Ls[tx] + Ls[N + ty] + Ls[2 * N + z]);
    }
    __syncthreads();
#pragma unroll
    for (int z = 0; z < N; z++) S0[z * N2 + l] = a[z];
    __syncthreads();
    // back x: e[z][ty][tx] = sum_x' Qx[tx][x'] c[z][ty][x']
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int x = 0; x < N; x++) s += Qx[tx * N + x] * S0[z * N2 + ty * N + x];
      S1[z * N2 + l] = s;
    }
    __syncthreads();
    // back y
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int y = 0; y < N; y++) s += Qy[ty * N + y] * S1[z * N2 + y * N + tx];
      a[z] = s;
    }
    // back z (registers)
    if (active) {
#pragma unroll
      for (int z = 0; z < N; z++) {
        T s = T(0);
#pragma unroll
        for (int zp = 0; zp < N; zp++) s += Qz[z * N + zp] * a[zp];
        v[(size_t)e * NB + z * N2 + l] = scale * s;
        part += col[z] * (scale * s);
      }
    }
  } else {
    const int tx = l;
    const T *Qx = Qs, *Qy = Qs + N2;
    T a[N];
#pragma unroll
    for (int yp = 0; yp < N; yp++) {
      T s = T(0);
#pragma unroll
      for (int y = 0; y < N; y++) s += Qy[y * N + yp] * col[y];
      a[yp] = s;
    }
#pragma unroll
    for (int y = 0; y < N; y++) S0[y * N + tx] = a[y];
    __syncthreads();
#pragma unroll
    for (int y = 0; y < N; y++) {
      T s = T(0);
#pragma unroll
      for (int x = 0; x < N; x++) s += Qx[x * N + tx] * S0[y * N + x];
      a[y] = Linv ? s * Linv[(size_t)ee * NB + y * N + tx] : qdiv(s, Ls[tx] + Ls[N + y]);
    }
#pragma unroll
    for (int y = 0; y < N; y++) S1[y * N + tx] = a[y];
    __syncthreads();
#pragma unroll
    for (int y = 0; y < N; y++) {
      T s = T(0);
#pragma unroll
      for (int x = 0; x < N; x++) s += Qx[tx * N + x] * S1[y * N + x];
      a[y] = s;
    }
    if (active) {
#pragma unroll
      for (int y = 0; y < N; y++) {
        T s = T(0);
#pragma unroll
        for (int yp = 0; yp < N; yp++) s += Qy[y * N + yp] * a[yp];
        v[(size_t)e * NB + y * N + tx] = scale * s;
        part += col[y] * (scale * s);
      }
    }
  }
  if (dot_part) {
    // FIN_CG_DEF_BETA takes (|d|^2, <d, v>); the plain fused dot (<d, v>)
    double s0 = (double)part, s1 = 0.0;
    if (rq) {
      s0 = (double)part2;
      s1 = (double)part;
    }
    reduce_tail_grouped<C::THREADS>(dot_part, dot_max_blocks, dot_cnt,
                                    RedCtx{nullptr, dot_scal, dot_flags}, s0, s1, dot_fin, -1,
                                    -1);
  }
}

// ---------------------------------------------------------------------------
// DENSE: block columns, Gauss-Jordan inversion, matvec apply
// ---------------------------------------------------------------------------
__global__ void k_unit_field(long ncell, int nb, int j, double *__restrict__ x) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncell * nb) x[i] = (i % nb) == j ? 1.0 : 0.0;
}
// D[e][i][j] = y[e][i]   (row-major blocks)
__global__ void k_scatter_col(long ncell, int nb, int j, const double *__restrict__ y,
                              double *__restrict__ D) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncell * nb) return;
  const long e = i / nb;
  const int r = (int)(i - e * nb);
  D[(e * nb + r) * nb + j] = y[i];
}

// In-place Gauss-Jordan inversion with row partial pivoting of one nb x nb
// block per CTA (FP64 in shared memory, nb*nb + 2 nb values).  The column
// permutation is undone at the end.  Writes the inverse transposed
// (column-major) in precision T so that the apply reads it coalesced.
// Singular blocks leave a zero inverse and raise *bad.
template <typename T>
__global__ void k_invert(int nb, const double *__restrict__ D, T *__restrict__ invT,
                         int *__restrict__ bad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *A = reinterpret_cast<double *>(smem_raw);   // [nb][nb]
  double *fcol = A + nb * nb;                         // [nb]
  int *perm = reinterpret_cast<int *>(fcol + nb);     // [nb]
  __shared__ int piv;
  __shared__ double pval;
  const long e = blockIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  for (int i = t; i < nb * nb; i += nt) A[i] = D[e * nb * nb + i];
  __syncthreads();
  bool singular = false;
  for (int c = 0; c < nb; c++) {
    if (t == 0) {
      int pr = c;
      double best = fabs(A[c * nb + c]);
      for (int r = c + 1; r < nb; r++) {
        const double v = fabs(A[r * nb + c]);
        if (v > best) { best = v; pr = r; }
      }
      piv = pr;
      pval = A[pr * nb + c];
      perm[c] = pr;
    }
    __syncthreads();
    if (pval == 0.0) { singular = true; break; }
    const int pr = piv;
    if (pr != c)
      for (int j = t; j < nb; j += nt) {
        const double tmp = A[c * nb + j];
        A[c * nb + j] = A[pr * nb + j];
        A[pr * nb + j] = tmp;
      }
    __syncthreads();
    const double inv = 1.0 / pval;
    for (int j = t; j < nb; j += nt) A[c * nb + j] = j == c ? inv : A[c * nb + j] * inv;
    for (int r = t; r < nb; r += nt) fcol[r] = r == c ? 0.0 : A[r * nb + c];
    __syncthreads();
    for (int i = t; i < nb * nb; i += nt) {
      const int r = i / nb, j = i - r * nb;
      if (r == c) continue;
      const double base = j == c ? 0.0 : A[i];
      A[i] = base - fcol[r] * A[c * nb + j];
    }
    __syncthreads();
  }
  if (singular) {
    if (t == 0) atomicExch(bad, 1);
    for (int i = t; i < nb * nb; i += nt) invT[e * nb * nb + i] = T(0);
    return;
  }
  // undo the row interchanges as column interchanges, last first
  for (int c = nb - 1; c >= 0; c--) {
    const int pc = perm[c];
    if (pc != c)
      for (int r = t; r < nb; r += nt) {
        const double tmp = A[r * nb + c];
        A[r * nb + c] = A[r * nb + pc];
        A[r * nb + pc] = tmp;
      }
    __syncthreads();
  }
  // invT[e][j][i] = Inv[i][j]
  for (int i = t; i < nb * nb; i += nt) {
    const int j = i / nb, r = i % nb;
    invT[e * nb * nb + i] = (T)A[r * nb + j];
  }
}

// v_e = Inv_e d_e (transpose: v_e = Inv_e^T d_e), one warp-multiple of
// threads per cell, d_e staged in shared memory.
template <typename T>
__global__ void k_dense_apply(long ncell, int nb, const T *__restrict__ invT,
                              const T *__restrict__ d, T *__restrict__ v, int transpose,
                              const int *__restrict__ skip, const int *__restrict__ cells,
                              T scale) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *ds = reinterpret_cast<T *>(smem_raw);
  const long e = cells ? (long)cells[blockIdx.x] : (long)blockIdx.x;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) ds[i] = d[e * nb + i];
  __syncthreads();
  const T *B = invT + e * (long)nb * nb;
  if (!transpose) {
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      T s = T(0);
      for (int j = 0; j < nb; j++) s += B[j * nb + i] * ds[j];
      v[e * nb + i] = scale * s;
    }
  } else {
    // v_i = sum_j B[i nb + j] d_j (column i contiguous): one warp per output,
    // lanes over j, warp sum
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int i = warp; i < nb; i += nwarps) {
      T s = T(0);
      for (int j = lane; j < nb; j += 32) s += B[i * nb + j] * ds[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) v[e * nb + i] = scale * s;
    }
  }
}

// FP16 copy of the FP32 block inverses: per block the largest magnitude as
// an FP32 scale, entries divided by it and rounded to FP16 (relative rounding
// 2^-11 of the block's largest entry).  Columns are padded to nbp = nb rounded
// up to 4 entries (zeros), so four rows of a column are one 8-byte load.  One
// block per CTA.
__global__ void k_inv_to_half(int nb, int nbp, const float *__restrict__ inv,
                              __half *__restrict__ inv16, float *__restrict__ scale) {
  __shared__ float red[32];
  const long e = blockIdx.x;
  const long n2 = (long)nb * nb;
  const float *B = inv + e * n2;
  float m = 0.f;
  for (long i = threadIdx.x; i < n2; i += blockDim.x) m = fmaxf(m, fabsf(B[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) red[0] = m;
  }
  __syncthreads();
  const float s = red[0] > 0.f ? red[0] : 1.f;
  const float is = 1.f / s;
  __half *O = inv16 + e * (long)nb * nbp;
  for (long k = threadIdx.x; k < (long)nb * nbp; k += blockDim.x) {
    const int j = (int)(k / nbp), i = (int)(k - (long)j * nbp);
    O[k] = __float2half_rn(i < nb ? B[(long)j * nb + i] * is : 0.f);
  }
  if (threadIdx.x == 0) scale[e] = s;
}

// v = scale * s_e * B16_e d  (B16 column-major with column stride nbp, FP16),
// FP32 vectors.  Thread (rg, jg): rows 4rg..4rg+3 over the columns j = jg mod
// JG, one 8-byte load per column; the JG partial sums of a row are added in
// shared memory.  The transposed apply reads rows of B^T (columns of B) with
// scalar loads.
constexpr int kDenseH = 128;   // threads per block of the FP16 apply
__global__ void __launch_bounds__(kDenseH)
    k_dense_apply_h(long ncell, int nb, int nbp, const __half *__restrict__ inv16,
                    const float *__restrict__ bscale, const float *__restrict__ d,
                    float *__restrict__ v, int transpose, const int *__restrict__ skip,
                    const int *__restrict__ cells, float scale) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *ds = reinterpret_cast<float *>(smem_raw);   // [nb]
  float *part = ds + nbp;                             // [JG][nbp]
  const long e = cells ? (long)cells[blockIdx.x] : (long)blockIdx.x;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) ds[i] = d[e * nb + i];
  __syncthreads();
  const __half *B = inv16 + e * (long)nb * nbp;
  const float sc = scale * bscale[e];
  if (!transpose) {
    const int ngroups = nbp / 4;                  // row groups
    const int JG = blockDim.x / ngroups;          // column subsets (>= 1)
    const int rg = threadIdx.x % ngroups, jg = threadIdx.x / ngroups;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    if (jg < JG) {
      for (int j = jg; j < nb; j += JG) {
        const uint2 w = *reinterpret_cast<const uint2 *>(B + (long)j * nbp + 4 * rg);
        const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&w.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&w.y));
        const float dj = ds[j];
        s0 += a.x * dj; s1 += a.y * dj; s2 += b.x * dj; s3 += b.y * dj;
      }
      float *pp = part + jg * nbp + 4 * rg;
      pp[0] = s0; pp[1] = s1; pp[2] = s2; pp[3] = s3;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      float r = 0.f;
      for (int g = 0; g < JG; g++) r += part[g * nbp + i];
      v[e * nb + i] = sc * r;
    }
  } else {
    // v_i = sum_j B16[i nbp + j] d_j: one warp per output, each lane four
    // consecutive j per 8-byte load (column i is contiguous), warp sum
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int i = warp; i < nb; i += nwarps) {
      float r = 0.f;
      for (int j = 4 * lane; j < nb; j += 128) {
        const uint2 w = *reinterpret_cast<const uint2 *>(B + (long)i * nbp + j);
        const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&w.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&w.y));
        r += a.x * ds[j];
        if (j + 1 < nb) r += a.y * ds[j + 1];
        if (j + 2 < nb) r += b.x * ds[j + 2];
        if (j + 3 < nb) r += b.y * ds[j + 3];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
      if (lane == 0) v[e * nb + i] = sc * r;
    }
  }
}


// ---------------------------------------------------------------------------
// FDM apply, 3D Q3 FP32 (the inner solves of the mixed-precision CG): one
// z-plane of one cell per thread.  The x and y contractions of the plane run in
// registers; the two z contractions go through one shared exchange buffer of
// 16-byte rows with the operator's row swizzle (conflict-free for a quarter warp
// of two cells x four planes).  d and, with the fused CG residual update, q are
// staged with coalesced 16-byte copies; the update b -= lambda q runs as one
// coalesced pass before the plane work.  Same fused dot products as k_fdm_apply.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int fswz(int r) { return r ^ (((r >> 3) & 1) | (((r >> 4) & 1) << 1)); }

struct FdmQ3Cfg {
  static constexpr int N = 4, NB = 64, CPB = 32, THREADS = 128;
  static constexpr int RUN = CPB * 16;               // 16-byte rows of a run of cells
  // factor rows per cell: 12 (Qx, Qy, Qz), stored with a stride of 13 so that
  // the scalar factor reads of the cells sharing a warp fall on distinct banks
  static constexpr int QSTRIDE = 13;
  static constexpr int QROWS = CPB * QSTRIDE, LROWS = CPB * 3;
  static constexpr int ROWS = 2 * RUN + QROWS + LROWS;
};

__global__ void __launch_bounds__(FdmQ3Cfg::THREADS)
    k_fdm32_q3(long ncell, const float *__restrict__ Q, const float *__restrict__ L, float *d,
               float *v, const int *__restrict__ skip, float scale, double *dot_part,
               long dot_max_blocks, int *dot_cnt, double *dot_scal, int *dot_flags, int dot_fin,
               const float *rq) {
  using C = FdmQ3Cfg;
  constexpr int N = 4, NB = 64, CPB = C::CPB;
  extern __shared__ __align__(16) float4 fsm[];
  if (skip && *skip) return;
  float4 *DR = fsm;                     // d (then b - lambda q) of the run, swizzled
  float4 *PR = DR + C::RUN;             // q of the run, then the z-exchange planes
  float4 *QS = PR + C::RUN;             // factors Q [cell][dir][4 rows]
  float4 *LS = QS + C::QROWS;           // eigenvalues L [cell][dir]
  const long e0 = (long)blockIdx.x * CPB;
  const long ndof = ncell * NB;
  const bool vec = ((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(v) |
                     reinterpret_cast<uintptr_t>(rq)) & 15) == 0;
  auto cp16 = [](float4 *dst, const float *src) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
  };
  for (int r = threadIdx.x; r < C::RUN; r += C::THREADS) {
    const long g = e0 * NB + 4L * r;
    float4 *dd = DR + fswz(r), *dq = PR + fswz(r);
    if (g < ndof) {
      if (vec) {
        cp16(dd, d + g);
        if (rq) cp16(dq, rq + g);
      } else {
        *dd = make_float4(d[g], d[g + 1], d[g + 2], d[g + 3]);
        if (rq) *dq = make_float4(rq[g], rq[g + 1], rq[g + 2], rq[g + 3]);
      }
    } else {
      *dd = make_float4(0.f, 0.f, 0.f, 0.f);
      *dq = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  // factors: contiguous runs, 16-byte aligned (48 and 12 floats per cell, 32 cells)
  const long cmax = ncell - e0 < CPB ? ncell - e0 : CPB;
  for (int r = threadIdx.x; r < CPB * 12; r += C::THREADS) {
    float4 *dst = QS + (r / 12) * C::QSTRIDE + r % 12;
    if (r < cmax * 12) cp16(dst, Q + e0 * 48 + 4L * r);
    else *dst = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int r = threadIdx.x; r < C::LROWS; r += C::THREADS) {
    if (r < cmax * 3) cp16(LS + r, L + e0 * 12 + 4L * r);
    else LS[r] = make_float4(1.f, 1.f, 1.f, 1.f);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  float part2 = 0.f;   // |b - lambda q|^2 (fused CG residual update)
  if (rq) {
    const float lambda = (float)dot_scal[S_ALPHA];
    for (int r = threadIdx.x; r < C::RUN; r += C::THREADS) {
      const long g = e0 * NB + 4L * r;
      if (g >= ndof) break;
      const float4 a = DR[fswz(r)], q = PR[fswz(r)];
      const float4 b = make_float4(a.x - lambda * q.x, a.y - lambda * q.y, a.z - lambda * q.z,
                                   a.w - lambda * q.w);
      DR[fswz(r)] = b;
      if (vec) *reinterpret_cast<float4 *>(d + g) = b;
      else { d[g] = b.x; d[g + 1] = b.y; d[g + 2] = b.z; d[g + 3] = b.w; }
      part2 += b.x * b.x + b.y * b.y + b.z * b.z + b.w * b.w;
    }
    __syncthreads();
  }

  const int t = threadIdx.x, cs = t >> 2, z = t & 3;
  const float4 *Qc = QS + cs * C::QSTRIDE;   // Qx rows 0..3, Qy rows 4..7, Qz rows 8..11
  auto el = [](const float4 &w, int i) -> float {
    return i == 0 ? w.x : (i == 1 ? w.y : (i == 2 ? w.z : w.w));
  };
  float u[N][N];
#pragma unroll
  for (int y = 0; y < N; y++) {
    const float4 w = DR[fswz(cs * 16 + z * 4 + y)];
    u[y][0] = w.x; u[y][1] = w.y; u[y][2] = w.z; u[y][3] = w.w;
  }
  // forward x then y (registers): w[y'][x'] = sum_y Qy[y][y'] sum_x Qx[x][x'] u[y][x]
  {
    float t1[N][N];
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xp = 0; xp < N; xp++) {
        float s = 0.f;
#pragma unroll
        for (int x = 0; x < N; x++) s += el(Qc[x], xp) * u[y][x];
        t1[y][xp] = s;
      }
#pragma unroll
    for (int yp = 0; yp < N; yp++)
#pragma unroll
      for (int xp = 0; xp < N; xp++) {
        float s = 0.f;
#pragma unroll
        for (int y = 0; y < N; y++) s += el(Qc[4 + y], yp) * t1[y][xp];
        u[yp][xp] = s;
      }
  }
#pragma unroll
  for (int y = 0; y < N; y++) PR[fswz(cs * 16 + z * 4 + y)] = make_float4(u[y][0], u[y][1], u[y][2], u[y][3]);
  __syncthreads();
  // forward z + scaling: c_z'[y][x] = sum_z Qz[z][z'] w_z[y][x] / (Lx[x] + Ly[y] + Lz[z'])
  {
    float qzc[N];
#pragma unroll
    for (int zz = 0; zz < N; zz++) qzc[zz] = el(Qc[8 + zz], z);
    const float4 lx = LS[cs * 3], ly = LS[cs * 3 + 1];
    const float lz = el(LS[cs * 3 + 2], z);
#pragma unroll
    for (int y = 0; y < N; y++) {
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int zz = 0; zz < N; zz++) {
        const float4 w = PR[fswz(cs * 16 + zz * 4 + y)];
        acc.x += qzc[zz] * w.x; acc.y += qzc[zz] * w.y; acc.z += qzc[zz] * w.z; acc.w += qzc[zz] * w.w;
      }
      const float lyz = el(ly, y) + lz;
      u[y][0] = __fdividef(acc.x, lx.x + lyz);
      u[y][1] = __fdividef(acc.y, lx.y + lyz);
      u[y][2] = __fdividef(acc.z, lx.z + lyz);
      u[y][3] = __fdividef(acc.w, lx.w + lyz);
    }
  }
  __syncthreads();
#pragma unroll
  for (int y = 0; y < N; y++) PR[fswz(cs * 16 + z * 4 + y)] = make_float4(u[y][0], u[y][1], u[y][2], u[y][3]);
  __syncthreads();
  // backward z: e_z[y][x] = sum_z' Qz[z][z'] c_z'[y][x]
  {
    const float4 qzr = Qc[8 + z];
#pragma unroll
    for (int y = 0; y < N; y++) {
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int zz = 0; zz < N; zz++) {
        const float4 w = PR[fswz(cs * 16 + zz * 4 + y)];
        const float qq = el(qzr, zz);
        acc.x += qq * w.x; acc.y += qq * w.y; acc.z += qq * w.z; acc.w += qq * w.w;
      }
      u[y][0] = acc.x; u[y][1] = acc.y; u[y][2] = acc.z; u[y][3] = acc.w;
    }
  }
  // backward y then x (registers): g[y][x] = sum_x' Qx[x][x'] sum_y' Qy[y][y'] e[y'][x']
  float g[N][N];
  {
    float t1[N][N];
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int x = 0; x < N; x++) {
        float s = 0.f;
#pragma unroll
        for (int yp = 0; yp < N; yp++) s += el(Qc[4 + y], yp) * u[yp][x];
        t1[y][x] = s;
      }
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int x = 0; x < N; x++) {
        float s = 0.f;
#pragma unroll
        for (int xp = 0; xp < N; xp++) s += el(Qc[x], xp) * t1[y][xp];
        g[y][x] = s;
      }
  }
  // coalesced write-back through the exchange buffer; fused <d, v>
  __syncthreads();
#pragma unroll
  for (int y = 0; y < N; y++) PR[fswz(cs * 16 + z * 4 + y)] = make_float4(g[y][0], g[y][1], g[y][2], g[y][3]);
  __syncthreads();
  float part = 0.f;
  for (int r = threadIdx.x; r < C::RUN; r += C::THREADS) {
    const long gi = e0 * NB + 4L * r;
    if (gi >= ndof) break;
    const float4 o = PR[fswz(r)], dd = DR[fswz(r)];
    const float4 w = make_float4(scale * o.x, scale * o.y, scale * o.z, scale * o.w);
    if (vec) *reinterpret_cast<float4 *>(v + gi) = w;
    else { v[gi] = w.x; v[gi + 1] = w.y; v[gi + 2] = w.z; v[gi + 3] = w.w; }
    part += dd.x * w.x + dd.y * w.y + dd.z * w.z + dd.w * w.w;
  }
  if (dot_part) {
    double s0 = (double)part, s1 = 0.0;
    if (rq) {
      s0 = (double)part2;
      s1 = (double)part;
    }
    reduce_tail_grouped<C::THREADS>(dot_part, dot_max_blocks, dot_cnt,
                                    RedCtx{nullptr, dot_scal, dot_flags}, s0, s1, dot_fin, -1, -1);
  }
}

// ---------------------------------------------------------------------------
// The same FDM apply with TMA staging and paired FP32 arithmetic (16-byte
// aligned d and q): the runs of d and q arrive as 128-byte-swizzled tensor
// copies and the factors as bulk copies, all on one mbarrier (bounded wait);
// each thread reads its plane rows at closed-form swizzled addresses, keeps
// b = d - lambda q in registers, writes b and its own plane of v with 32-byte
// stores, and runs every contraction as paired multiply-adds (one issue for
// two lanes).  The two z exchanges reuse the q run's swizzled rows: a thread
// rewrites exactly the rows it read.
// ---------------------------------------------------------------------------
struct FdmQ3T {
  static constexpr int CPB = 32, THREADS = 128;
  static constexpr int DR_B = 0, QR_B = 8192, QS_B = 16384, LS_B = QS_B + CPB * 192,
                       END = LS_B + CPB * 48;
  static constexpr int SMEM = 1024 + END;
};

__global__ void __launch_bounds__(FdmQ3T::THREADS)
    k_fdm32_q3t(long ncell, const float *__restrict__ Q, const float *__restrict__ L, float *d,
                float *v, const int *__restrict__ skip, float scale, double *dot_part,
                long dot_max_blocks, int *dot_cnt, double *dot_scal, int *dot_flags, int dot_fin,
                const float *rq, const __grid_constant__ CUtensorMap map_d,
                const __grid_constant__ CUtensorMap map_q, int *tma_err) {
  using C = FdmQ3T;
  constexpr int N = 4, NB = 64, CPB = C::CPB;
  extern __shared__ __align__(16) unsigned char fsraw[];
  __shared__ __align__(8) unsigned long long fbar;
  if (skip && *skip) return;
  unsigned char *base = fsraw + ((1024u - (smem_u32(fsraw) & 1023u)) & 1023u);
  const long e0 = (long)blockIdx.x * CPB;
  const long cmax = ncell - e0 < CPB ? ncell - e0 : CPB;
  {
    const unsigned bar = smem_u32(&fbar);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned fb = (unsigned)(cmax * 240);
      mbar_expect_tx(bar, (rq ? 2u : 1u) * kLinesRun * 128u + fb);
      tma_load_2d(smem_u32(base + C::DR_B), &map_d, 0, (int)(e0 * 2), bar);
      if (rq) tma_load_2d(smem_u32(base + C::QR_B), &map_q, 0, (int)(e0 * 2), bar);
      bulk_load(smem_u32(base + C::QS_B), Q + e0 * 48, (unsigned)(cmax * 192), bar);
      bulk_load(smem_u32(base + C::LS_B), L + e0 * 12, (unsigned)(cmax * 48), bar);
    }
    if (!mbar_wait(bar, 0, kTmaPolls)) {
      if (threadIdx.x == 0) atomicExch(tma_err, 1);
      mbar_wait(bar, 0, kTmaPolls);
      return;
    }
  }
  const int cs = threadIdx.x >> 2, z = threadIdx.x & 3;
  const long e = e0 + cs;
  const bool active = cs < cmax;
  const unsigned char *F = base + C::QS_B + cs * 192;   // Qx rows 0..3, Qy 4..7, Qz 8..11
  const float4 lx = sh4(base + C::LS_B, cs * 48u), ly = sh4(base + C::LS_B, cs * 48u + 16u);
  const float lz = f4c(sh4(base + C::LS_B, cs * 48u + 32u), z);
  unsigned char *X = base + C::QR_B;

  // b (= d, or d - lambda q with the fused residual update), own plane
  float2 b[N][2];
#pragma unroll
  for (int y = 0; y < N; y++) {
    const float4 w = sh4(base + C::DR_B, q3_swz_row(cs, z, y));
    b[y][0] = make_float2(w.x, w.y);
    b[y][1] = make_float2(w.z, w.w);
  }
  float part2 = 0.f;   // |b - lambda q|^2
  const bool v32 = ((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(v)) & 31) == 0;
  if (rq) {
    const float2 ml = bc2(-(float)dot_scal[S_ALPHA]);
#pragma unroll
    for (int y = 0; y < N; y++) {
      const float4 q = sh4(X, q3_swz_row(cs, z, y));
      b[y][0] = ffma2(ml, make_float2(q.x, q.y), b[y][0]);
      b[y][1] = ffma2(ml, make_float2(q.z, q.w), b[y][1]);
    }
    float w[16];
#pragma unroll
    for (int y = 0; y < N; y++) {
      w[4 * y] = b[y][0].x; w[4 * y + 1] = b[y][0].y;
      w[4 * y + 2] = b[y][1].x; w[4 * y + 3] = b[y][1].y;
    }
#pragma unroll
    for (int j = 0; j < 16; j++) part2 += w[j] * w[j];
    if (active) {
      float *dp = d + e * NB + z * 16;
      if (v32) {
        st8(dp, w);
        st8(dp + 8, w + 8);
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++) dp[j] = w[j];
      }
    } else {
      part2 = 0.f;
    }
  }

  float2 u[N][2];
  {
    // forward x then y: w[y'][x'] = sum_y Qy[y][y'] sum_x Qx[x][x'] b[y][x]
    float2 t1[N][2];
#pragma unroll
    for (int y = 0; y < N; y++) {
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int x = 0; x < N; x++) {
        const float4 qx = sh4(F, 16u * x);
        const float bx = f4c(make_float4(b[y][0].x, b[y][0].y, b[y][1].x, b[y][1].y), x);
        a0 = ffma2(make_float2(qx.x, qx.y), bc2(bx), a0);
        a1 = ffma2(make_float2(qx.z, qx.w), bc2(bx), a1);
      }
      t1[y][0] = a0;
      t1[y][1] = a1;
    }
#pragma unroll
    for (int yp = 0; yp < N; yp++) {
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int y = 0; y < N; y++) {
        const float qy = f4c(sh4(F, 64u + 16u * y), yp);
        a0 = ffma2(bc2(qy), t1[y][0], a0);
        a1 = ffma2(bc2(qy), t1[y][1], a1);
      }
      u[yp][0] = a0;
      u[yp][1] = a1;
    }
  }
#pragma unroll
  for (int y = 0; y < N; y++)
    st4(X, q3_swz_row(cs, z, y), make_float4(u[y][0].x, u[y][0].y, u[y][1].x, u[y][1].y));
  __syncthreads();
  // forward z and scaling: c_z'[y][x] = sum_z Qz[z][z'] w_z[y][x] / (Lx[x] + Ly[y] + Lz[z'])
  {
    float qzc[N];
#pragma unroll
    for (int zz = 0; zz < N; zz++) qzc[zz] = f4c(sh4(F, 128u + 16u * zz), z);
#pragma unroll
    for (int y = 0; y < N; y++) {
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int zz = 0; zz < N; zz++) {
        const float4 w = sh4(X, q3_swz_row(cs, zz, y));
        a0 = ffma2(bc2(qzc[zz]), make_float2(w.x, w.y), a0);
        a1 = ffma2(bc2(qzc[zz]), make_float2(w.z, w.w), a1);
      }
      const float lyz = f4c(ly, y) + lz;
      u[y][0] = make_float2(__fdividef(a0.x, lx.x + lyz), __fdividef(a0.y, lx.y + lyz));
      u[y][1] = make_float2(__fdividef(a1.x, lx.z + lyz), __fdividef(a1.y, lx.w + lyz));
    }
  }
  __syncthreads();
#pragma unroll
  for (int y = 0; y < N; y++)
    st4(X, q3_swz_row(cs, z, y), make_float4(u[y][0].x, u[y][0].y, u[y][1].x, u[y][1].y));
  __syncthreads();
  // backward z: e_z[y][x] = sum_z' Qz[z][z'] c_z'[y][x]
  {
    const float4 qzr = sh4(F, 128u + 16u * z);
#pragma unroll
    for (int y = 0; y < N; y++) {
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int zz = 0; zz < N; zz++) {
        const float4 w = sh4(X, q3_swz_row(cs, zz, y));
        a0 = ffma2(bc2(f4c(qzr, zz)), make_float2(w.x, w.y), a0);
        a1 = ffma2(bc2(f4c(qzr, zz)), make_float2(w.z, w.w), a1);
      }
      u[y][0] = a0;
      u[y][1] = a1;
    }
  }
  // backward y then x: g[y][x] = sum_x' Qx[x][x'] sum_y' Qy[y][y'] e[y'][x']
  float g[16];
  {
    float2 t1[N][2];
#pragma unroll
    for (int y = 0; y < N; y++) {
      const float4 qy = sh4(F, 64u + 16u * y);
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int yp = 0; yp < N; yp++) {
        a0 = ffma2(bc2(f4c(qy, yp)), u[yp][0], a0);
        a1 = ffma2(bc2(f4c(qy, yp)), u[yp][1], a1);
      }
      t1[y][0] = a0;
      t1[y][1] = a1;
    }
    const float4 q0 = sh4(F, 0u), q1 = sh4(F, 16u), q2 = sh4(F, 32u), q3 = sh4(F, 48u);
#pragma unroll
    for (int y = 0; y < N; y++) {
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int xp = 0; xp < N; xp++) {
        const float tv = xp < 2 ? (xp == 0 ? t1[y][0].x : t1[y][0].y)
                                : (xp == 2 ? t1[y][1].x : t1[y][1].y);
        a0 = ffma2(make_float2(f4c(q0, xp), f4c(q1, xp)), bc2(tv), a0);
        a1 = ffma2(make_float2(f4c(q2, xp), f4c(q3, xp)), bc2(tv), a1);
      }
      const float2 s0 = fmul2(bc2(scale), a0), s1 = fmul2(bc2(scale), a1);
      g[4 * y] = s0.x; g[4 * y + 1] = s0.y; g[4 * y + 2] = s1.x; g[4 * y + 3] = s1.y;
    }
  }
  // own plane of v; fused <b, v>
  float part = 0.f;
  if (active) {
    float *vp = v + e * NB + z * 16;
    if (v32) {
      st8(vp, g);
      st8(vp + 8, g + 8);
    } else {
#pragma unroll
      for (int j = 0; j < 16; j++) vp[j] = g[j];
    }
#pragma unroll
    for (int y = 0; y < N; y++)
      part += b[y][0].x * g[4 * y] + b[y][0].y * g[4 * y + 1] + b[y][1].x * g[4 * y + 2] +
              b[y][1].y * g[4 * y + 3];
  }
  if (dot_part) {
    double s0 = (double)part, s1 = 0.0;
    if (rq) {
      s0 = (double)part2;
      s1 = (double)part;
    }
    reduce_tail_grouped<C::THREADS>(dot_part, dot_max_blocks, dot_cnt,
                                    RedCtx{nullptr, dot_scal, dot_flags}, s0, s1, dot_fin, -1, -1);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int fdm_setup(pdg_context *ctx, int precision) {
  const int N = ctx->N, dim = ctx->dim;
  // Cholesky of Mhat (host, from the FP64 table) and its inverse
  std::vector<double> tab(2 * N * N + 2 * N);
  PDG_CUDA_TRY(cudaMemcpy(tab.data(), ctx->tab64, sizeof(double) * tab.size(),
                          cudaMemcpyDeviceToHost));
  std::vector<double> Lc(N * N, 0.0), Li(N * N, 0.0);
  for (int i = 0; i < N; i++)
    for (int j = 0; j <= i; j++) {
      double s = tab[i * N + j];
      for (int q = 0; q < j; q++) s -= Lc[i * N + q] * Lc[j * N + q];
      if (i == j) {
        if (s <= 0) return set_error(PDG_EINVAL, "mass matrix not SPD");
        Lc[i * N + i] = std::sqrt(s);
      } else {
        Lc[i * N + j] = s / Lc[j * N + j];
      }
    }
  for (int c = 0; c < N; c++)
    for (int i = 0; i < N; i++) {
      double s = i == c ? 1.0 : 0.0;
      for (int q = 0; q < i; q++) s -= Lc[i * N + q] * Li[q * N + c];
      Li[i * N + c] = s / Lc[i * N + i];
    }
  double *dLi = nullptr;
  PDG_CUDA_TRY(cudaMalloc(&dLi, sizeof(double) * N * N));
  PDG_CUDA_TRY(cudaMemcpyAsync(dLi, Li.data(), sizeof(double) * N * N, cudaMemcpyHostToDevice,
                               ctx->stream));
  const size_t nq = (size_t)ctx->ncell * dim * N * N, nl = (size_t)ctx->ncell * dim * N;
  const size_t es = precision == PDG_F64 ? sizeof(double) : sizeof(float);
  PrecData &pd = ctx->prec[precision];
  PDG_CUDA_TRY(cudaMalloc(&pd.Q, nq * es));
  PDG_CUDA_TRY(cudaMalloc(&pd.L, nl * es));
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  const long work = ctx->ncell * dim;
  const unsigned blocks = (unsigned)((work + 127) / 128);
  double *Q64 = precision == PDG_F64 ? (double *)pd.Q : nullptr;
  double *L64 = precision == PDG_F64 ? (double *)pd.L : nullptr;
  float *Q32 = precision == PDG_F32 ? (float *)pd.Q : nullptr;
  float *L32 = precision == PDG_F32 ? (float *)pd.L : nullptr;
  switch (N) {
    case 2: k_fdm_setup<2><<<blocks, 128, 0, ctx->stream>>>(p, dim, dLi, Q64, L64, Q32, L32); break;
    case 3: k_fdm_setup<3><<<blocks, 128, 0, ctx->stream>>>(p, dim, dLi, Q64, L64, Q32, L32); break;
    case 4: k_fdm_setup<4><<<blocks, 128, 0, ctx->stream>>>(p, dim, dLi, Q64, L64, Q32, L32); break;
    case 5: k_fdm_setup<5><<<blocks, 128, 0, ctx->stream>>>(p, dim, dLi, Q64, L64, Q32, L32); break;
    default: cudaFree(dLi); return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
  PDG_CUDA_TRY(cudaGetLastError());
  if (precision == PDG_F64) {
    // the scaling of the FP64 apply as one multiply per DOF: FP64 division is a
    // multi-instruction sequence on the FP64 pipe that bounds the apply
    PDG_CUDA_TRY(cudaMalloc(&pd.Lsum_inv, sizeof(double) * ctx->ndof));
    const unsigned b2 = (unsigned)((ctx->ndof + 255) / 256);
    k_fdm_lsum_inv<<<b2, 256, 0, ctx->stream>>>(ctx->ndof, dim, N, (const double *)pd.L,
                                                   pd.Lsum_inv);
    PDG_CUDA_TRY(cudaGetLastError());
  }
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  cudaFree(dLi);
  return PDG_OK;
}

// The diagonal blocks D_e (row-major, FP64) by probing the operator kernel
// restricted to the cell; *D is allocated here and freed by the caller.
int diag_blocks(pdg_context *ctx, double **Dout) {
  const long nc = ctx->ncell;
  const int nb = ctx->nb;
  const size_t blk = (size_t)nc * nb * nb;
  double *D = nullptr, *x = nullptr, *y = nullptr;
  *Dout = nullptr;
  PDG_CUDA_TRY(cudaMalloc(&D, blk * sizeof(double)));
  if (cudaMalloc(&x, sizeof(double) * ctx->ndof) != cudaSuccess ||
      cudaMalloc(&y, sizeof(double) * ctx->ndof) != cudaSuccess) {
    cudaFree(D);
    if (x) cudaFree(x);
    return set_error(PDG_ECUDA, "out of device memory for the diagonal blocks");
  }
  const unsigned g = (unsigned)((ctx->ndof + 255) / 256);
  int st = PDG_OK;
  for (int j = 0; j < nb && st == PDG_OK; j++) {
    k_unit_field<<<g, 256, 0, ctx->stream>>>(nc, nb, j, x);
    ApplyArgs<double> a{x, y, nullptr, 1.0, 0, 0, 1, nullptr};
    st = launch_apply<double>(ctx, a, ctx->K64, ctx->c64, ctx->tab64);
    if (st == PDG_OK) k_scatter_col<<<g, 256, 0, ctx->stream>>>(nc, nb, j, y, D);
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(x);
  cudaFree(y);
  if (st != PDG_OK) {
    cudaFree(D);
    return st;
  }
  PDG_CUDA_TRY(cudaGetLastError());
  *Dout = D;
  return PDG_OK;
}

static int dense_setup(pdg_context *ctx, int precision) {
  const long nc = ctx->ncell;
  const int nb = ctx->nb;
  const size_t blk = (size_t)nc * nb * nb;
  double *D = nullptr;
  int *bad = nullptr;
  PDG_TRY(diag_blocks(ctx, &D));
  if (cudaMalloc(&bad, sizeof(int)) != cudaSuccess) {
    cudaFree(D);
    return set_error(PDG_ECUDA, "cudaMalloc failed");
  }
  PDG_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  const size_t es = precision == PDG_F64 ? sizeof(double) : sizeof(float);
  PrecData &pd = ctx->prec[precision];
  PDG_CUDA_TRY(cudaMalloc(&pd.inv, blk * es));
  const size_t smem = sizeof(double) * (nb * nb + nb) + sizeof(int) * nb;
  if (precision == PDG_F64) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_invert<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_invert<double><<<(unsigned)nc, 128, smem, ctx->stream>>>(nb, D, (double *)pd.inv, bad);
  } else {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_invert<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_invert<float><<<(unsigned)nc, 128, smem, ctx->stream>>>(nb, D, (float *)pd.inv, bad);
  }
  PDG_CUDA_TRY(cudaGetLastError());
  int hbad = 0;
  PDG_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  cudaFree(D); cudaFree(bad);
  if (hbad) return set_error(PDG_EINVAL, "singular diagonal block");
  if (precision == PDG_F32 && ctx->popt.dense_fp16) {
    const int nbp = (nb + 3) / 4 * 4;
    PDG_CUDA_TRY(cudaMalloc(&pd.inv16, (size_t)nc * nb * nbp * sizeof(__half)));
    PDG_CUDA_TRY(cudaMalloc(&pd.invscale, nc * sizeof(float)));
    k_inv_to_half<<<(unsigned)nc, 128, 0, ctx->stream>>>(nb, nbp, (const float *)pd.inv,
                                                        (__half *)pd.inv16, pd.invscale);
    PDG_CUDA_TRY(cudaGetLastError());
    PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    cudaFree(pd.inv);
    pd.inv = nullptr;
  }
  return PDG_OK;
}

void prec_free(pdg_context *ctx, int precision) {
  PrecData &pd = ctx->prec[precision];
  if (pd.Q) cudaFree(pd.Q);
  if (pd.L) cudaFree(pd.L);
  if (pd.inv) cudaFree(pd.inv);
  if (pd.blk) cudaFree(pd.blk);
  if (pd.invdiag) cudaFree(pd.invdiag);
  if (pd.iters) cudaFree(pd.iters);
  if (pd.inv16) cudaFree(pd.inv16);
  if (pd.invscale) cudaFree(pd.invscale);
  if (pd.Lsum_inv) cudaFree(pd.Lsum_inv);
  pd = PrecData{0, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
}

int prec_setup_impl(pdg_context *ctx, int kind, int precision) {
  if (precision != PDG_F64 && precision != PDG_F32)
    return set_error(PDG_EINVAL, "precision must be PDG_F64 or PDG_F32");
  prec_free(ctx, precision);
  ctx->op_gen++;
  if (kind == PDG_PREC_NONE) {
    ctx->prec[precision].kind = kind;
    ctx->prec[precision].ready = 1;
    return PDG_OK;
  }
  const int base = kind & PDG_PREC_BLOCK_MASK;
  if ((kind & ~(PDG_PREC_BLOCK_MASK | PDG_PREC_SOR)) != 0 || base > PDG_PREC_BJ_ITERATIVE)
    return set_error(PDG_EINVAL, "unknown preconditioner kind");
  if (base == PDG_PREC_BJ_FDM) {
    if (ctx->cfg.method != PDG_SIPG)
      return set_error(PDG_EUNSUPPORTED,
                       "FDM block Jacobi needs symmetric blocks (SIPG); use PDG_PREC_BJ_DENSE");
    if (general_coefficients(ctx))
      return set_error(PDG_EUNSUPPORTED,
                       "FDM block Jacobi needs separable blocks (A = K I per cell, c per cell); "
                       "use PDG_PREC_BJ_DENSE with a tensor or per-point coefficients");
    PDG_TRY(fdm_setup(ctx, precision));
  } else if (base == PDG_PREC_BJ_DENSE) {
    PDG_TRY(dense_setup(ctx, precision));
  } else if (base == PDG_PREC_BJ_ITERATIVE) {
    PDG_TRY(bj_iterative_setup(ctx, precision));
  }
  if (kind & PDG_PREC_SOR) PDG_TRY(sor_setup(ctx));
  ctx->prec[precision].kind = kind;
  ctx->prec[precision].ready = 1;
  return PDG_OK;
}

template <typename T, int D, int N>
static int fdm_apply_dn(pdg_context *ctx, const T *d, T *v, const int *skip, const int *cells,
                        int ncells, T scale) {
  if constexpr (std::is_same<T, float>::value && D == 3 && N == 4) {
    if (!cells) {
      using Q = FdmQ3Cfg;
      const size_t smem = 16 * Q::ROWS;
      static int attr_dev = -1;
      if (attr_dev != ctx->device) {
        PDG_CUDA_TRY(cudaFuncSetAttribute(k_fdm32_q3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        attr_dev = ctx->device;
      }
      const bool fuse = ctx->fuse_fin != 0;
      const unsigned blocks = (unsigned)((ctx->ncell + Q::CPB - 1) / Q::CPB);
      const float *rq = (fuse && ctx->fuse_fin == FIN_CG_DEF_BETA) ? (const float *)ctx->fuse_q
                                                                   : nullptr;
      const CUtensorMap *md = nullptr, *mq = nullptr, *unused = nullptr;
      const bool aligned = ((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(rq) |
                             reinterpret_cast<uintptr_t>(ctx->prec[PDG_F32].Q) |
                             reinterpret_cast<uintptr_t>(ctx->prec[PDG_F32].L)) & 15) == 0;
      if (aligned && q3_lines_maps(d, ctx->ndof, &unused, &md) &&
          (!rq || q3_lines_maps(rq, ctx->ndof, &unused, &mq))) {
        static int attr_t = -1;
        if (attr_t != ctx->device) {
          PDG_CUDA_TRY(cudaFuncSetAttribute(
              k_fdm32_q3t, cudaFuncAttributeMaxDynamicSharedMemorySize, FdmQ3T::SMEM));
          attr_t = ctx->device;
        }
        k_fdm32_q3t<<<blocks, FdmQ3T::THREADS, FdmQ3T::SMEM, ctx->stream>>>(
            ctx->ncell, (const float *)ctx->prec[PDG_F32].Q, (const float *)ctx->prec[PDG_F32].L,
            const_cast<float *>(d), v, skip, scale, fuse ? ctx->fuse_part : nullptr,
            ctx->fuse_max_blocks, ctx->fuse_cnt, ctx->red_out, ctx->d_flag, ctx->fuse_fin, rq,
            *md, rq ? *mq : *md, ctx->d_flag + F_TMA);
        PDG_CUDA_TRY(cudaGetLastError());
        return PDG_OK;
      }
      k_fdm32_q3<<<blocks, Q::THREADS, smem, ctx->stream>>>(
          ctx->ncell, (const float *)ctx->prec[PDG_F32].Q, (const float *)ctx->prec[PDG_F32].L,
          const_cast<float *>(d), v, skip, scale, fuse ? ctx->fuse_part : nullptr,
          ctx->fuse_max_blocks, ctx->fuse_cnt, ctx->red_out, ctx->d_flag, ctx->fuse_fin,
          (fuse && ctx->fuse_fin == FIN_CG_DEF_BETA) ? (const float *)ctx->fuse_q : nullptr);
      PDG_CUDA_TRY(cudaGetLastError());
      return PDG_OK;
    }
  }
  using C = PCfg<D, N>;
  const size_t smem = sizeof(T) * C::CPB * (C::PER_CELL + fdm_pad<T, D, N>());
  const long work = cells ? ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  const bool fuse = ctx->fuse_fin != 0;
  k_fdm_apply<T, D, N><<<blocks, C::THREADS, smem, ctx->stream>>>(
      ctx->ncell, (const T *)ctx->prec[std::is_same<T, double>::value ? 0 : 1].Q,
      (const T *)ctx->prec[std::is_same<T, double>::value ? 0 : 1].L, const_cast<T *>(d), v, skip,
      cells, ncells, scale, fuse ? ctx->fuse_part : nullptr, ctx->fuse_max_blocks, ctx->fuse_cnt,
      ctx->red_out, ctx->d_flag, ctx->fuse_fin,
      (fuse && ctx->fuse_fin == FIN_CG_DEF_BETA) ? (const T *)ctx->fuse_q : nullptr,
      std::is_same<T, double>::value ? (const T *)ctx->prec[0].Lsum_inv : nullptr);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <typename T>
__global__ void k_scale_cells(long ncell, int nb, const T *__restrict__ d, T *__restrict__ v,
                              const int *__restrict__ cells, int ncells, T scale,
                              const int *__restrict__ skip) {
  if (skip && *skip) return;
  const long n = (cells ? (long)ncells : ncell) * nb;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const long li = t / nb;
    const long e = cells ? (long)cells[li] : li;
    const long idx = e * nb + (t - li * nb);
    v[idx] = scale * d[idx];
  }
}

// v_e = scale * D_e^{-1} d_e (D_e^{-T} with `transpose`) on the listed cells
// (all cells if `cells` is null), with the block solver of the instance.
template <typename T>
static int fdm_dispatch(pdg_context *ctx, const T *d, T *v, const int *skip, const int *cells,
                        int ncells, T scale) {
  switch (ctx->dim * 10 + ctx->k) {
    case 21: return fdm_apply_dn<T, 2, 2>(ctx, d, v, skip, cells, ncells, scale);
    case 22: return fdm_apply_dn<T, 2, 3>(ctx, d, v, skip, cells, ncells, scale);
    case 23: return fdm_apply_dn<T, 2, 4>(ctx, d, v, skip, cells, ncells, scale);
    case 24: return fdm_apply_dn<T, 2, 5>(ctx, d, v, skip, cells, ncells, scale);
    case 31: return fdm_apply_dn<T, 3, 2>(ctx, d, v, skip, cells, ncells, scale);
    case 32: return fdm_apply_dn<T, 3, 3>(ctx, d, v, skip, cells, ncells, scale);
    case 33: return fdm_apply_dn<T, 3, 4>(ctx, d, v, skip, cells, ncells, scale);
    case 34: return fdm_apply_dn<T, 3, 5>(ctx, d, v, skip, cells, ncells, scale);
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
}

template <typename T>
int block_solve(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip,
                const int *cells, int ncells, T scale) {
  const int pi = std::is_same<T, double>::value ? PDG_F64 : PDG_F32;
  const PrecData &pd = ctx->prec[pi];
  const int base = pd.kind & PDG_PREC_BLOCK_MASK;
  const long work = cells ? ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  if (base == PDG_PREC_NONE) {
    long g = (work * ctx->nb + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_scale_cells<T><<<(unsigned)g, 256, 0, ctx->stream>>>(ctx->ncell, ctx->nb, d, v, cells,
                                                           ncells, scale, skip);
    PDG_CUDA_TRY(cudaGetLastError());
    return PDG_OK;
  }
  if (base == PDG_PREC_BJ_DENSE) {
    const int nb = ctx->nb;
    const int threads = ((nb + 31) / 32) * 32;
    if constexpr (std::is_same<T, float>::value) {
      if (pd.inv16) {
        // blocks up to nb = 512 (degree 7 in 3D): at least one column subset
        const int nbp = (nb + 3) / 4 * 4;
        if (nbp / 4 > kDenseH) return set_error(PDG_EUNSUPPORTED, "FP16 dense blocks: nb > 512");
        const size_t sm = sizeof(float) * (nbp + (kDenseH / (nbp / 4)) * nbp);
        k_dense_apply_h<<<(unsigned)work, kDenseH, sm, ctx->stream>>>(
            ctx->ncell, nb, nbp, (const __half *)pd.inv16, pd.invscale, d, v, transpose, skip,
            cells, scale);
        PDG_CUDA_TRY(cudaGetLastError());
        return PDG_OK;
      }
    }
    k_dense_apply<T><<<(unsigned)work, threads, sizeof(T) * nb, ctx->stream>>>(
        ctx->ncell, nb, (const T *)pd.inv, d, v, transpose, skip, cells, scale);
    PDG_CUDA_TRY(cudaGetLastError());
    return PDG_OK;
  }
  if (base == PDG_PREC_BJ_ITERATIVE)
    return bj_iterative_apply<T>(ctx, d, v, transpose, skip, cells, ncells, scale);
  if (ctx->basis == PDG_BASIS_LEGENDRE) {
    // the FDM factors invert the nodal block: D_L^{-1} = T^{-1} D^{-1} T^{-T}
    if (cells) return set_error(PDG_EUNSUPPORTED, "block SOR needs a nodal basis");
    const bool dbl = std::is_same<T, double>::value;
    T *w0 = dbl ? (T *)ctx->legw64[0] : (T *)ctx->legw32[0];
    T *w1 = dbl ? (T *)ctx->legw64[1] : (T *)ctx->legw32[1];
    PDG_TRY(basis_change<T>(ctx, 1, 1, d, w0, T(1), 0, nullptr, skip));
    PDG_TRY(fdm_dispatch<T>(ctx, w0, w1, skip, nullptr, 0, T(1)));
    return basis_change<T>(ctx, 1, 0, w1, v, scale, 0, nullptr, skip);
  }
  // FDM blocks are symmetric: D^{-T} = D^{-1}
  return fdm_dispatch<T>(ctx, d, v, skip, cells, ncells, scale);
}

template <typename T>
int prec_apply_skip(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip) {
  const int pi = std::is_same<T, double>::value ? PDG_F64 : PDG_F32;
  const PrecData &pd = ctx->prec[pi];
  if (!pd.ready) return set_error(PDG_ESTATE, "preconditioner not set up in this precision");
  if (pd.kind == PDG_PREC_NONE) return vec_copy<T>(ctx, ctx->ndof, d, v);
  if (pd.kind & PDG_PREC_SOR) return sor_apply<T>(ctx, d, v, transpose, skip);
  return block_solve<T>(ctx, d, v, transpose, skip, nullptr, 0, T(1));
}

template <typename T>
int prec_apply_impl(pdg_context *ctx, const T *d, T *v, int transpose) {
  return prec_apply_skip<T>(ctx, d, v, transpose, nullptr);
}

template int prec_apply_impl<double>(pdg_context *, const double *, double *, int);
template int prec_apply_impl<float>(pdg_context *, const float *, float *, int);
template int prec_apply_skip<double>(pdg_context *, const double *, double *, int, const int *);
template int prec_apply_skip<float>(pdg_context *, const float *, float *, int, const int *);
template int block_solve<double>(pdg_context *, const double *, double *, int, const int *,
                                 const int *, int, double);
template int block_solve<float>(pdg_context *, const float *, float *, int, const int *,
                                const int *, int, float);

}  // namespace pdg
