// pdg_conv.cu -- the convection part of ConvectionDiffusionDG:
//   volume   -int u b.grad(psi)                    (convectiondiffusiondg.hh:175-186)
//   faces    upwind flux (b.n >= 0 ? u_s : u_n) b.n psi, once per face with
//            r_s += term1 psi_s, r_n -= term1 psi_n  (:424-443)
//   Dirichlet faces (apply): (b.n >= 0 ? u : 0) b.n psi  (:842-849)
//   outflow faces: u b.n psi                      (:799-820)
// evaluated at the reference's Gauss points (order 2k), 3D.
//
// b is the velocity field b(x) = sum_m c_m sin(2 pi k_m.x + phase_m).  Since
// b does not change during a solve, a set-up kernel stores per cell the
// weighted velocity at every volume point, G_dir(q) = b_dir(x_q) w_q |J| / h_dir,
// and at every point of the six faces, F_f(p) = (b(x_p).n_f) w_p |F|, in FP64
// (and a FP32 copy), so the apply evaluates no trigonometric function.
//
// Apply (N*N threads per cell, z-columns, shared-memory line exchange):
//   volume: u_q = (B (x) B (x) B) u, then
//           y -= (Bt (x) Bt (x) Dt)(G_x u_q) + (Bt (x) Dt (x) Bt)(G_y u_q) + (Dt (x) Bt (x) Bt)(G_z u_q)
//   faces:  traces at face points by direct tensor evaluation of the face
//           node layer, upwind flux per point, tested with the face basis.
// Transposed apply (adjoint): volume -int psi b.grad(u); faces contribute to
// the upwind side only: y_e += int phi (b.n_e) (u_e - u_n) where b.n_e >= 0.
// diag_only (block-Jacobi blocks): neighbour traces are dropped.
#include <cmath>

#include "pdg_ops.cuh"
#include "pdg_vec.cuh"

namespace pdg {

template <int N>
struct CCfg {
  static constexpr int N2 = N * N, NB = N * N * N, TPC = N * N;
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  // S0..S3, then the face region: fluxes / face test results, own and
  // neighbour partial traces (the latter two reused for the partial tests)
  static constexpr int PER_CELL_RAW = 4 * NB + 18 * N2;
  // padding that puts the cells of a warp on different shared-memory banks
  // (counted wavefronts of the volume part's accesses, 4-byte elements)
  static constexpr int PAD = N == 2 ? 4 : N == 3 ? 27 : N == 4 ? 16 : N == 5 ? 3 : 0;
  // (FP32; FP64 keeps the raw stride)
  template <typename T>
  static constexpr int per_cell() { return sizeof(T) == 4 ? PER_CELL_RAW + PAD : PER_CELL_RAW; }
  static constexpr int TAB = 2 * N2;                 // B[q][a], D[q][a]
  static constexpr int VREC = 3 * NB;                // G_dir(q)
  static constexpr int FREC = 6 * N2;                // F_f(p)
};

__device__ __forceinline__ void conv_velocity(const Velocity &vel, const double *xg, double *b) {
  b[0] = b[1] = b[2] = 0.0;
  for (int m = 0; m < vel.nmodes; m++) {
    double arg = vel.m[m][3];
    for (int j = 0; j < 3; j++) arg += 2.0 * M_PI * vel.m[m][j] * xg[j];
    const double s = sin(arg);
    for (int j = 0; j < 3; j++) b[j] += vel.m[m][4 + j] * s;
  }
}

// Per-cell velocity record: [3][N^3] volume weights then [6][N^2] face fluxes.
// Flags *bad if an outflow boundary point has inflow (b.n < -1e-30).
template <int N>
__global__ void k_conv_setup(const OpParams<double> p, const Velocity vel, const RhsTables tb,
                             double *__restrict__ rec64, float *__restrict__ rec32,
                             int *__restrict__ bad) {
  using C = CCfg<N>;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  int ix[3];
  {
    long r = e;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  const double detJ = p.h[0] * p.h[1] * p.h[2];
  double *r64 = rec64 + e * (C::VREC + C::FREC);
  float *r32 = rec32 + e * (C::VREC + C::FREC);
  for (int q = 0; q < C::NB; q++) {
    const int qa[3] = {q % N, (q / N) % N, q / (N * N)};
    double xg[3], b[3];
    for (int j = 0; j < 3; j++) xg[j] = (ix[j] + tb.x[qa[j]]) * p.h[j];
    conv_velocity(vel, xg, b);
    const double w = tb.w[qa[0]] * tb.w[qa[1]] * tb.w[qa[2]] * detJ;
    for (int d = 0; d < 3; d++) {
      const double g = b[d] * w / p.h[d];
      r64[d * C::NB + q] = g;
      r32[d * C::NB + q] = (float)g;
    }
  }
  for (int f = 0; f < 6; f++) {
    const int dir = f >> 1, hi = f & 1;
    const double area = detJ / p.h[dir];
    const double sgn = hi ? 1.0 : -1.0;
    const bool bnd = hi ? ix[dir] == p.nc[dir] - 1 : ix[dir] == 0;
    for (int q = 0; q < C::N2; q++) {
      const int qt[2] = {q % N, q / N};
      double xg[3], b[3], w = area;
      int t = 0;
      for (int j = 0; j < 3; j++) {
        if (j == dir) { xg[j] = (ix[j] + (hi ? 1.0 : 0.0)) * p.h[j]; continue; }
        xg[j] = (ix[j] + tb.x[qt[t]]) * p.h[j];
        w *= tb.w[qt[t]];
        t++;
      }
      conv_velocity(vel, xg, b);
      const double bn = sgn * b[dir];
      if (bnd && p.bc[f] == PDG_BC_OUTFLOW && bn < -1e-30) atomicExch(bad, 1);
      r64[C::VREC + f * C::N2 + q] = bn * w;
      r32[C::VREC + f * C::N2 + q] = (float)(bn * w);
    }
  }
}

// The same record from velocity point data (pdg_set_velocity_points): b at
// the volume points [ncell][N^3][3] and at the face-lattice points
// [faces][N^2][3], one value per face point for both sides (the reference
// upwinds with b of the inside cell and assumes an H(div) field,
// convectiondiffusiondg.hh:425-426).
template <int N>
__global__ void k_conv_setup_points(const OpParams<double> p, const RhsTables tb,
                                    const double *__restrict__ bqv, const double *__restrict__ bqf,
                                    double *__restrict__ rec64, float *__restrict__ rec32,
                                    int *__restrict__ bad) {
  using C = CCfg<N>;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  int ix[3];
  {
    long r = e;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  const double detJ = p.h[0] * p.h[1] * p.h[2];
  double *r64 = rec64 + e * (C::VREC + C::FREC);
  float *r32 = rec32 + e * (C::VREC + C::FREC);
  for (int q = 0; q < C::NB; q++) {
    const int qa[3] = {q % N, (q / N) % N, q / (N * N)};
    const double w = tb.w[qa[0]] * tb.w[qa[1]] * tb.w[qa[2]] * detJ;
    for (int d = 0; d < 3; d++) {
      const double g = bqv[(e * C::NB + q) * 3 + d] * w / p.h[d];
      r64[d * C::NB + q] = g;
      r32[d * C::NB + q] = (float)g;
    }
  }
  for (int f = 0; f < 6; f++) {
    const int dir = f >> 1, hi = f & 1;
    const double area = detJ / p.h[dir];
    const double sgn = hi ? 1.0 : -1.0;
    const bool bnd = hi ? ix[dir] == p.nc[dir] - 1 : ix[dir] == 0;
    const long fi = face_lattice_index(p.nc, 3, dir, ix[dir] + hi, ix);
    for (int q = 0; q < C::N2; q++) {
      const int qt[2] = {q % N, q / N};
      const double w = area * tb.w[qt[0]] * tb.w[qt[1]];
      const double bn = sgn * bqf[(fi * C::N2 + q) * 3 + dir];
      if (bnd && p.bc[f] == PDG_BC_OUTFLOW && bn < -1e-30) atomicExch(bad, 1);
      r64[C::VREC + f * C::N2 + q] = bn * w;
      r32[C::VREC + f * C::N2 + q] = (float)(bn * w);
    }
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(CCfg<N>::THREADS)
    k_conv(const OpParams<T> p, const ApplyArgs<T> a, const T *__restrict__ vrec,
           const T *__restrict__ tabBD) {
  using C = CCfg<N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *tB = reinterpret_cast<T *>(smem_raw);   // B[q][a]
  T *tD = tB + N2;                           // D[q][a] (xi-derivative)
  const int t = threadIdx.x, cs = t / TPC, l = t - cs * TPC;
  T *S0 = tB + C::TAB + cs * C::template per_cell<T>();
  T *S1 = S0 + NB, *S2 = S1 + NB, *S3 = S2 + NB;
  T *fl = S3 + NB;                           // [6][N2] fluxes, then face test results
  T *Ue = fl + 6 * N2, *Un = Ue + 6 * N2;    // [6][N2] partial traces (own, neighbour)
  if (a.skip && *a.skip) return;
  for (int i = t; i < C::TAB; i += blockDim.x) tB[i] = tabBD[i];
  const long li = (long)blockIdx.x * CPB + cs;
  const bool ranged = !a.cells && a.ncells > 0;
  const bool active = (a.cells || ranged) ? li < a.ncells : li < p.ncell;
  const long e = a.cells ? (active ? (long)a.cells[li] : 0) : (ranged ? (long)a.cell0 + li : li);
  const long ee = active ? e : 0;
  int ix[3];
  {
    long r = ee;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  const long stride[3] = {1, (long)p.nc[0], (long)p.nc[0] * p.nc[1]};
  const T *rec = vrec + ee * (C::VREC + C::FREC);
  const int tx = l % N, ty = l / N;
  T col[N];
  const T *xe = a.x + ee * NB;
#pragma unroll
  for (int z = 0; z < N; z++) {
    col[z] = xe[z * N2 + l];
    S3[z * N2 + l] = col[z];   // own values for the face traces
  }
  __syncthreads();

  // ---------------- volume ----------------
  T r[N];
  if (!a.transpose) {
    // u_q = (B (x) B (x) B) u
    T v[N];
#pragma unroll
    for (int qz = 0; qz < N; qz++) {
      T s = T(0);
#pragma unroll
      for (int z = 0; z < N; z++) s += tB[qz * N + z] * col[z];
      v[qz] = s;
    }
#pragma unroll
    for (int z = 0; z < N; z++) S0[z * N2 + l] = v[z];
    __syncthreads();
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int b = 0; b < N; b++) s += tB[ty * N + b] * S0[z * N2 + b * N + tx];
      S1[z * N2 + l] = s;
    }
    __syncthreads();
    // point (qx=tx, qy=ty, qz): u_q, then F_dir = G_dir u_q -> S0 (x), S1 (y), S2 (z)
    T uq[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int aa = 0; aa < N; aa++) s += tB[tx * N + aa] * S1[z * N2 + ty * N + aa];
      uq[z] = s;
    }
    __syncthreads();
#pragma unroll
    for (int z = 0; z < N; z++) {
      const int q = z * N2 + l;
      S0[q] = rec[0 * NB + q] * uq[z];
      S1[q] = rec[1 * NB + q] * uq[z];
      S2[q] = rec[2 * NB + q] * uq[z];
    }
    __syncthreads();
    // x-step (node tx): Tx = Dt F_x, Ty = Bt F_y, Tz = Bt F_z
    T Tx[N], Ty[N], Tz[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T sx = T(0), sy = T(0), sz = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        const int i = z * N2 + ty * N + q;
        sx += tD[q * N + tx] * S0[i];
        sy += tB[q * N + tx] * S1[i];
        sz += tB[q * N + tx] * S2[i];
      }
      Tx[z] = sx; Ty[z] = sy; Tz[z] = sz;
    }
    __syncthreads();
#pragma unroll
    for (int z = 0; z < N; z++) {
      S0[z * N2 + l] = Tx[z];
      S1[z * N2 + l] = Ty[z];
      S2[z * N2 + l] = Tz[z];
    }
    __syncthreads();
    // y-step (node ty): Sxy = Bt Tx + Dt Ty ; Sz = Bt Tz
    T Sxy[N], Sz[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s1 = T(0), s2 = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) {
        const int i = z * N2 + q * N + tx;
        s1 += tB[q * N + ty] * S0[i] + tD[q * N + ty] * S1[i];
        s2 += tB[q * N + ty] * S2[i];
      }
      Sxy[z] = s1;
      Sz[z] = s2;
    }
    // z-step (registers): r = -(Bt Sxy + Dt Sz)
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) s += tB[q * N + z] * Sxy[q] + tD[q * N + z] * Sz[q];
      r[z] = -s;
    }
  } else {
    // gradient at the points: g_x = (B (x) B (x) D) u, g_y = (B (x) D (x) B) u,
    // g_z = (D (x) B (x) B) u; F = -(G_x g_x + G_y g_y + G_z g_z); r = (Bt (x) Bt (x) Bt) F
    T vb[N], vd[N];
#pragma unroll
    for (int qz = 0; qz < N; qz++) {
      T sb = T(0), sd = T(0);
#pragma unroll
      for (int z = 0; z < N; z++) {
        sb += tB[qz * N + z] * col[z];
        sd += tD[qz * N + z] * col[z];
      }
      vb[qz] = sb;
      vd[qz] = sd;
    }
#pragma unroll
    for (int z = 0; z < N; z++) {
      S0[z * N2 + l] = vb[z];   // z interpolated
      S1[z * N2 + l] = vd[z];   // z differentiated
    }
    __syncthreads();
    // y-step: A = B_y S0 (for x- and z-gradients use S0/S1 with B_y), Bd = D_y S0
#pragma unroll
    for (int z = 0; z < N; z++) {
      T sbb = T(0), sbd = T(0), sdb = T(0);
#pragma unroll
      for (int b = 0; b < N; b++) {
        const int i = z * N2 + b * N + tx;
        sbb += tB[ty * N + b] * S0[i];   // B_y B_z u
        sdb += tD[ty * N + b] * S0[i];   // D_y B_z u
        sbd += tB[ty * N + b] * S1[i];   // B_y D_z u
      }
      S2[z * N2 + l] = sbb;
      vb[z] = sdb;
      vd[z] = sbd;
    }
    __syncthreads();
#pragma unroll
    for (int z = 0; z < N; z++) {
      S0[z * N2 + l] = vb[z];
      S1[z * N2 + l] = vd[z];
    }
    __syncthreads();
    T F[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T gx = T(0), gy = T(0), gz = T(0);
#pragma unroll
      for (int aa = 0; aa < N; aa++) {
        const int i = z * N2 + ty * N + aa;
        gx += tD[tx * N + aa] * S2[i];   // D_x B_y B_z
        gy += tB[tx * N + aa] * S0[i];   // B_x D_y B_z
        gz += tB[tx * N + aa] * S1[i];   // B_x B_y D_z
      }
      const int q = z * N2 + l;
      F[z] = -(rec[q] * gx + rec[NB + q] * gy + rec[2 * NB + q] * gz);
    }
    __syncthreads();
    // test with Bt (x) Bt (x) Bt
#pragma unroll
    for (int z = 0; z < N; z++) S0[z * N2 + l] = F[z];
    __syncthreads();
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) s += tB[q * N + tx] * S0[z * N2 + ty * N + q];
      S1[z * N2 + l] = s;
    }
    __syncthreads();
    T w[N];
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) s += tB[q * N + ty] * S1[z * N2 + q * N + tx];
      w[z] = s;
    }
#pragma unroll
    for (int z = 0; z < N; z++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++) s += tB[q * N + z] * w[q];
      r[z] = s;
    }
  }

  // ---------------- faces ----------------
  // Traces at the face points and the test with the face basis are
  // sum-factorised through shared memory (the volume part has released
  // S0..S2): thread l = (pa, pb) first contracts row pb of a node layer with
  // B[pa][.], then column pa of the partial results with B[pb][.].
  const int pa = l % N, pb = l / N;
  const int st[3] = {1, N, N2};
  long nbr[6];
#pragma unroll
  for (int f = 0; f < 6; f++) {
    const int dir = f >> 1, hi = f & 1;
    if (hi) nbr[f] = ix[dir] + 1 < p.nc[dir] ? ee + stride[dir] : -1;
    else nbr[f] = ix[dir] > 0 ? ee - stride[dir] : -1;
  }
  T Bp[N], Bq[N];   // B[pa][.] and B[pb][.] (face point -> node layer)
#pragma unroll
  for (int i = 0; i < N; i++) {
    Bp[i] = tB[pa * N + i];
    Bq[i] = tB[pb * N + i];
  }
  // per face, U[j][pa] = sum_i B[pa][i] layer[j][i] into Ue (own), Un (neighbour)
#pragma unroll 1
  for (int f = 0; f < 6; f++) {
    const int dir = f >> 1, hi = f & 1;
    const int od0 = dir == 0 ? 1 : 0, od1 = dir == 2 ? 1 : 2;   // tangential dirs
    const int lay_e = hi ? N - 1 : 0, lay_n = hi ? 0 : N - 1;
    // row j = pb of the own and the neighbour's node layer
    T se = T(0), sn = T(0);
    const int rowe = lay_e * st[dir] + pb * st[od1], rown = lay_n * st[dir] + pb * st[od1];
#pragma unroll
    for (int i = 0; i < N; i++) se += Bp[i] * S3[rowe + i * st[od0]];
    if (nbr[f] >= 0 && !a.diag_only) {
      const T *xn = a.x + nbr[f] * NB;
#pragma unroll
      for (int i = 0; i < N; i++) sn += Bp[i] * xn[rown + i * st[od0]];
    }
    Ue[f * N2 + pb * N + pa] = se;
    Un[f * N2 + pb * N + pa] = sn;
  }
  __syncthreads();
#pragma unroll 1
  for (int f = 0; f < 6; f++) {
    T ue = T(0), un = T(0);
#pragma unroll
    for (int j = 0; j < N; j++) {
      ue += Bq[j] * Ue[f * N2 + j * N + pa];
      un += Bq[j] * Un[f * N2 + j * N + pa];
    }
    const T bnw = rec[C::VREC + f * N2 + l];
    T flux = T(0);
    if (nbr[f] >= 0) {
      if (a.diag_only) un = T(0);
      if (!a.transpose) flux = (bnw >= T(0) ? ue : un) * bnw;
      else flux = bnw >= T(0) ? (ue - un) * bnw : T(0);
    } else {
      const int bc = p.bc[f];
      if (bc == PDG_BC_DIRICHLET) flux = bnw >= T(0) ? ue * bnw : T(0);
      else if (bc == PDG_BC_OUTFLOW) flux = ue * bnw;
    }
    fl[f * N2 + l] = flux;
  }
  __syncthreads();
  // test with the face basis: W[j][pa] = sum_i B[i][pa] flux[j][i] (into S2),
  // then R[pb][pa] = sum_j B[j][pb] W[j][pa] (into fl, in place per face)
  T Cp[N], Cq[N];   // B[.][pa] and B[.][pb]
#pragma unroll
  for (int i = 0; i < N; i++) {
    Cp[i] = tB[i * N + pa];
    Cq[i] = tB[i * N + pb];
  }
  T *Wt = Ue;       // [6][N2]; Ue's last reads were before the previous barrier
#pragma unroll 1
  for (int f = 0; f < 6; f++) {
    T w = T(0);
#pragma unroll
    for (int i = 0; i < N; i++) w += Cp[i] * fl[f * N2 + pb * N + i];
    Wt[f * N2 + pb * N + pa] = w;
  }
  __syncthreads();
  T Rf[6];
#pragma unroll
  for (int f = 0; f < 6; f++) {
    T rr = T(0);
#pragma unroll
    for (int j = 0; j < N; j++) rr += Cq[j] * Wt[f * N2 + j * N + pa];
    Rf[f] = rr;
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < 6; f++) fl[f * N2 + pb * N + pa] = Rf[f];   // R[f][n1][n0]
  __syncthreads();
  // node (tx, ty, z) on the layer of face f receives R[f][n1][n0]
#pragma unroll
  for (int z = 0; z < N; z++) {
    T s = T(0);
    const int node[3] = {tx, ty, z};
#pragma unroll
    for (int f = 0; f < 6; f++) {
      const int dir = f >> 1, hi = f & 1;
      if (node[dir] != (hi ? N - 1 : 0)) continue;
      const int od0 = dir == 0 ? 1 : 0, od1 = dir == 2 ? 1 : 2;
      s += fl[f * N2 + node[od1] * N + node[od0]];
    }
    r[z] += s;
  }
  if (active) {
    T *ye = a.y + e * NB;
#pragma unroll
    for (int z = 0; z < N; z++) ye[z * N2 + l] += a.alpha * r[z];
  }
}

// ---------------------------------------------------------------------------
template <int N>
static int conv_setup_n(pdg_context *ctx) {
  using C = CCfg<N>;
  const size_t per = (size_t)(C::VREC + C::FREC);
  if (!ctx->conv64) PDG_CUDA_TRY(cudaMalloc(&ctx->conv64, sizeof(double) * per * ctx->ncell));
  if (!ctx->conv32) PDG_CUDA_TRY(cudaMalloc(&ctx->conv32, sizeof(float) * per * ctx->ncell));
  if (!ctx->convtab64) {
    RhsTables tb = make_rhs_tables(ctx);
    double h[2 * N * N];
    float h32[2 * N * N];
    // B[q][a] = phi_a(x_q), D[q][a] = phi_a'(x_q)
    for (int q = 0; q < N; q++)
      for (int aa = 0; aa < N; aa++) {
        h[q * N + aa] = tb.B[q * N + aa];
        h[N * N + q * N + aa] = lagrange_derivative(ctx, aa, tb.x[q]);
      }
    for (int i = 0; i < 2 * N * N; i++) h32[i] = (float)h[i];
    PDG_CUDA_TRY(cudaMalloc(&ctx->convtab64, sizeof(h)));
    PDG_CUDA_TRY(cudaMalloc(&ctx->convtab32, sizeof(h32)));
    PDG_CUDA_TRY(cudaMemcpy(ctx->convtab64, h, sizeof(h), cudaMemcpyHostToDevice));
    PDG_CUDA_TRY(cudaMemcpy(ctx->convtab32, h32, sizeof(h32), cudaMemcpyHostToDevice));
  }
  int *bad = nullptr;
  PDG_CUDA_TRY(cudaMalloc(&bad, sizeof(int)));
  PDG_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  RhsTables tb = make_rhs_tables(ctx);
  if (ctx->vel_points)
    k_conv_setup_points<N><<<(unsigned)((ctx->ncell + 127) / 128), 128, 0, ctx->stream>>>(
        p, tb, ctx->bqv64, ctx->bqf64, ctx->conv64, ctx->conv32, bad);
  else
    k_conv_setup<N><<<(unsigned)((ctx->ncell + 127) / 128), 128, 0, ctx->stream>>>(
        p, ctx->vel, tb, ctx->conv64, ctx->conv32, bad);
  PDG_CUDA_TRY(cudaGetLastError());
  int hbad = 0;
  PDG_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  cudaFree(bad);
  if (hbad) return set_error(PDG_EOUTFLOW, "outflow boundary condition on inflow");
  return PDG_OK;
}

int conv_setup(pdg_context *ctx) {
  if (ctx->dim != 3) return set_error(PDG_EUNSUPPORTED, "convection is implemented for 3D grids");
  switch (ctx->N) {
    case 2: return conv_setup_n<2>(ctx);
    case 3: return conv_setup_n<3>(ctx);
    case 4: return conv_setup_n<4>(ctx);
    case 5: return conv_setup_n<5>(ctx);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

template <typename T, int N>
static int conv_launch_n(pdg_context *ctx, const ApplyArgs<T> &a) {
  using C = CCfg<N>;
  const size_t smem = sizeof(T) * (C::TAB + C::CPB * C::template per_cell<T>());
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_conv<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_dev = ctx->device;
  }
  const bool dbl = std::is_same<T, double>::value;
  OpParams<T> p = make_params<T>(ctx, dbl ? (const T *)ctx->K64 : (const T *)ctx->K32, nullptr,
                                 dbl ? (const T *)ctx->tab64 : (const T *)ctx->tab32);
  const T *rec = dbl ? (const T *)ctx->conv64 : (const T *)ctx->conv32;
  const T *tab = dbl ? (const T *)ctx->convtab64 : (const T *)ctx->convtab32;
  const long work = (a.cells || a.ncells > 0) ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  k_conv<T, N><<<blocks, C::THREADS, smem, ctx->stream>>>(p, a, rec, tab);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// y += alpha C x (C^T when a.transpose); a.accumulate / a.add are ignored
// (the diffusion launch before it has already produced y).
template <typename T>
int launch_convection(pdg_context *ctx, const ApplyArgs<T> &a) {
  switch (ctx->N) {
    case 2: return conv_launch_n<T, 2>(ctx, a);
    case 3: return conv_launch_n<T, 3>(ctx, a);
    case 4: return conv_launch_n<T, 4>(ctx, a);
    case 5: return conv_launch_n<T, 5>(ctx, a);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}
template int launch_convection<double>(pdg_context *, const ApplyArgs<double> &);
template int launch_convection<float>(pdg_context *, const ApplyArgs<float> &);

}  // namespace pdg
