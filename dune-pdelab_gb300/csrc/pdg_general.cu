// pdg_general.cu -- ConvectionDiffusionDG's diffusion and reaction terms for
// parameter fields that are not a scalar K per cell: a full diffusion tensor
// A per cell, a tensor per quadrature point (permeabilityIsConstantPerCell()
// == false) and a reaction c per quadrature point.
//
// Reference: alpha_volume (dune/pdelab/localoperator/convectiondiffusiondg.hh:
// 105-188, A at the cell centre :124-127 or per point :141-146, c per point
// :181), alpha_skeleton (:270-471; A_s n and A_n n, the weights and the
// penalty from delta = (A n).n, per point when A is not constant :365-382),
// residual_boundary_integral on Dirichlet faces (:683-879, per point
// :750-761).  The convection terms stay in pdg_conv.cu.
//
// With a full tensor the operator is no longer a Kronecker product of 1D
// matrices, so this kernel evaluates the reference's forms at its Gauss
// points (order 2k, k+1 points per direction) by sum factorisation:
//   volume  u, grad u at the N^d points (9 line passes in 3D), the point
//           flux w|J| A grad u and w|J| c u, tested with grad psi and psi
//           (9 transposed line passes);
//   faces   value and normal-derivative layers of both sides (one line
//           reduction per face node), their tangential interpolation to the
//           N^(d-1) face points with the tangential derivatives, the point
//           terms 2-4 of the skeleton / Dirichlet boundary, and the test with
//           psi and (A_s n).grad psi (transposed passes, lifted along the
//           normal).
// Every cell computes the face terms of its own rows (the reference visits a
// face once and adds to both sides; the two are equal up to rounding, as the
// one-sided form is symmetric under exchanging the sides and n -> -n).
// The transposed operator (adjoint) uses the same point quantities with the
// roles of the trial traces (u, (A n).grad u) and the test traces (psi,
// (A n).grad psi) exchanged, and A^T in the volume.
//
// Thread mapping: N^(d-1) threads per cell.  Line passes: one line per
// thread.  Face steps: one face node or face point per thread.  Thread l
// owns the output column (z-column in 3D, y-column in 2D) of k_apply.
#include <cmath>

#include "pdg_ops.cuh"
#include "pdg_vec.cuh"

namespace pdg {

template <typename T, int N>
struct GpTab {
  T B[N * N];   // B[q*N + a] = phi_a(x_q) at the Gauss points
  T D[N * N];   // D[q*N + a] = phi_a'(x_q)
  T v[2][N];    // phi_a(0), phi_a(1)
  T d[2][N];    // phi_a'(0), phi_a'(1)
  T w[N];       // Gauss weights on [0,1]
  double x[N];  // Gauss points on [0,1] (velocity evaluation)
};

// Convection inside this kernel (2D grids; 3D runs pdg_conv.cu): b from point
// data (volume points [ncell][nqv][3], face lattice [faces][nqf][3]) or from
// the Fourier modes at the point's coordinates
struct GenConv {
  int on;
  const double *bqv, *bqf;
  Velocity vel;
};

template <int D>
__device__ __forceinline__ void velocity_modes(const Velocity &vel, const double *xg, double *b) {
  b[0] = b[1] = b[2] = 0.0;
  for (int m = 0; m < vel.nmodes; m++) {
    double arg = vel.m[m][3];
    for (int j = 0; j < D; j++) arg += 2.0 * M_PI * vel.m[m][j] * xg[j];
    const double s = sin(arg);
    for (int j = 0; j < D; j++) b[j] += vel.m[m][4 + j] * s;
  }
}

template <typename T>
struct GenCoef {
  const T *Ac;          // [ncell][d*d] per-cell tensor, row-major (or null)
  const T *Aqv, *Aqf;   // per-point tensors [ncell][nqv][d*d], [ncell][2d][nqf][d*d]
  const T *cq;          // [ncell][nqv] reaction per point (or null), added to p.c
};

template <int D, int N>
struct GCfg {
  static constexpr int N2 = N * N;
  static constexpr int NB = D == 3 ? N * N * N : N * N;
  static constexpr int NQF = D == 3 ? N * N : N;
  static constexpr int TPC = NQF;                      // threads per cell
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  static constexpr int DD = D * D;
  // U, S0..S4, Yf; face layers Vs Ds Vn Dn, interpolation F0..F5, point
  // coefficients G0..G3
  static constexpr int PER_CELL = 7 * NB + 14 * NQF + 1;
};

template <typename T, int D>
__device__ __forceinline__ void tensor_at(const T *src, T *A) {
#pragma unroll
  for (int i = 0; i < D * D; i++) A[i] = src[i];
}

// A of cell e: per point (volume point q, or point q of the cell's face f),
// per cell, or K_e I
template <typename T, int D, int N>
__device__ __forceinline__ void cell_tensor(const OpParams<T> &p, const GenCoef<T> &g, long e,
                                            int f, int q, T *A) {
  using C = GCfg<D, N>;
  if (g.Aqv) {
    const T *src = f < 0 ? g.Aqv + ((size_t)e * C::NB + q) * C::DD
                         : g.Aqf + (((size_t)e * 2 * D + f) * C::NQF + q) * C::DD;
    tensor_at<T, D>(src, A);
  } else if (g.Ac) {
    tensor_at<T, D>(g.Ac + (size_t)e * C::DD, A);
  } else {
    const T k = p.K[e];
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int j = 0; j < D; j++) A[i * D + j] = i == j ? k : T(0);
  }
}

template <typename T, int D, int N>
__global__ void __launch_bounds__(GCfg<D, N>::THREADS)
    k_apply_gp(const OpParams<T> p, const ApplyArgs<T> a, const GenCoef<T> g,
               const GpTab<T, N> tb, const GenConv cv_) {
  using C = GCfg<D, N>;
  constexpr int NB = C::NB, NQF = C::NQF, TPC = C::TPC, CPB = C::CPB, DD = C::DD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.skip && *a.skip) return;
  const int t = threadIdx.x;
  const int cs = t / TPC;
  const int l = t - cs * TPC;
  T *U = reinterpret_cast<T *>(smem_raw) + cs * C::PER_CELL;
  T *S0 = U + NB, *S1 = S0 + NB, *S2 = S1 + NB, *S3 = S2 + NB, *S4 = S3 + NB;
  T *Yf = S4 + NB;
  T *Vs = Yf + NB, *Ds = Vs + NQF, *Vn = Ds + NQF, *Dn = Vn + NQF;
  T *F0 = Dn + NQF, *F1 = F0 + NQF, *F2 = F1 + NQF, *F3 = F2 + NQF, *F4 = F3 + NQF,
    *F5 = F4 + NQF;
  T *G0 = F5 + NQF, *G1 = G0 + NQF, *G2 = G1 + NQF, *G3 = G2 + NQF;

  const int li = blockIdx.x * CPB + cs;
  const bool ranged = !a.cells && a.ncells > 0;
  const bool active = (a.cells || ranged) ? li < a.ncells : li < p.ncell;
  const int e = a.cells ? (active ? a.cells[li] : 0) : (ranged ? a.cell0 + li : li);
  const int ee = active ? e : 0;
  int ix[3];
  {
    const unsigned q0 = p.div0.div((unsigned)ee);
    const unsigned q1 = p.div1.div(q0);
    ix[0] = (int)((unsigned)ee - q0 * (unsigned)p.nc[0]);
    ix[1] = (int)(q0 - q1 * (unsigned)p.nc[1]);
    ix[2] = (int)q1;
  }
  const int gstride[3] = {1, p.nc[0], p.nc[0] * p.nc[1]};
  // stride of direction j inside a cell block (x fastest)
  auto ls = [](int j) { return j == 0 ? 1 : (j == 1 ? N : N * N); };
  const bool tr = a.transpose != 0;
  T detJ = T(1);
#pragma unroll
  for (int j = 0; j < D; j++) detJ *= p.h[j];

  // own values and a zeroed face accumulator
  const T *xe = a.x + (size_t)ee * NB;
  for (int i = l; i < NB; i += TPC) {
    U[i] = xe[i];
    Yf[i] = T(0);
  }
  __syncthreads();

  // ------------------------------------------------------------ volume ----
  T out[N];
  if constexpr (D == 3) {
    // z pass: S0 = B_z u, S1 = D_z u           (line base l = a0 + N a1)
#pragma unroll
    for (int q = 0; q < N; q++) {
      T s0 = T(0), s1 = T(0);
#pragma unroll
      for (int k = 0; k < N; k++) {
        const T u = U[l + k * (N * N)];
        s0 += tb.B[q * N + k] * u;
        s1 += tb.D[q * N + k] * u;
      }
      S0[l + q * (N * N)] = s0;
      S1[l + q * (N * N)] = s1;
    }
    __syncthreads();
    // y pass: S2 = B_y S0, S3 = D_y S0, S4 = B_y S1   (base a0 + N^2 q2)
    {
      const int base = (l % N) + (l / N) * (N * N);
#pragma unroll
      for (int q = 0; q < N; q++) {
        T s2 = T(0), s3 = T(0), s4 = T(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T v0 = S0[base + k * N], v1 = S1[base + k * N];
          s2 += tb.B[q * N + k] * v0;
          s3 += tb.D[q * N + k] * v0;
          s4 += tb.B[q * N + k] * v1;
        }
        S2[base + q * N] = s2;
        S3[base + q * N] = s3;
        S4[base + q * N] = s4;
      }
    }
    __syncthreads();
    // x pass to the points (base N q1 + N^2 q2), point terms, and the
    // transposed x pass back into S2 (y/z-gradient tests: S3, S4)
    {
      const int q1 = l % N, q2 = l / N;
      const int base = q1 * N + q2 * (N * N);
      T R[N], Fx[N], Fy[N], Fz[N];
#pragma unroll
      for (int q = 0; q < N; q++) {
        T uq = T(0), gx = T(0), gy = T(0), gz = T(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T v2 = S2[base + k], v3 = S3[base + k], v4 = S4[base + k];
          uq += tb.B[q * N + k] * v2;
          gx += tb.D[q * N + k] * v2;
          gy += tb.B[q * N + k] * v3;
          gz += tb.B[q * N + k] * v4;
        }
        const int qi = base + q;
        T A[DD];
        cell_tensor<T, 3, N>(p, g, ee, -1, qi, A);
        const T w = tb.w[q] * tb.w[q1] * tb.w[q2] * detJ;
        const T gr[3] = {over_h(p, 0, gx), over_h(p, 1, gy), over_h(p, 2, gz)};
        T F[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
          T s = T(0);
#pragma unroll
          for (int j = 0; j < 3; j++) s += (tr ? A[j * 3 + i] : A[i * 3 + j]) * gr[j];
          F[i] = w * s;
        }
        T cc = p.c ? p.c[ee] : T(0);
        if (g.cq) cc += g.cq[(size_t)ee * NB + qi];
        R[q] = w * cc * uq;
        if (cv_.on) {
          // -u b.grad psi (:175-186); transposed: -psi b.grad z
          double b[3];
          if (cv_.bqv) {
            for (int j = 0; j < 3; j++) b[j] = cv_.bqv[((size_t)ee * NB + qi) * 3 + j];
          } else {
            const double xg[3] = {(ix[0] + tb.x[q]) * (double)p.h[0],
                                  (ix[1] + tb.x[q1]) * (double)p.h[1],
                                  (ix[2] + tb.x[q2]) * (double)p.h[2]};
            velocity_modes<3>(cv_.vel, xg, b);
          }
          if (!tr) {
#pragma unroll
            for (int j = 0; j < 3; j++) F[j] -= w * uq * (T)b[j];
          } else {
            R[q] -= w * ((T)b[0] * gr[0] + (T)b[1] * gr[1] + (T)b[2] * gr[2]);
          }
        }
        Fx[q] = over_h(p, 0, F[0]);
        Fy[q] = over_h(p, 1, F[1]);
        Fz[q] = over_h(p, 2, F[2]);
      }
#pragma unroll
      for (int k = 0; k < N; k++) {
        T s2 = T(0), s3 = T(0), s4 = T(0);
#pragma unroll
        for (int q = 0; q < N; q++) {
          s2 += tb.D[q * N + k] * Fx[q] + tb.B[q * N + k] * R[q];
          s3 += tb.B[q * N + k] * Fy[q];
          s4 += tb.B[q * N + k] * Fz[q];
        }
        S2[base + k] = s2;
        S3[base + k] = s3;
        S4[base + k] = s4;
      }
    }
    __syncthreads();
    // transposed y pass: S0 = B_y^T S2 + D_y^T S3, S1 = B_y^T S4
    {
      const int base = (l % N) + (l / N) * (N * N);
#pragma unroll
      for (int k = 0; k < N; k++) {
        T s0 = T(0), s1 = T(0);
#pragma unroll
        for (int q = 0; q < N; q++) {
          s0 += tb.B[q * N + k] * S2[base + q * N] + tb.D[q * N + k] * S3[base + q * N];
          s1 += tb.B[q * N + k] * S4[base + q * N];
        }
        S0[base + k * N] = s0;
        S1[base + k * N] = s1;
      }
    }
    __syncthreads();
    // transposed z pass into the thread's z-column
#pragma unroll
    for (int k = 0; k < N; k++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++)
        s += tb.B[q * N + k] * S0[l + q * (N * N)] + tb.D[q * N + k] * S1[l + q * (N * N)];
      out[k] = s;
    }
  } else {
    // 2D: y pass (thread l = a0), x pass to the points (thread l = q1)
#pragma unroll
    for (int q = 0; q < N; q++) {
      T s0 = T(0), s1 = T(0);
#pragma unroll
      for (int k = 0; k < N; k++) {
        const T u = U[l + k * N];
        s0 += tb.B[q * N + k] * u;
        s1 += tb.D[q * N + k] * u;
      }
      S0[l + q * N] = s0;
      S1[l + q * N] = s1;
    }
    __syncthreads();
    {
      const int q1 = l, base = q1 * N;
      T R[N], Fx[N], Fy[N];
#pragma unroll
      for (int q = 0; q < N; q++) {
        T uq = T(0), gx = T(0), gy = T(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T v0 = S0[base + k], v1 = S1[base + k];
          uq += tb.B[q * N + k] * v0;
          gx += tb.D[q * N + k] * v0;
          gy += tb.B[q * N + k] * v1;
        }
        const int qi = base + q;
        T A[DD];
        cell_tensor<T, 2, N>(p, g, ee, -1, qi, A);
        const T w = tb.w[q] * tb.w[q1] * detJ;
        const T gr[2] = {over_h(p, 0, gx), over_h(p, 1, gy)};
        T F[2];
#pragma unroll
        for (int i = 0; i < 2; i++) {
          T s = T(0);
#pragma unroll
          for (int j = 0; j < 2; j++) s += (tr ? A[j * 2 + i] : A[i * 2 + j]) * gr[j];
          F[i] = w * s;
        }
        T cc = p.c ? p.c[ee] : T(0);
        if (g.cq) cc += g.cq[(size_t)ee * NB + qi];
        R[q] = w * cc * uq;
        if (cv_.on) {
          // -u b.grad psi (:175-186); transposed: -psi b.grad z
          double b[3];
          if (cv_.bqv) {
            for (int j = 0; j < 2; j++) b[j] = cv_.bqv[((size_t)ee * NB + qi) * 3 + j];
          } else {
            const double xg[2] = {(ix[0] + tb.x[q]) * (double)p.h[0],
                                  (ix[1] + tb.x[q1]) * (double)p.h[1]};
            velocity_modes<2>(cv_.vel, xg, b);
          }
          if (!tr) {
            F[0] -= w * uq * (T)b[0];
            F[1] -= w * uq * (T)b[1];
          } else {
            R[q] -= w * ((T)b[0] * gr[0] + (T)b[1] * gr[1]);
          }
        }
        Fx[q] = over_h(p, 0, F[0]);
        Fy[q] = over_h(p, 1, F[1]);
      }
      __syncthreads();   // the x pass read other threads' y-pass lines
#pragma unroll
      for (int k = 0; k < N; k++) {
        T s0 = T(0), s1 = T(0);
#pragma unroll
        for (int q = 0; q < N; q++) {
          s0 += tb.D[q * N + k] * Fx[q] + tb.B[q * N + k] * R[q];
          s1 += tb.B[q * N + k] * Fy[q];
        }
        S0[base + k] = s0;
        S1[base + k] = s1;
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; k++) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; q++)
        s += tb.B[q * N + k] * S0[l + q * N] + tb.D[q * N + k] * S1[l + q * N];
      out[k] = s;
    }
  }

  // ------------------------------------------------------------- faces ----
#pragma unroll 1
  for (int f = 0; f < 2 * D; f++) {
    const int dir = f >> 1, hi = f & 1;
    int o1 = 0, o2 = 0;       // tangential directions, ascending
    {
      int c = 0;
#pragma unroll
      for (int j = 0; j < D; j++)
        if (j != dir) { if (c == 0) o1 = j; else o2 = j; c++; }
    }
    long nb;
    if (hi) nb = ix[dir] + 1 < p.nc[dir] ? (long)ee + gstride[dir] : -1;
    else nb = ix[dir] > 0 ? (long)ee - gstride[dir] : -1;
    const bool interior = nb >= 0;
    const bool dirichlet = !interior && p.bc[f] == PDG_BC_DIRICHLET;
    const bool outflow = !interior && cv_.on && p.bc[f] == PDG_BC_OUTFLOW;
    const bool live = interior || dirichlet || outflow;
    const bool coupled = interior && !a.diag_only;

    // step 1: value and normal-derivative layers at the face (thread l:
    // tangential node (i1, i2))
    {
      const int i1 = D == 3 ? l % N : l, i2 = D == 3 ? l / N : 0;
      const int base = i1 * ls(o1) + (D == 3 ? i2 * ls(o2) : 0);
      T vs = T(0), ds = T(0), vn = T(0), dn = T(0);
      if (live) {
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T u = U[base + k * ls(dir)];
          vs += tb.v[hi][k] * u;
          ds += tb.d[hi][k] * u;
        }
      }
      if (coupled) {
        const T *xn = a.x + (size_t)nb * NB;
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T u = xn[base + k * ls(dir)];
          vn += tb.v[1 - hi][k] * u;
          dn += tb.d[1 - hi][k] * u;
        }
      }
      Vs[l] = vs;
      Ds[l] = ds;
      Vn[l] = vn;
      Dn[l] = dn;
    }
    __syncthreads();
    // steps 2-3: traces at the face point of thread l: value, normal and
    // tangential derivatives (reference coordinates) of both sides
    T us, dns, dt1s, dt2s = T(0), un, dnn, dt1n, dt2n = T(0);
    const int q1 = D == 3 ? l % N : l, q2 = D == 3 ? l / N : 0;
    if constexpr (D == 3) {
      {
        // tangential-1 pass (thread l = (q1, i2))
        const int i2 = l / N;
        T b0 = T(0), b1 = T(0), b2 = T(0), b3 = T(0), b4 = T(0), b5 = T(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T B = tb.B[q1 * N + k], Dd = tb.D[q1 * N + k];
          b0 += B * Vs[k + N * i2];
          b1 += Dd * Vs[k + N * i2];
          b2 += B * Ds[k + N * i2];
          b3 += B * Vn[k + N * i2];
          b4 += Dd * Vn[k + N * i2];
          b5 += B * Dn[k + N * i2];
        }
        F0[l] = b0; F1[l] = b1; F2[l] = b2; F3[l] = b3; F4[l] = b4; F5[l] = b5;
      }
      __syncthreads();
      us = dns = dt1s = un = dnn = dt1n = T(0);
#pragma unroll
      for (int k = 0; k < N; k++) {
        const T B = tb.B[q2 * N + k], Dd = tb.D[q2 * N + k];
        us += B * F0[q1 + N * k];
        dt1s += B * F1[q1 + N * k];
        dt2s += Dd * F0[q1 + N * k];
        dns += B * F2[q1 + N * k];
        un += B * F3[q1 + N * k];
        dt1n += B * F4[q1 + N * k];
        dt2n += Dd * F3[q1 + N * k];
        dnn += B * F5[q1 + N * k];
      }
    } else {
      us = dns = dt1s = un = dnn = dt1n = T(0);
#pragma unroll
      for (int k = 0; k < N; k++) {
        const T B = tb.B[q1 * N + k], Dd = tb.D[q1 * N + k];
        us += B * Vs[k];
        dt1s += Dd * Vs[k];
        dns += B * Ds[k];
        un += B * Vn[k];
        dt1n += Dd * Vn[k];
        dnn += B * Dn[k];
      }
    }
    // point terms (terms 2-4 of the skeleton, :445-469; Dirichlet boundary
    // with g = 0, :851-877)
    T cv = T(0), cn = T(0), ct1 = T(0), ct2 = T(0);
    if (live && active) {
      const int pq = q1 + (D == 3 ? N * q2 : 0);
      const T sgn = hi ? T(1) : T(-1);
      T As[DD], An[DD];
      cell_tensor<T, D, N>(p, g, ee, f, pq, As);
      // A n of both sides; the normal derivative is the dir component
      T AnS[3], AnN[3];
#pragma unroll
      for (int j = 0; j < D; j++) AnS[j] = As[j * D + dir] * sgn;
      const T delta_s = As[dir * D + dir];
      // physical gradients (components dir, o1, o2)
      T gs[3], gn[3];
      gs[dir] = over_h(p, dir, dns);
      gs[o1] = over_h(p, o1, dt1s);
      if (D == 3) gs[o2] = over_h(p, o2, dt2s);
      T wq = tb.w[q1] * (D == 3 ? tb.w[q2] : T(1));
      wq *= p.h[o1] * (D == 3 ? p.h[o2] : T(1));
      // convection: b.n_F at the face point (one value for both sides) and
      // the upwind side (:425-443, 796-849)
      T nflux = T(0);
      if (cv_.on) {
        double b[3];
        if (cv_.bqf) {
          const long fi = face_lattice_index(p.nc, D, dir, ix[dir] + hi, ix);
          b[dir] = cv_.bqf[(fi * NQF + pq) * 3 + dir];
        } else {
          double xg[3];
          xg[dir] = (ix[dir] + hi) * (double)p.h[dir];
          xg[o1] = (ix[o1] + tb.x[q1]) * (double)p.h[o1];
          if (D == 3) xg[o2] = (ix[o2] + tb.x[q2]) * (double)p.h[o2];
          velocity_modes<D>(cv_.vel, xg, b);
        }
        nflux = (T)(hi ? b[dir] : -b[dir]);
      }
      const T up_s = nflux >= T(0) ? T(1) : T(0);
      T Cv, Cg;
      if (outflow) {
        // u b.n psi (:799-820), symmetric in trial and test
        Cv = us * nflux * wq;
        Cg = T(0);
      } else if (interior) {
        cell_tensor<T, D, N>(p, g, nb, f ^ 1, pq, An);
#pragma unroll
        for (int j = 0; j < D; j++) AnN[j] = An[j * D + dir] * sgn;
        const T delta_n = An[dir * D + dir];
        T om_s, om_n, harm;
        if (p.weights == PDG_WEIGHTS_ON) {
          const T S = delta_s + delta_n + T(1e-20);
          om_s = qdiv(delta_n, S);
          om_n = qdiv(delta_s, S);
          harm = qdiv(T(2) * delta_s * delta_n, S);
        } else {
          om_s = om_n = T(0.5);
          harm = T(1);
        }
        const T pen = over_h(p, dir, p.pen_fac) * harm;
        gn[dir] = over_h(p, dir, dnn);
        gn[o1] = over_h(p, o1, dt1n);
        if (D == 3) gn[o2] = over_h(p, o2, dt2n);
        T As_g = T(0), An_g = T(0);   // (A n).grad of the traces
#pragma unroll
        for (int j = 0; j < D; j++) { As_g += AnS[j] * gs[j]; An_g += AnN[j] * gn[j]; }
        const T jump = us - un;
        if (!tr) {
          Cv = (-(om_s * As_g + om_n * An_g) + pen * jump) * wq;
          Cg = p.theta * om_s * jump * wq;
          // term 1: (up_s u_s + up_n u_n) b.n psi_s
          if (cv_.on) Cv += (up_s * us + (T(1) - up_s) * un) * nflux * wq;
        } else {
          Cv = (pen * jump + p.theta * (om_s * As_g + om_n * An_g)) * wq;
          Cg = -om_s * jump * wq;
          if (cv_.on) Cv += up_s * nflux * jump * wq;
        }
      } else {
        const T harm = p.weights == PDG_WEIGHTS_ON ? delta_s : T(1);
        const T pen = over_h(p, dir, p.pen_fac) * harm;
        T As_g = T(0);
#pragma unroll
        for (int j = 0; j < D; j++) As_g += AnS[j] * gs[j];
        if (!tr) {
          Cv = (-As_g + pen * us) * wq;
          Cg = p.theta * us * wq;
        } else {
          Cv = (pen * us + p.theta * As_g) * wq;
          Cg = -us * wq;
        }
        // Dirichlet inflow upwind term with g = 0 (:842-849), symmetric
        if (cv_.on) Cv += up_s * us * nflux * wq;
      }
      // test: Cv psi + Cg (A_s n).grad psi, the gradient in reference
      // coordinates scaled by 1/h per direction
      cv = Cv;
      cn = over_h(p, dir, Cg * AnS[dir]);
      ct1 = over_h(p, o1, Cg * AnS[o1]);
      if (D == 3) ct2 = over_h(p, o2, Cg * AnS[o2]);
    }
    // steps 4-5: back to the face nodes and along the normal into Yf
    if constexpr (D == 3) {
      G0[l] = cv; G1[l] = cn; G2[l] = ct1; G3[l] = ct2;
      __syncthreads();
      {
        // transposed tangential-2 pass (thread l = (q1, i2))
        const int i2 = l / N;
        T x1 = T(0), x2 = T(0), x3 = T(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
          const T B = tb.B[k * N + i2], Dd = tb.D[k * N + i2];
          x1 += B * G0[q1 + N * k] + Dd * G3[q1 + N * k];
          x2 += B * G2[q1 + N * k];
          x3 += B * G1[q1 + N * k];
        }
        F0[l] = x1; F1[l] = x2; F2[l] = x3;
      }
      __syncthreads();
      {
        // transposed tangential-1 pass (thread l = (i1, i2)) and the lift
        const int i1 = l % N, i2 = l / N;
        T wv = T(0), wn = T(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
          wv += tb.B[k * N + i1] * F0[k + N * i2] + tb.D[k * N + i1] * F1[k + N * i2];
          wn += tb.B[k * N + i1] * F2[k + N * i2];
        }
        const int base = i1 * ls(o1) + i2 * ls(o2);
        if (live) {
#pragma unroll
          for (int k = 0; k < N; k++) Yf[base + k * ls(dir)] += tb.v[hi][k] * wv + tb.d[hi][k] * wn;
        }
      }
    } else {
      G0[l] = cv; G1[l] = cn; G2[l] = ct1;
      __syncthreads();
      const int i1 = l;
      T wv = T(0), wn = T(0);
#pragma unroll
      for (int k = 0; k < N; k++) {
        wv += tb.B[k * N + i1] * G0[k] + tb.D[k * N + i1] * G2[k];
        wn += tb.B[k * N + i1] * G1[k];
      }
      const int base = i1 * ls(o1);
      if (live) {
#pragma unroll
        for (int k = 0; k < N; k++) Yf[base + k * ls(dir)] += tb.v[hi][k] * wv + tb.d[hi][k] * wn;
      }
    }
    __syncthreads();
  }

  if (active) {
    T *ye = a.y + (size_t)e * NB;
    const T *ad = a.add ? a.add + (size_t)e * NB : nullptr;
    const bool scale = a.alpha != T(1);
#pragma unroll
    for (int k = 0; k < N; k++) {
      const int idx = l + k * (D == 3 ? (N * N) : N);
      T r = out[k] + Yf[idx];
      if (scale) r *= a.alpha;
      if (a.accumulate) r += ye[idx];
      if (ad) r += ad[idx];
      ye[idx] = r;
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename T, int N>
static GpTab<T, N> make_gp_tab(const pdg_context *ctx) {
  const RhsTables r = make_rhs_tables(ctx);
  GpTab<T, N> tb{};
  for (int q = 0; q < N; q++) {
    tb.w[q] = (T)r.w[q];
    tb.x[q] = r.x[q];
    for (int k = 0; k < N; k++) {
      tb.B[q * N + k] = (T)r.B[q * N + k];
      tb.D[q * N + k] = (T)lagrange_derivative(ctx, k, r.x[q]);
    }
  }
  // the nodal bases have their first node at 0 and their last at 1
  for (int k = 0; k < N; k++) {
    tb.v[0][k] = (T)(k == 0 ? 1.0 : 0.0);
    tb.v[1][k] = (T)(k == N - 1 ? 1.0 : 0.0);
    tb.d[0][k] = (T)r.d0[k];
    tb.d[1][k] = (T)r.d1[k];
  }
  return tb;
}

template <typename T, int D, int N>
static int launch_gp_dn(pdg_context *ctx, const ApplyArgs<T> &a, const OpParams<T> &p,
                        const GenCoef<T> &g, const GenConv &cv) {
  using C = GCfg<D, N>;
  const size_t smem = sizeof(T) * C::CPB * C::PER_CELL;
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply_gp<T, D, N>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_dev = ctx->device;
  }
  const long work = (a.cells || a.ncells > 0) ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  k_apply_gp<T, D, N><<<blocks, C::THREADS, smem, ctx->stream>>>(p, a, g, make_gp_tab<T, N>(ctx),
                                                                  cv);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// R(0)'s Dirichlet-data diffusion terms with a tensor A (residual_boundary_
// integral with u = 0, :851-877): r_i += w [-pen g psi_i - theta g
// (A_s n).grad psi_i], pen from delta = (A_s n).n at the point (per point
// when A is) or per cell.  One thread per cell, dense loops (once per solve).
template <int D, int N>
__global__ void k_rhs_gp(const OpParams<double> p, const GenCoef<double> g, const GpTab<double, N> tb,
                         const double *__restrict__ gq, double *__restrict__ r0) {
  using C = GCfg<D, N>;
  constexpr int NB = C::NB, NQF = C::NQF, DD = C::DD;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  int ix[3];
  {
    long r = e;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  for (int f = 0; f < 2 * D; f++) {
    const int dir = f >> 1, hi = f & 1;
    const bool bnd = hi ? ix[dir] == p.nc[dir] - 1 : ix[dir] == 0;
    if (!bnd || p.bc[f] != PDG_BC_DIRICHLET) continue;
    int od[2] = {0, 0};
    {
      int c = 0;
      for (int j = 0; j < D; j++)
        if (j != dir) od[c++] = j;
    }
    // boundary points: sides in order, faces lexicographic over the other
    // directions, NQF points per face
    long base = 0;
    for (int sd = 0; sd < f; sd++) {
      long cnt = 1;
      for (int j = 0; j < D; j++)
        if (j != (sd >> 1)) cnt *= p.nc[j];
      base += cnt * NQF;
    }
    long fidx = 0;
    for (int j = D - 1; j >= 0; j--) {
      if (j == dir) continue;
      fidx = fidx * p.nc[j] + ix[j];
    }
    base += fidx * NQF;
    const double sgn = hi ? 1.0 : -1.0;
    double area = 1.0;
    for (int j = 0; j < D; j++)
      if (j != dir) area *= p.h[j];
    for (int q = 0; q < NQF; q++) {
      const double gv = gq[base + q];
      if (gv == 0.0) continue;
      const int qt[2] = {q % N, D == 3 ? q / N : 0};
      double A[DD];
      cell_tensor<double, D, N>(p, g, e, f, q, A);
      double An[3];
      for (int j = 0; j < D; j++) An[j] = A[j * D + dir] * sgn;
      const double harm = p.weights == PDG_WEIGHTS_ON ? A[dir * D + dir] : 1.0;
      const double pen = p.pen_fac / p.h[dir] * harm;
      double w = area * tb.w[qt[0]] * (D == 3 ? tb.w[qt[1]] : 1.0);
      for (int i = 0; i < NB; i++) {
        const int ia[3] = {i % N, (i / N) % N, i / (N * N)};
        // value and reference derivatives of psi_i at the point
        double tv[2], td[2];
        for (int t = 0; t < D - 1; t++) {
          tv[t] = tb.B[qt[t] * N + ia[od[t]]];
          td[t] = tb.D[qt[t] * N + ia[od[t]]];
        }
        const double vn = tb.v[hi][ia[dir]], dn = tb.d[hi][ia[dir]];
        double tang = 1.0;
        for (int t = 0; t < D - 1; t++) tang *= tv[t];
        const double psi = vn * tang;
        double agrad = An[dir] * dn / p.h[dir] * tang;
        for (int t = 0; t < D - 1; t++) {
          double gt = vn * td[t] / p.h[od[t]];
          for (int s2 = 0; s2 < D - 1; s2++)
            if (s2 != t) gt *= tv[s2];
          agrad += An[od[t]] * gt;
        }
        r0[e * NB + i] += w * (-pen * gv * psi - p.theta * gv * agrad);
      }
    }
  }
}

long face_lattice_count(const pdg_context *ctx) {
  long n = 0;
  for (int dir = 0; dir < ctx->dim; dir++) {
    long c = ctx->cfg.cells[dir] + 1;
    for (int j = 0; j < ctx->dim; j++)
      if (j != dir) c *= ctx->cfg.cells[j];
    n += c;
  }
  return n;
}

int launch_rhs_general(pdg_context *ctx) {
  if (!ctx->gq || !(ctx->gen_A == 1 || ctx->gen_A == 2)) return PDG_OK;
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  GenCoef<double> g{};
  if (ctx->gen_A == 1) g.Ac = ctx->Ac64;
  if (ctx->gen_A == 2) { g.Aqv = ctx->Aqv64; g.Aqf = ctx->Aqf64; }
  const unsigned blocks = (unsigned)((ctx->ncell + 127) / 128);
#define PDG_RGP(D, N)                                                            \
  k_rhs_gp<D, N><<<blocks, 128, 0, ctx->stream>>>(p, g, make_gp_tab<double, N>(ctx), ctx->gq, \
                                                  ctx->r0)
  switch (ctx->dim * 10 + ctx->k) {
    case 21: PDG_RGP(2, 2); break;
    case 22: PDG_RGP(2, 3); break;
    case 23: PDG_RGP(2, 4); break;
    case 24: PDG_RGP(2, 5); break;
    case 31: PDG_RGP(3, 2); break;
    case 32: PDG_RGP(3, 3); break;
    case 33: PDG_RGP(3, 4); break;
    case 34: PDG_RGP(3, 5); break;
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
#undef PDG_RGP
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

bool general_coefficients(const pdg_context *ctx) {
  // a diagonal tensor per cell (gen_A 3) stays in Kronecker form; 2D
  // convection runs here (3D convection has its own kernel)
  return ctx->gen_A == 1 || ctx->gen_A == 2 || ctx->cq64 != nullptr ||
         (ctx->dim == 2 && convection_on(ctx));
}

template <typename T>
int launch_apply_general(pdg_context *ctx, const ApplyArgs<T> &a) {
  const bool dbl = std::is_same<T, double>::value;
  const T *K = dbl ? (const T *)ctx->K64 : (const T *)ctx->K32;
  const T *c = dbl ? (const T *)ctx->c64 : (const T *)ctx->c32;
  const T *tab = dbl ? (const T *)ctx->tab64 : (const T *)ctx->tab32;
  OpParams<T> p = make_params<T>(ctx, K, c, tab);
  GenCoef<T> g{};
  if (ctx->gen_A == 1 || ctx->gen_A == 3) g.Ac = dbl ? (const T *)ctx->Ac64 : (const T *)ctx->Ac32;
  if (ctx->gen_A == 2) {
    g.Aqv = dbl ? (const T *)ctx->Aqv64 : (const T *)ctx->Aqv32;
    g.Aqf = dbl ? (const T *)ctx->Aqf64 : (const T *)ctx->Aqf32;
  }
  g.cq = dbl ? (const T *)ctx->cq64 : (const T *)ctx->cq32;
  GenConv cv{};
  cv.on = ctx->dim == 2 && convection_on(ctx);
  if (cv.on) {
    cv.bqv = ctx->vel_points ? ctx->bqv64 : nullptr;
    cv.bqf = ctx->vel_points ? ctx->bqf64 : nullptr;
    cv.vel = ctx->vel;
  }
  switch (ctx->dim * 10 + ctx->k) {
    case 21: return launch_gp_dn<T, 2, 2>(ctx, a, p, g, cv);
    case 22: return launch_gp_dn<T, 2, 3>(ctx, a, p, g, cv);
    case 23: return launch_gp_dn<T, 2, 4>(ctx, a, p, g, cv);
    case 24: return launch_gp_dn<T, 2, 5>(ctx, a, p, g, cv);
    case 31: return launch_gp_dn<T, 3, 2>(ctx, a, p, g, cv);
    case 32: return launch_gp_dn<T, 3, 3>(ctx, a, p, g, cv);
    case 33: return launch_gp_dn<T, 3, 4>(ctx, a, p, g, cv);
    case 34: return launch_gp_dn<T, 3, 5>(ctx, a, p, g, cv);
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in");
  }
}
template int launch_apply_general<double>(pdg_context *, const ApplyArgs<double> &);
template int launch_apply_general<float>(pdg_context *, const ApplyArgs<float> &);

}  // namespace pdg
