// pdg_ops.cuh -- per-face coefficients and per-cell 1D operators of
// ConvectionDiffusionDG on axis-parallel cells with A = K I, shared by the
// operator, preconditioner-setup and gradient kernels.
#pragma once

#include "pdg_internal.cuh"

namespace pdg {

// Division helpers: exact IEEE division in FP64 (the reference's
// arithmetic); fast reciprocal-based forms in FP32, whose apply only feeds
// the inner solve of the defect-correction loop.
__device__ __forceinline__ double qdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }
template <typename T>
__device__ __forceinline__ T over_h(const OpParams<T> &p, int dir, T x) {
  if (sizeof(T) == 8) return x / p.h[dir];
  return x * p.inv_h[dir];
}

// K of cell e for the terms of direction dir: with a diagonal tensor per
// cell A = diag(K_x, K_y, K_z), (A n).n = K_dir on a face normal to dir and
// the volume term of direction dir is K_dir d_dir u d_dir psi
// (convectiondiffusiondg.hh:124-127, 318-338)
template <typename T>
__device__ __forceinline__ T kdir(const OpParams<T> &p, long e, int dir) {
  return p.Kd ? p.Kd[3 * e + dir] : p.K[e];
}

// Ke: K of this cell in the face's normal direction (kdir)
template <typename T>
__device__ __forceinline__ void face_coefficients(const OpParams<T> &p, int f, T Ke,
                                                  long nb, T *coef) {
  // coef = {kappa_e/h, kappa_o/h, penalty}
  const int dir = f >> 1;
  T kap_e = T(0), kap_o = T(0), pen = T(0);
  if (nb >= 0) {
    const T Ko = kdir(p, nb, dir);
    if (p.weights == PDG_WEIGHTS_ON) {
      // convectiondiffusiondg.hh:326-332: delta = (A n).n = K
      const T S = Ke + Ko + T(1e-20);
      const T omega_e = qdiv(Ko, S);
      const T omega_o = qdiv(Ke, S);
      kap_e = omega_e * Ke;
      kap_o = omega_o * Ko;
      const T harm = qdiv(T(2) * Ke * Ko, S);
      pen = over_h(p, dir, p.pen_fac) * harm;   // h_F = min(|T_s|,|T_n|)/|F| = h
    } else {
      kap_e = T(0.5) * Ke;
      kap_o = T(0.5) * Ko;
      pen = over_h(p, dir, p.pen_fac);
    }
  } else if (p.bc[f] == PDG_BC_DIRICHLET) {
    // residual_boundary_integral: A_s n uses K_s; harmonic_average = K_s
    // (weightsOn) or 1 (:720-734)
    kap_e = Ke;
    pen = over_h(p, dir, p.pen_fac) * (p.weights == PDG_WEIGHTS_ON ? Ke : T(1));
  }
  coef[0] = over_h(p, dir, kap_e);
  coef[1] = over_h(p, dir, kap_o);
  coef[2] = pen;
}

// Entry (i = test, aa = trial) of the per-cell 1D operator of direction
// `dir`: (K_e/h) Shat + c h Mhat (dir 0 only) + the self terms of the two
// faces normal to dir, in the scaling y = hperp (A (x) Mhat (x) Mhat) u.
//   lower face (xi=0, n = -e_dir):  (kappa_e/h) v0 d0^T + pen v0 v0^T
//                                   - theta (kappa_e/h) d0 v0^T
//   upper face (xi=1, n = +e_dir): -(kappa_e/h) v1 d1^T + pen v1 v1^T
//                                   + theta (kappa_e/h) d1 v1^T
// (alpha_skeleton terms 2-4, convectiondiffusiondg.hh:452-469; boundary
// terms 2-4, :858-877).  cf = {kappa_e/h, kappa_o/h, pen} per face.
template <typename T, int N>
__device__ __forceinline__ T a_entry(const OpParams<T> &p, int dir, int i, int aa, T Ke, T cc,
                                     const T *cf, const T *tM, const T *tS, const T *td0,
                                     const T *td1) {
  const T h = p.h[dir];
  T v = over_h(p, dir, Ke) * tS[i * N + aa];
  if (dir == 0) v += cc * h * tM[i * N + aa];
  const T *cl = cf + 3 * (2 * dir);
  const T *ch = cf + 3 * (2 * dir + 1);
  if (i == 0) v += cl[0] * td0[aa];
  if (i == 0 && aa == 0) v += cl[2];
  if (aa == 0) v -= p.theta * cl[0] * td0[i];
  if (i == N - 1) v -= ch[0] * td1[aa];
  if (i == N - 1 && aa == N - 1) v += ch[2];
  if (aa == N - 1) v += p.theta * ch[0] * td1[i];
  return v;
}

}  // namespace pdg
