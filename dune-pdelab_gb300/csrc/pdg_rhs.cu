// pdg_rhs.cu -- the x-independent part of the residual, R(0), and the
// fused adjoint gradient kernels.
//
// R(x) = J x + R(0) for this linear operator, so GridOperator::residual
// (gridoperator.hh:176-181) is evaluated as one operator launch that adds a
// precomputed R(0):
//   R(0) = - int f psi                              (lambda_volume, :1047-1075)
//        + Dirichlet faces:  (b.n < 0 ? g b.n : 0) psi - theta K g dpsi/dn
//                            - penalty g psi       (:842-877 with u = 0)
//        + Neumann faces:    j psi                  (:775-786)
//        + Outflow faces:    o psi                  (:799-820)
// evaluated at the same Gauss points as the reference (order 2k).
//
// Gradient (no reference counterpart):  dJ/d(log K_e) = -lambda^T dR/d(log K_e).
// With weightsOn every diffusion term is linear in one coefficient: the
// volume term in K_e, an interior face in H = 2 K_s K_n/(K_s+K_n+1e-20)
// (kappa_s = kappa_n = H/2, penalty ~ H; :326-346), a Dirichlet face in K_e
// (:720-734).  So
//   g_e = -K_e [ lambda_e^T Avol(1) u_e + sum_faces dH/dK_e a_f(1)(u, lambda)
//               + sum_Dirichlet a_B(1)(u_e, lambda_e) ] - lambda_e . R0_K,e
// where (1) marks unit coefficient and R0_K is the K-proportional Dirichlet
// data part of R(0).  Face forms are evaluated on face nodes with the exact
// tangential mass Mhat (x) Mhat (Gauss k+1 is exact for degree 2k).
#include <cmath>

#include "pdg_ops.cuh"

namespace pdg {


__device__ __forceinline__ void velocity_at(const Velocity &vel, int dim, const double *xg,
                                            double *b) {
  b[0] = b[1] = b[2] = 0.0;
  for (int m = 0; m < vel.nmodes; m++) {
    double arg = vel.m[m][3];
    for (int j = 0; j < dim; j++) arg += 2.0 * M_PI * vel.m[m][j] * xg[j];
    const double s = sin(arg);
    for (int j = 0; j < dim; j++) b[j] += vel.m[m][4 + j] * s;
  }
}

template <int D, int N>
__global__ void k_rhs(const OpParams<double> p, const RhsTables tb, const Velocity vel,
                      const double *__restrict__ fq, const double *__restrict__ fc,
                      const double *__restrict__ gq, const double *__restrict__ jq,
                      const double *__restrict__ oq, double *__restrict__ r0,
                      double *__restrict__ r0K, int skipK, const double *__restrict__ bqf) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  constexpr int NQF = D == 3 ? N * N : N;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  int ix[3];
  {
    long r = e;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  double detJ = 1.0;
  for (int j = 0; j < D; j++) detJ *= p.h[j];
  double out[NB], outK[NB];
  for (int i = 0; i < NB; i++) { out[i] = 0.0; outK[i] = 0.0; }
  // volume: -sum_q f_q w_q |J| psi_i(q)
  if (fq || fc) {
    for (int q = 0; q < NB; q++) {
      int qa[3] = {q % N, (q / N) % N, q / (N * N)};
      double f = 0.0;
      if (fq) f += fq[e * NB + q];
      if (fc) f += fc[e];
      double wq = detJ;
      for (int j = 0; j < D; j++) wq *= tb.w[qa[j]];
      const double s = -f * wq;
      for (int i = 0; i < NB; i++) {
        int ia[3] = {i % N, (i / N) % N, i / (N * N)};
        double phi = 1.0;
        for (int j = 0; j < D; j++) phi *= tb.B[qa[j] * N + ia[j]];
        out[i] += s * phi;
      }
    }
  }
  // boundary faces
  for (int f = 0; f < 2 * D; f++) {
    const int dir = f >> 1, hi = f & 1;
    const bool bnd = hi ? ix[dir] == p.nc[dir] - 1 : ix[dir] == 0;
    if (!bnd) continue;
    const double Ke = kdir(p, e, dir);   // (A n).n on this face
    const int bc = p.bc[f];
    if (bc == PDG_BC_NONE) continue;
    // boundary point base index: sides in order, faces lexicographic over the
    // remaining directions, NQF points per face
    long base = 0;
    for (int s = 0; s < f; s++) {
      long cnt = 1;
      for (int j = 0; j < D; j++)
        if (j != (s >> 1)) cnt *= p.nc[j];
      base += cnt * NQF;
    }
    long fidx = 0;
    for (int j = D - 1; j >= 0; j--) {
      if (j == dir) continue;
      fidx = fidx * p.nc[j] + ix[j];
    }
    base += fidx * NQF;
    const double h = p.h[dir];
    const double area = detJ / h;
    const double sgn = hi ? 1.0 : -1.0;
    const double *dface = hi ? tb.d1 : tb.d0;
    const int inode = hi ? N - 1 : 0;
    const double pen = (p.pen_fac / h) * (p.weights == PDG_WEIGHTS_ON ? Ke : 1.0);
    for (int q = 0; q < NQF; q++) {
      int qt[2] = {q % N, q / N};
      double loc[3];
      double wf = area;
      int t = 0;
      for (int j = 0; j < D; j++) {
        if (j == dir) { loc[j] = hi ? 1.0 : 0.0; continue; }
        loc[j] = tb.x[qt[t]];
        wf *= tb.w[qt[t]];
        t++;
      }
      double cv = 0.0, cd = 0.0;   // coefficients of psi and dpsi/dn
      double cvK = 0.0, cdK = 0.0;
      if (bc == PDG_BC_NEUMANN) {
        cv = jq ? jq[base + q] : 0.0;
      } else if (bc == PDG_BC_OUTFLOW) {
        cv = oq ? oq[base + q] : 0.0;
      } else {
        const double g = gq ? gq[base + q] : 0.0;
        double bn = 0.0;
        if (bqf) {
          // velocity given at the face-lattice points
          const long fi = face_lattice_index(p.nc, D, dir, ix[dir] + hi, ix);
          bn = sgn * bqf[(fi * NQF + q) * 3 + dir];
        } else if (vel.nmodes > 0) {
          double xg[3], b[3];
          for (int j = 0; j < D; j++) xg[j] = (ix[j] + loc[j]) * p.h[j];
          velocity_at(vel, D, xg, b);
          bn = sgn * b[dir];
        }
        if (bn < 0.0) cv += g * bn;
        if (!skipK) {
          // with a tensor A these terms come from launch_rhs_general
          cdK = -p.theta * Ke * g;
          cvK = -pen * g;
        }
      }
      for (int i = 0; i < NB; i++) {
        int ia[3] = {i % N, (i / N) % N, i / (N * N)};
        double tang = 1.0;
        t = 0;
        for (int j = 0; j < D; j++) {
          if (j == dir) continue;
          tang *= tb.B[qt[t] * N + ia[j]];
          t++;
        }
        const double val = (ia[dir] == inode ? 1.0 : 0.0) * tang;
        const double dn = sgn * dface[ia[dir]] / h * tang;
        out[i] += wf * (cv * val);
        outK[i] += wf * (cvK * val + cdK * dn);
      }
    }
  }
  for (int i = 0; i < NB; i++) {
    r0[e * NB + i] = out[i] + outK[i];
    if (r0K) r0K[e * NB + i] = outK[i];
  }
}

// ---------------------------------------------------------------------------
// gradient
// ---------------------------------------------------------------------------
template <int D, int N>
__device__ __forceinline__ void contract(const double *mat, int dir, const double *in,
                                         double *out) {
  // out[.., i_dir, ..] = sum_a mat[i][a] in[.., a, ..]
  constexpr int NB = D == 3 ? N * N * N : N * N;
  const int st = dir == 0 ? 1 : (dir == 1 ? N : N * N);
  for (int idx = 0; idx < NB; idx++) {
    const int i = (idx / st) % N;
    const int base = idx - i * st;
    double s = 0.0;
    for (int a = 0; a < N; a++) s += mat[i * N + a] * in[base + a * st];
    out[idx] = s;
  }
}

// traces on the face normal to dir at node layer `layer`: value and the
// xi-derivative with the 1D vector dv, for every face node (tangential
// lexicographic order)
template <int D, int N>
__device__ __forceinline__ void face_trace(const double *u, int dir, int layer, const double *dv,
                                           double *val, double *der) {
  constexpr int NQF = D == 3 ? N * N : N;
  const int st = dir == 0 ? 1 : (dir == 1 ? N : N * N);
  for (int q = 0; q < NQF; q++) {
    int qt[2] = {q % N, q / N};
    int base = 0, t = 0;
    for (int j = 0; j < D; j++) {
      if (j == dir) continue;
      const int sj = j == 0 ? 1 : (j == 1 ? N : N * N);
      base += qt[t] * sj;
      t++;
    }
    val[q] = u[base + layer * st];
    double s = 0.0;
    for (int a = 0; a < N; a++) s += dv[a] * u[base + a * st];
    der[q] = s;
  }
}

template <int D, int N>
__device__ __forceinline__ double face_mass_dot(const double *M, const double *a,
                                                const double *b) {
  // a^T (Mhat (x) Mhat) b over face nodes (D = 3) or a^T Mhat b (D = 2)
  double s = 0.0;
  if (D == 3) {
    for (int i = 0; i < N * N; i++) {
      const int i0 = i % N, i1 = i / N;
      double t = 0.0;
      for (int j = 0; j < N * N; j++) t += M[i0 * N + (j % N)] * M[i1 * N + (j / N)] * b[j];
      s += a[i] * t;
    }
  } else {
    for (int i = 0; i < N; i++) {
      double t = 0.0;
      for (int j = 0; j < N; j++) t += M[i * N + j] * b[j];
      s += a[i] * t;
    }
  }
  return s;
}

template <int D, int N>
__global__ void k_grad_logK(const OpParams<double> p, const double *__restrict__ u,
                            const double *__restrict__ lam, const double *__restrict__ r0K,
                            double *__restrict__ g) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  constexpr int NQF = D == 3 ? N * N : N;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  const double *tM = p.tab, *tS = p.tab + N * N, *td0 = tS + N * N, *td1 = td0 + N;
  int ix[3];
  {
    long r = e;
    ix[0] = (int)(r % p.nc[0]); r /= p.nc[0];
    ix[1] = (int)(r % p.nc[1]); r /= p.nc[1];
    ix[2] = (int)r;
  }
  const long stride[3] = {1, (long)p.nc[0], (long)p.nc[0] * p.nc[1]};
  double ue[NB], le[NB], t1[NB], t2[NB];
  for (int i = 0; i < NB; i++) { ue[i] = u[e * NB + i]; le[i] = lam[e * NB + i]; }
  // volume: sum_dir hperp/h_dir lambda^T (S (x) M (x) M)_dir u
  double vol = 0.0;
  for (int dir = 0; dir < D; dir++) {
    const double *src = ue;
    double *a = t1, *b = t2;
    for (int j = 0; j < D; j++) {
      contract<D, N>(j == dir ? tS : tM, j, src, a);
      src = a;
      double *tmp = a; a = b; b = tmp;
    }
    double hp = 1.0;
    for (int j = 0; j < D; j++)
      if (j != dir) hp *= p.h[j];
    double s = 0.0;
    for (int i = 0; i < NB; i++) s += le[i] * src[i];
    vol += hp / p.h[dir] * s;
  }
  const double Ke = p.K[e];
  double acc = vol;
  double uv[NQF], ud[NQF], ov[NQF], od[NQF], lv[NQF], ld[NQF], mv[NQF], md[NQF];
  double Ju[NQF], Fu[NQF], Jl[NQF], Fl[NQF];
  for (int f = 0; f < 2 * D; f++) {
    const int dir = f >> 1, hi = f & 1;
    long nb;
    if (hi) nb = ix[dir] + 1 < p.nc[dir] ? e + stride[dir] : -1;
    else nb = ix[dir] > 0 ? e - stride[dir] : -1;
    if (nb < 0 && p.bc[f] != PDG_BC_DIRICHLET) continue;
    const double h = p.h[dir];
    const double sgn = hi ? 1.0 : -1.0;     // d/dn = sgn/h d/dxi
    face_trace<D, N>(ue, dir, hi ? N - 1 : 0, hi ? td1 : td0, uv, ud);
    face_trace<D, N>(le, dir, hi ? N - 1 : 0, hi ? td1 : td0, lv, ld);
    double ke, ko, cfac;
    if (nb >= 0) {
      face_trace<D, N>(u + nb * NB, dir, hi ? 0 : N - 1, hi ? td0 : td1, ov, od);
      face_trace<D, N>(lam + nb * NB, dir, hi ? 0 : N - 1, hi ? td0 : td1, mv, md);
      ke = ko = 0.5;
      const double Ko = p.K[nb];
      const double S = Ke + Ko + 1e-20;
      cfac = 2.0 * Ko * (Ko + 1e-20) / (S * S);   // dH/dK_e
    } else {
      for (int q = 0; q < NQF; q++) ov[q] = od[q] = mv[q] = md[q] = 0.0;
      ke = 1.0;
      ko = 0.0;
      cfac = 1.0;
    }
    for (int q = 0; q < NQF; q++) {
      const double dnu = sgn / h * ud[q], dno = sgn / h * od[q];
      const double dnl = sgn / h * ld[q], dnm = sgn / h * md[q];
      Ju[q] = uv[q] - ov[q];
      Fu[q] = -(ke * dnu + ko * dno);
      Jl[q] = lv[q] - mv[q];
      Fl[q] = -(ke * dnl + ko * dnm);
    }
    const double pen1 = p.pen_fac / h;
    double hp = 1.0;
    for (int j = 0; j < D; j++)
      if (j != dir) hp *= p.h[j];
    const double af = hp * (face_mass_dot<D, N>(tM, Jl, Fu) -
                            p.theta * face_mass_dot<D, N>(tM, Ju, Fl) +
                            pen1 * face_mass_dot<D, N>(tM, Ju, Jl));
    acc += cfac * af;
  }
  double out = -Ke * acc;
  if (r0K) {
    double s = 0.0;
    for (int i = 0; i < NB; i++) s += le[i] * r0K[e * NB + i];
    out -= s;
  }
  g[e] = out;
}

template <int D, int N>
__global__ void k_grad_source(long ncell, const RhsTables tb, double detJ,
                              const double *__restrict__ lam, double *__restrict__ g) {
  constexpr int NB = D == 3 ? N * N * N : N * N;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ncell) return;
  double wi[kMaxN1];
  for (int a = 0; a < N; a++) {
    double s = 0.0;
    for (int q = 0; q < N; q++) s += tb.w[q] * tb.B[q * N + a];
    wi[a] = s;
  }
  double s = 0.0;
  for (int i = 0; i < NB; i++) {
    const int ia[3] = {i % N, (i / N) % N, i / (N * N)};
    double v = detJ;
    for (int j = 0; j < D; j++) v *= wi[ia[j]];
    s += lam[e * NB + i] * v;
  }
  g[e] = s;
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------

#define PDG_DISPATCH_DN(ctx, MACRO)                  \
  switch ((ctx)->dim * 10 + (ctx)->k) {              \
    case 21: MACRO(2, 2); break;                     \
    case 22: MACRO(2, 3); break;                     \
    case 23: MACRO(2, 4); break;                     \
    case 24: MACRO(2, 5); break;                     \
    case 31: MACRO(3, 2); break;                     \
    case 32: MACRO(3, 3); break;                     \
    case 33: MACRO(3, 4); break;                     \
    case 34: MACRO(3, 5); break;                     \
    default: return set_error(PDG_EUNSUPPORTED, "dim/degree not compiled in"); \
  }


int launch_rhs(pdg_context *ctx) {
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  RhsTables tb = make_rhs_tables(ctx);
  double *r0K = rhs_r0K(ctx, ctx->gq != nullptr);
  const unsigned blocks = (unsigned)((ctx->ncell + 127) / 128);
#define PDG_RHS(D, N)                                                                       \
  k_rhs<D, N><<<blocks, 128, 0, ctx->stream>>>(p, tb, ctx->vel, ctx->fq, ctx->fc, ctx->gq, \
                                               ctx->jq, ctx->oq, ctx->r0, r0K,                   \
                                               ctx->gen_A == 1 || ctx->gen_A == 2,       \
                                               ctx->vel_points ? ctx->bqf64 : nullptr)
  PDG_DISPATCH_DN(ctx, PDG_RHS);
#undef PDG_RHS
  PDG_CUDA_TRY(cudaGetLastError());
  PDG_TRY(launch_rhs_general(ctx));
  return PDG_OK;
}

int launch_grad_logK(pdg_context *ctx, const double *u, const double *lam, double *g) {
  if (ctx->basis == PDG_BASIS_LEGENDRE) {
    // lambda_L^T dA_L u_L = (T lambda_L)^T dA (T u_L): nodal coefficients
    PDG_TRY(basis_change<double>(ctx, 0, 0, u, ctx->legw64[0], 1.0, 0, nullptr, nullptr));
    PDG_TRY(basis_change<double>(ctx, 0, 0, lam, ctx->legw64[1], 1.0, 0, nullptr, nullptr));
    u = ctx->legw64[0];
    lam = ctx->legw64[1];
  }
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  const double *r0K = rhs_r0K(ctx, false);
  const unsigned blocks = (unsigned)((ctx->ncell + 63) / 64);
#define PDG_GRAD(D, N) \
  k_grad_logK<D, N><<<blocks, 64, 0, ctx->stream>>>(p, u, lam, r0K, g)
  PDG_DISPATCH_DN(ctx, PDG_GRAD);
#undef PDG_GRAD
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int launch_grad_source(pdg_context *ctx, const double *lam, double *g) {
  if (ctx->basis == PDG_BASIS_LEGENDRE) {
    PDG_TRY(basis_change<double>(ctx, 0, 0, lam, ctx->legw64[1], 1.0, 0, nullptr, nullptr));
    lam = ctx->legw64[1];
  }
  RhsTables tb = make_rhs_tables(ctx);
  double detJ = 1.0;
  for (int j = 0; j < ctx->dim; j++) detJ *= ctx->h[j];
  const unsigned blocks = (unsigned)((ctx->ncell + 127) / 128);
#define PDG_GS(D, N) \
  k_grad_source<D, N><<<blocks, 128, 0, ctx->stream>>>(ctx->ncell, tb, detJ, lam, g)
  PDG_DISPATCH_DN(ctx, PDG_GS);
#undef PDG_GS
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

}  // namespace pdg
