// pdg_apply32.cu -- the FP32 cell operator of the mixed-precision inner
// solve (3D, degrees 1 and 2), laid out for shared-memory throughput.
//
// Same operator as k_apply (pdg_apply.cu; reference: ConvectionDiffusionDG::
// jacobian_apply_volume / _skeleton / _boundary, localoperator/
// convectiondiffusiondg.hh:191-195, 474-481, 892-899) in the Kronecker form
//   y_e = sum_dir (A'_dir (x) Mhat (x) Mhat)_dir u_e + neighbour couplings,
// with A'_dir and the face coefficients read from a per-cell FP32 record
// (built from the FP64 arithmetic once per coefficient field).
//
// Layout.  A CTA owns CPB consecutive cells.  Its own cells (plus one halo
// cell each side, the x-neighbours) and the four runs of y- and
// z-neighbour cells (cells e -/+ nx and e -/+ nx*ny of a consecutive run
// are consecutive runs as well) are copied into shared memory with
// coalesced loads, so every cell value crosses the L1 once per CTA.  Each
// thread then owns one z-plane of one cell (N threads per cell): the x and y
// contractions of its plane run in registers, the z contractions read the
// other planes from shared memory.
//
//   stage 1 (plane z, registers):
//     X = A'_x u_z + x-face terms,     P  = Mhat_y X
//     Y = A'_y u_z + y-face terms,     P += Mhat_x Y
//   stage 2 (after P is shared):
//     Z   = sum_z' A'_z[z][z'] u_z' + z-face terms
//     out = (Mhat_y (x) Mhat_x) Z + sum_z' Mhat_z[z][z'] P_z'
//
// The output is staged in shared memory and written back coalesced.
#include <cstdint>
#include <mutex>

#include "pdg_internal.cuh"

namespace pdg {

// 1D tables by value (kernel parameter space)
struct EdgeTab {
  float M[kMaxN1 * kMaxN1];
  float d0[kMaxN1], d1[kMaxN1];
};

template <int N>
struct P32Cfg {
  static constexpr int N2 = N * N, NB = N * N * N;
  static constexpr int CPB = 128 / N;                 // cells per CTA
  static constexpr int THREADS = CPB * N;
  static constexpr int REC = 3 * N2 + 30;             // A'_x, A'_y, A'_z, 5 per face
  // shared floats: own run (CPB+2 cells), 4 neighbour runs, P, records;
  // the staged runs carry 4 floats of slack (16-byte phase of their source)
  static constexpr int OWN = (CPB + 2) * NB;
  static constexpr int RUN = CPB * NB;
  static constexpr int OWNP = (OWN + 4 + 3) / 4 * 4, RUNP = (RUN + 4 + 3) / 4 * 4;
  static constexpr int RECP = (CPB * REC + 4 + 3) / 4 * 4;
  static constexpr int RUN4 = (RUN + 3) / 4 * 4;       // P, keeps RS 16-byte aligned
  static constexpr int SMEM = OWNP + 4 * RUNP + RUN4 + RECP;
};

// face coupling of a neighbour trace (val, dv) into (s1, s2); cf = {hp ke,
// hp ko, hp pen, th hp ke, th hp ko} of the face, `hi` = upper face
__device__ __forceinline__ void face_s(const float *cf, bool hi, bool tr, float val, float dv,
                                       float &s1, float &s2) {
  if (!hi) {
    if (!tr) { s1 = cf[1] * dv - cf[2] * val; s2 = cf[3] * val; }
    else { s1 = -cf[2] * val - cf[4] * dv; s2 = -cf[0] * val; }
  } else {
    if (!tr) { s1 = -cf[1] * dv - cf[2] * val; s2 = -cf[3] * val; }
    else { s1 = -cf[2] * val + cf[4] * dv; s2 = cf[0] * val; }
  }
}

__device__ __forceinline__ void coords32(const OpParams<float> &p, unsigned e, int *ix) {
  const unsigned q0 = p.div0.div(e);
  const unsigned q1 = p.div1.div(q0);
  ix[0] = (int)(e - q0 * (unsigned)p.nc[0]);
  ix[1] = (int)(q0 - q1 * (unsigned)p.nc[1]);
  ix[2] = (int)q1;
}

template <int N>
__global__ void __launch_bounds__(P32Cfg<N>::THREADS)
    k_apply32(const OpParams<float> p, const ApplyArgs<float> a, const float *__restrict__ rec,
              const EdgeTab tb) {
  using C = P32Cfg<N>;
  constexpr int N2 = C::N2, NB = C::NB, CPB = C::CPB, REC = C::REC;
  extern __shared__ __align__(16) float sm[];
  if (a.skip && *a.skip) return;
  float *OWN0 = sm;                    // cells e0-1 .. e0+CPB
  float *YL0 = OWN0 + C::OWNP;         // cells e - nx
  float *YH0 = YL0 + C::RUNP;          // cells e + nx
  float *ZL0 = YH0 + C::RUNP;          // cells e - nx ny
  float *ZH0 = ZL0 + C::RUNP;          // cells e + nx ny
  float *PS = ZH0 + C::RUNP;           // stage-1 planes P
  float *RS0 = PS + C::RUN4;           // records

  const long e0 = (long)blockIdx.x * CPB;
  const long ncell = p.ncell;
  const long ndof = ncell * NB;
  const long sx = p.nc[0], sxy = (long)p.nc[0] * p.nc[1];
  const float *__restrict__ x = a.x;
  const bool coupled = !a.diag_only;

  // ---- coalesced staging: asynchronous global -> shared copies (cp.async),
  // all in flight at once, one wait before the barrier.  A run of source
  // elements [g0, g0+count) lands at dst[ph + i] with ph = g0 mod 4, so that
  // source and destination share their 16-byte phase and whole 16-byte
  // chunks are copied; chunks that reach outside [0, lim) go element-wise.
  // Returns the run's base pointer (dst + ph). ----
  auto stage = [&](float *dst, const float *src, long g0, long lim, int count,
                   bool on) -> float * {
    const int ph = (int)(((g0 % 4) + 4) % 4);
    const long ga = g0 - ph;
    const int nch = (ph + count + 3) / 4;
    const bool vec_ok = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    for (int c = threadIdx.x; c < nch; c += C::THREADS) {
      const long gc = ga + 4L * c;
      if (on && vec_ok && gc >= 0 && gc + 4 <= lim) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + 4 * c);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + gc)
                     : "memory");
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const long g = gc + j;
          dst[4 * c + j] = (on && g >= 0 && g < lim) ? src[g] : 0.f;
        }
      }
    }
    return dst + ph;
  };
  float *OWN = stage(OWN0, x, (e0 - 1) * NB, ndof, C::OWN, true);
  float *YL = stage(YL0, x, (e0 - sx) * NB, ndof, C::RUN, coupled);
  float *YH = stage(YH0, x, (e0 + sx) * NB, ndof, C::RUN, coupled);
  float *ZL = stage(ZL0, x, (e0 - sxy) * NB, ndof, C::RUN, coupled);
  float *ZH = stage(ZH0, x, (e0 + sxy) * NB, ndof, C::RUN, coupled);
  float *RS = stage(RS0, rec, e0 * REC, ncell * REC, CPB * REC, true);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  const int t = threadIdx.x, cs = t / N, z = t - cs * N;
  const long e = e0 + cs;
  const bool active = e < ncell;
  int ix[3];
  coords32(p, (unsigned)(active ? e : 0), ix);
  const bool has[6] = {coupled && ix[0] > 0, coupled && ix[0] + 1 < p.nc[0],
                       coupled && ix[1] > 0, coupled && ix[1] + 1 < p.nc[1],
                       coupled && ix[2] > 0, coupled && ix[2] + 1 < p.nc[2]};
  const bool tr = a.transpose != 0;
  const float *R = RS + cs * REC;
  const float *cf = R + 3 * N2;
  auto A = [&](int dir, int i, int q) -> float {
    return R[dir * N2 + (tr ? q * N + i : i * N + q)];
  };
  const float *U = OWN + (cs + 1) * NB;           // this cell
  const float *UXL = OWN + cs * NB;               // x-lower neighbour (if has[0])
  const float *UXH = OWN + (cs + 2) * NB;
  const float *UYL = YL + cs * NB, *UYH = YH + cs * NB;
  const float *UZL = ZL + cs * NB, *UZH = ZH + cs * NB;

  // ---- stage 1: plane z ----
  float u[N][N];
#pragma unroll
  for (int y = 0; y < N; y++)
#pragma unroll
    for (int xx = 0; xx < N; xx++) u[y][xx] = U[z * N2 + y * N + xx];

  // x faces: per row y the neighbour's x-line at (y, z)
  float xs1l[N], xs2l[N], xs1h[N], xs2h[N];
#pragma unroll
  for (int y = 0; y < N; y++) {
    float dvl = 0.f, dvh = 0.f;
#pragma unroll
    for (int q = 0; q < N; q++) {
      dvl += tb.d1[q] * UXL[z * N2 + y * N + q];
      dvh += tb.d0[q] * UXH[z * N2 + y * N + q];
    }
    const float vl = UXL[z * N2 + y * N + N - 1], vh = UXH[z * N2 + y * N];
    face_s(cf + 0, false, tr, vl, dvl, xs1l[y], xs2l[y]);
    face_s(cf + 5, true, tr, vh, dvh, xs1h[y], xs2h[y]);
    if (!has[0]) { xs1l[y] = 0.f; xs2l[y] = 0.f; }
    if (!has[1]) { xs1h[y] = 0.f; xs2h[y] = 0.f; }
  }
  // y faces: per column x the neighbour's y-line at (x, z)
  float ys1l[N], ys2l[N], ys1h[N], ys2h[N];
#pragma unroll
  for (int xx = 0; xx < N; xx++) {
    float dvl = 0.f, dvh = 0.f;
#pragma unroll
    for (int q = 0; q < N; q++) {
      dvl += tb.d1[q] * UYL[z * N2 + q * N + xx];
      dvh += tb.d0[q] * UYH[z * N2 + q * N + xx];
    }
    const float vl = UYL[z * N2 + (N - 1) * N + xx], vh = UYH[z * N2 + xx];
    face_s(cf + 10, false, tr, vl, dvl, ys1l[xx], ys2l[xx]);
    face_s(cf + 15, true, tr, vh, dvh, ys1h[xx], ys2h[xx]);
    if (!has[2]) { ys1l[xx] = 0.f; ys2l[xx] = 0.f; }
    if (!has[3]) { ys1h[xx] = 0.f; ys2h[xx] = 0.f; }
  }

  float P[N][N];
  {
    // X = A'_x u + x faces ; P = Mhat_y X
    float X[N][N];
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xx = 0; xx < N; xx++) {
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < N; q++) s += A(0, xx, q) * u[y][q];
        if (xx == 0) s += xs1l[y];
        s += tb.d0[xx] * xs2l[y];
        if (xx == N - 1) s += xs1h[y];
        s += tb.d1[xx] * xs2h[y];
        X[y][xx] = s;
      }
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xx = 0; xx < N; xx++) {
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < N; r++) s += tb.M[y * N + r] * X[r][xx];
        P[y][xx] = s;
      }
  }
  {
    // Y = A'_y u + y faces ; P += Mhat_x Y
    float Y[N][N];
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xx = 0; xx < N; xx++) {
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < N; q++) s += A(1, y, q) * u[q][xx];
        if (y == 0) s += ys1l[xx];
        s += tb.d0[y] * ys2l[xx];
        if (y == N - 1) s += ys1h[xx];
        s += tb.d1[y] * ys2h[xx];
        Y[y][xx] = s;
      }
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xx = 0; xx < N; xx++) {
        float s = P[y][xx];
#pragma unroll
        for (int r = 0; r < N; r++) s += tb.M[xx * N + r] * Y[y][r];
        P[y][xx] = s;
      }
  }
  float *Pc = PS + cs * NB;
#pragma unroll
  for (int y = 0; y < N; y++)
#pragma unroll
    for (int xx = 0; xx < N; xx++) Pc[z * N2 + y * N + xx] = P[y][xx];
  __syncthreads();

  // ---- stage 2: z contractions ----
  float Zp[N][N];
#pragma unroll
  for (int y = 0; y < N; y++)
#pragma unroll
    for (int xx = 0; xx < N; xx++) {
      const int o = y * N + xx;
      float s = 0.f;
#pragma unroll
      for (int q = 0; q < N; q++) s += A(2, z, q) * U[q * N2 + o];
      // z faces at face point (x, y)
      float dvl = 0.f, dvh = 0.f;
#pragma unroll
      for (int q = 0; q < N; q++) {
        dvl += tb.d1[q] * UZL[q * N2 + o];
        dvh += tb.d0[q] * UZH[q * N2 + o];
      }
      float s1, s2;
      if (has[4]) {
        face_s(cf + 20, false, tr, UZL[(N - 1) * N2 + o], dvl, s1, s2);
        if (z == 0) s += s1;
        s += tb.d0[z] * s2;
      }
      if (has[5]) {
        face_s(cf + 25, true, tr, UZH[o], dvh, s1, s2);
        if (z == N - 1) s += s1;
        s += tb.d1[z] * s2;
      }
      Zp[y][xx] = s;
    }
  float out[N][N];
  {
    float T1[N][N];   // Mhat_x along x
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xx = 0; xx < N; xx++) {
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < N; r++) s += tb.M[xx * N + r] * Zp[y][r];
        T1[y][xx] = s;
      }
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int xx = 0; xx < N; xx++) {
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < N; r++) s += tb.M[y * N + r] * T1[r][xx];
#pragma unroll
        for (int q = 0; q < N; q++) s += tb.M[z * N + q] * Pc[q * N2 + y * N + xx];
        out[y][xx] = s;
      }
  }

  // ---- coalesced write-back through shared memory (the YL run is free) ----
  __syncthreads();
  float *O = YL0;
#pragma unroll
  for (int y = 0; y < N; y++)
#pragma unroll
    for (int xx = 0; xx < N; xx++) O[cs * NB + z * N2 + y * N + xx] = out[y][xx];
  __syncthreads();
  const long ob = e0 * NB;
  const float alpha = a.alpha;
  for (int i = threadIdx.x; i < C::RUN; i += C::THREADS) {
    const long g = ob + i;
    if (g >= ndof) break;
    float r = alpha * O[i];
    if (a.accumulate) r += a.y[g];
    if (a.add) r += a.add[g];
    a.y[g] = r;
  }
}

static EdgeTab make_edge_tab_uncached(const pdg_context *ctx) {
  EdgeTab t{};
  const RhsTables r = make_rhs_tables(ctx);
  const int N = ctx->N;
  // Mhat on [0,1]: sum_q w_q phi_i(x_q) phi_j(x_q) (exact for degree 2k)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double s = 0.0;
      for (int q = 0; q < N; q++) s += r.w[q] * r.B[q * N + i] * r.B[q * N + j];
      t.M[i * N + j] = (float)s;
    }
  for (int i = 0; i < N; i++) {
    t.d0[i] = (float)r.d0[i];
    t.d1[i] = (float)r.d1[i];
  }
  return t;
}

// the tables depend on the degree and the nodal basis only: built once each
static const EdgeTab &edge_tab(const pdg_context *ctx) {
  static std::mutex mu;
  static EdgeTab tabs[3][kMaxN1 + 1];
  static bool ready[3][kMaxN1 + 1] = {};
  std::lock_guard<std::mutex> lock(mu);
  const int b = ctx->basis;
  if (!ready[b][ctx->N]) {
    tabs[b][ctx->N] = make_edge_tab_uncached(ctx);
    ready[b][ctx->N] = true;
  }
  return tabs[b][ctx->N];
}

template <int N>
static int launch32_n(pdg_context *ctx, const ApplyArgs<float> &a, const OpParams<float> &p,
                      const float *rec) {
  using C = P32Cfg<N>;
  const size_t smem = sizeof(float) * C::SMEM;
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_dev = ctx->device;
  }
  const EdgeTab &tb = edge_tab(ctx);
  const unsigned blocks = (unsigned)((ctx->ncell + C::CPB - 1) / C::CPB);
  k_apply32<N><<<blocks, C::THREADS, smem, ctx->stream>>>(p, a, rec, tb);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int launch_apply32_3d(pdg_context *ctx, const ApplyArgs<float> &a, const OpParams<float> &p,
                      const float *rec) {
  switch (ctx->N) {
    case 2: return launch32_n<2>(ctx, a, p, rec);
    case 3: return launch32_n<3>(ctx, a, p, rec);
    default: return set_error(PDG_EUNSUPPORTED, "staged FP32 kernel: degree 1 or 2 only");
  }
}

}  // namespace pdg
