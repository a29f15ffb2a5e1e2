// pdg_apply32.cu -- the FP32 cell operator of the mixed-precision inner
// solve (3D, degrees 1 to 3), laid out for shared-memory throughput.
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
#include <cuda.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "pdg_tma.cuh"
#include "pdg_vec.cuh"

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
  float part = 0.f;
  for (int i = threadIdx.x; i < C::RUN; i += C::THREADS) {
    const long g = ob + i;
    if (g >= ndof) break;
    float r = alpha * O[i];
    if (a.accumulate) r += a.y[g];
    if (a.add) r += a.add[g];
    a.y[g] = r;
    part += OWN[NB + i] * r;
  }
  if (a.dot_part)
    reduce_tail_grouped<128>(a.dot_part, a.dot_max_blocks, a.dot_cnt,
                             RedCtx{nullptr, a.dot_scal, a.dot_flags}, (double)part, 0.0,
                             a.dot_fin, -1, -1);
}


// ---------------------------------------------------------------------------
// Q3 (N = 4) variant.  A row of a cell (4 floats along x at fixed y, z) is one
// 16-byte vector, so every exchange goes through 128-bit shared accesses.
// Staged runs are stored with the row swizzle swz(), the 128-byte pattern of
// the tensor memory accelerator (16-byte chunk c of 128-byte line L at chunk
// c ^ (L mod 8), buffers 1024-byte aligned): a quarter warp (two cells x four
// planes) then reads eight distinct 16-byte bank groups for every row pattern
// of the kernel (own / neighbour planes, all planes of one row, P planes), and
// consecutive staging stores stay conflict-free.  With 16-byte aligned
// vectors the runs are loaded by TMA tensor copies (the vector as a 2D tensor
// of 128-byte lines; lines outside it read as zeros) and the record run by a
// bulk copy, all completing on one mbarrier.
// The z faces are not staged: thread z loads row y = z of the four planes of
// each z neighbour straight from global memory (64 contiguous bytes per cell),
// forms the face terms of the face points of that row and hands them to the
// other planes through a small shared array.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int swz(int r) { return (r & ~7) | ((r & 7) ^ ((r >> 3) & 7)); }

struct Q3Cfg {
  static constexpr int N = 4, N2 = 16, NB = 64, CPB = 32, THREADS = 128;
  static constexpr int REC = 3 * N2 + 30;
  // shared layout in 16-byte rows; once the y-neighbour rows are read, the
  // P planes reuse the YL run and the z-face terms (FS rows) the YH run
  static constexpr int OWN = (CPB + 2) * 16, RUN = CPB * 16, FS = 4 * CPB * 4;
  static constexpr int RECR = (CPB * REC + 4 + 3) / 4;   // records (+ phase slack)
  // byte offsets from a 1024-byte aligned base (the swizzle atom)
  static constexpr int OWN_B = 0, OWN_BYTES = (OWN * 16 + 1023) / 1024 * 1024;
  static constexpr int YL_B = OWN_B + OWN_BYTES, YH_B = YL_B + RUN * 16;
  static constexpr int REC_B = YH_B + RUN * 16;
  static constexpr int SMEM = 1024 + REC_B + RECR * 16;   // + alignment slack
  static constexpr int LINES_OWN = (CPB + 2) * 2, LINES_RUN = CPB * 2;   // 128-byte lines
  static_assert(FS <= RUN, "z-face terms must fit the YH run");
  static_assert((RUN * 16) % 1024 == 0, "runs must keep the 1024-byte alignment");
};


__device__ __forceinline__ float4 ld4(const float *p, bool vec) {
  if (vec) return *reinterpret_cast<const float4 *>(p);
  return make_float4(p[0], p[1], p[2], p[3]);
}

// 5 blocks of 128 threads per SM (96 registers; 35 KB of shared memory each):
// with the z-neighbour rows loaded before the staging wait, 325 us at 96^3 Q3,
// against 334 us with those loads after stage 1 at 6 blocks per SM (80
// registers), 350 us at 4 blocks and 351 us with the compiler's free register
// choice; 378 us without the aliased runs
template <bool kTma>
__global__ void __launch_bounds__(Q3Cfg::THREADS, 5)
    k_apply32_q3(const OpParams<float> p, const ApplyArgs<float> a, const float *__restrict__ rec,
                 const EdgeTab tb, const __grid_constant__ CUtensorMap map_own,
                 const __grid_constant__ CUtensorMap map_run, int *tma_err) {
  using C = Q3Cfg;
  constexpr int N = 4, N2 = 16, NB = 64, CPB = C::CPB, REC = C::REC;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) unsigned long long stage_bar;
  if (a.skip && *a.skip) return;
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smraw) + 1023) & ~static_cast<uintptr_t>(1023));
  float4 *OWN = reinterpret_cast<float4 *>(base + C::OWN_B);   // cells e0-1 .. e0+CPB
  float4 *YL = reinterpret_cast<float4 *>(base + C::YL_B);     // cells e - nx; then P
  float4 *YH = reinterpret_cast<float4 *>(base + C::YH_B);     // cells e + nx; then z faces
  float4 *PS = YL;                   // [cell][plane][row], swizzled
  float4 *FS = YH;                   // [lo s1, lo s2, hi s1, hi s2][cell][row]
  float *RS0 = reinterpret_cast<float *>(base + C::REC_B);

  const long e0 = (long)blockIdx.x * CPB;
  const long ncell = p.ncell;
  const long sx = p.nc[0], sxy = (long)p.nc[0] * p.nc[1];
  const float *__restrict__ x = a.x;
  const bool coupled = !a.diag_only;
  const bool vec = (reinterpret_cast<uintptr_t>(x) & 15) == 0;
  const int t = threadIdx.x, cs = t >> 2, z = t & 3;
  const long e = e0 + cs;
  const bool active = e < ncell;
  const long ee = active ? e : 0;
  int ix[3];
  coords32(p, (unsigned)ee, ix);
  const bool has[6] = {coupled && ix[0] > 0, coupled && ix[0] + 1 < p.nc[0],
                       coupled && ix[1] > 0, coupled && ix[1] + 1 < p.nc[1],
                       coupled && ix[2] > 0, coupled && ix[2] + 1 < p.nc[2]};
  const bool tr = a.transpose != 0;
  // the z-neighbour rows (plane q, row y = z of each z neighbour) come straight
  // from global memory; issued before the staging wait so that their latency
  // overlaps the staging copies and stage 1
  float4 zl[N], zh[N];
#pragma unroll
  for (int q = 0; q < N; q++) {
    zl[q] = has[4] ? ld4(x + (ee - sxy) * NB + q * N2 + z * N, vec)
                   : make_float4(0.f, 0.f, 0.f, 0.f);
    zh[q] = has[5] ? ld4(x + (ee + sxy) * NB + q * N2 + z * N, vec)
                   : make_float4(0.f, 0.f, 0.f, 0.f);
  }

  // rows of cells [c0, c0 + ncells) into dst (swizzled); absent cells read 0
  auto stage_rows = [&](float4 *dst, long c0, int ncells, bool on) {
    for (int r = threadIdx.x; r < ncells * 16; r += C::THREADS) {
      const long cell = c0 + (r >> 4);
      float4 *d = dst + swz(r);
      if (on && cell >= 0 && cell < ncell) {
        const float *src = x + cell * NB + (r & 15) * 4;
        if (vec) {
          const unsigned sa = (unsigned)__cvta_generic_to_shared(d);
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src)
                       : "memory");
        } else {
          *d = make_float4(src[0], src[1], src[2], src[3]);
        }
      } else {
        *d = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
  };
  float *RS = RS0;
  if constexpr (kTma) {
    // one elected thread issues the copies; everyone waits on the barrier
    const unsigned bar = smem_u32(&stage_bar);
    const long ncp = ncell - e0 < CPB ? ncell - e0 : CPB;
    const unsigned rbytes = (unsigned)((ncp * REC * 4 + 15) / 16 * 16);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned lines = (unsigned)C::LINES_OWN + (coupled ? 2u * C::LINES_RUN : 0u);
      mbar_expect_tx(bar, lines * 128u + rbytes);
      tma_load_2d(smem_u32(OWN), &map_own, 0, (int)((e0 - 1) * 2), bar);
      if (coupled) {
        tma_load_2d(smem_u32(YL), &map_run, 0, (int)((e0 - sx) * 2), bar);
        tma_load_2d(smem_u32(YH), &map_run, 0, (int)((e0 + sx) * 2), bar);
      }
      bulk_load(smem_u32(RS0), rec + e0 * REC, rbytes, bar);
    }
    if (!mbar_wait(bar, 0, kTmaPolls)) {
      // record the failure, give the copies a last chance to land, leave
      if (threadIdx.x == 0) atomicExch(tma_err, 1);
      mbar_wait(bar, 0, kTmaPolls);
      return;
    }
  } else {
  stage_rows(OWN, e0 - 1, CPB + 2, true);
  stage_rows(YL, e0 - sx, CPB, coupled);
  stage_rows(YH, e0 + sx, CPB, coupled);
  {
    // records: one contiguous run, copied in 16-byte chunks in phase with
    // their source (element-wise where a chunk leaves the array)
    const long g0 = e0 * REC, lim = ncell * REC;
    const int ph = (int)(g0 & 3);
    const long ga = g0 - ph;
    const int nch = (ph + CPB * REC + 3) / 4;
    const bool rvec = (reinterpret_cast<uintptr_t>(rec) & 15) == 0;
    for (int c = threadIdx.x; c < nch; c += C::THREADS) {
      const long gc = ga + 4L * c;
      if (rvec && gc >= 0 && gc + 4 <= lim) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(RS0 + 4 * c);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(rec + gc)
                     : "memory");
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const long g = gc + j;
          RS0[4 * c + j] = (g >= 0 && g < lim) ? rec[g] : 0.f;
        }
      }
    }
    RS = RS0 + ph;
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  }


  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();

  const float *R = RS + cs * REC;
  const float *cf = R + 3 * N2;
  auto A = [&](int dir, int i, int q) -> float {
    return R[dir * N2 + (tr ? q * N + i : i * N + q)];
  };
  auto row = [](const float4 &v, int i) -> float {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
  };

  // ---- stage 1: plane z ----
  float u[N][N];
#pragma unroll
  for (int y = 0; y < N; y++) {
    const float4 v = OWN[swz((cs + 1) * 16 + z * 4 + y)];
    u[y][0] = v.x; u[y][1] = v.y; u[y][2] = v.z; u[y][3] = v.w;
  }
  float xs1l[N], xs2l[N], xs1h[N], xs2h[N];
#pragma unroll
  for (int y = 0; y < N; y++) {
    const float4 l = OWN[swz(cs * 16 + z * 4 + y)];
    const float4 h = OWN[swz((cs + 2) * 16 + z * 4 + y)];
    const float dvl = tb.d1[0] * l.x + tb.d1[1] * l.y + tb.d1[2] * l.z + tb.d1[3] * l.w;
    const float dvh = tb.d0[0] * h.x + tb.d0[1] * h.y + tb.d0[2] * h.z + tb.d0[3] * h.w;
    face_s(cf + 0, false, tr, l.w, dvl, xs1l[y], xs2l[y]);
    face_s(cf + 5, true, tr, h.x, dvh, xs1h[y], xs2h[y]);
    if (!has[0]) { xs1l[y] = 0.f; xs2l[y] = 0.f; }
    if (!has[1]) { xs1h[y] = 0.f; xs2h[y] = 0.f; }
  }
  float ys1l[N], ys2l[N], ys1h[N], ys2h[N];
  {
    float yl[N][N], yh[N][N];
#pragma unroll
    for (int y = 0; y < N; y++) {
      const float4 l = YL[swz(cs * 16 + z * 4 + y)];
      const float4 h = YH[swz(cs * 16 + z * 4 + y)];
      yl[y][0] = l.x; yl[y][1] = l.y; yl[y][2] = l.z; yl[y][3] = l.w;
      yh[y][0] = h.x; yh[y][1] = h.y; yh[y][2] = h.z; yh[y][3] = h.w;
    }
#pragma unroll
    for (int xx = 0; xx < N; xx++) {
      float dvl = 0.f, dvh = 0.f;
#pragma unroll
      for (int q = 0; q < N; q++) {
        dvl += tb.d1[q] * yl[q][xx];
        dvh += tb.d0[q] * yh[q][xx];
      }
      face_s(cf + 10, false, tr, yl[N - 1][xx], dvl, ys1l[xx], ys2l[xx]);
      face_s(cf + 15, true, tr, yh[0][xx], dvh, ys1h[xx], ys2h[xx]);
      if (!has[2]) { ys1l[xx] = 0.f; ys2l[xx] = 0.f; }
      if (!has[3]) { ys1h[xx] = 0.f; ys2h[xx] = 0.f; }
    }
  }
  // every thread has read its y-neighbour rows: YL and YH are free
  __syncthreads();

  // ---- z faces of the face points of row z ----
  {
    // z-neighbour rows (plane q, row z) straight from global memory
    float s1l[N], s2l[N], s1h[N], s2h[N];
#pragma unroll
    for (int xx = 0; xx < N; xx++) {
      float dvl = 0.f, dvh = 0.f;
#pragma unroll
      for (int q = 0; q < N; q++) {
        dvl += tb.d1[q] * row(zl[q], xx);
        dvh += tb.d0[q] * row(zh[q], xx);
      }
      face_s(cf + 20, false, tr, row(zl[N - 1], xx), dvl, s1l[xx], s2l[xx]);
      face_s(cf + 25, true, tr, row(zh[0], xx), dvh, s1h[xx], s2h[xx]);
      if (!has[4]) { s1l[xx] = 0.f; s2l[xx] = 0.f; }
      if (!has[5]) { s1h[xx] = 0.f; s2h[xx] = 0.f; }
    }
    FS[(0 * CPB + cs) * 4 + z] = make_float4(s1l[0], s1l[1], s1l[2], s1l[3]);
    FS[(1 * CPB + cs) * 4 + z] = make_float4(s2l[0], s2l[1], s2l[2], s2l[3]);
    FS[(2 * CPB + cs) * 4 + z] = make_float4(s1h[0], s1h[1], s1h[2], s1h[3]);
    FS[(3 * CPB + cs) * 4 + z] = make_float4(s2h[0], s2h[1], s2h[2], s2h[3]);
  }

  float P[N][N];
  {
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
#pragma unroll
  for (int y = 0; y < N; y++)
    PS[swz(cs * 16 + z * 4 + y)] = make_float4(P[y][0], P[y][1], P[y][2], P[y][3]);
  __syncthreads();

  // ---- stage 2: z contractions ----
  float Zp[N][N];
  {
    float az[N];
#pragma unroll
    for (int q = 0; q < N; q++) az[q] = A(2, z, q);
    const float d0z = tb.d0[z], d1z = tb.d1[z];
#pragma unroll
    for (int y = 0; y < N; y++) {
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int q = 0; q < N; q++) {
        const float4 v = OWN[swz((cs + 1) * 16 + q * 4 + y)];
        acc.x += az[q] * v.x; acc.y += az[q] * v.y; acc.z += az[q] * v.z; acc.w += az[q] * v.w;
      }
      const float4 s2l = FS[(1 * CPB + cs) * 4 + y], s2h = FS[(3 * CPB + cs) * 4 + y];
      acc.x += d0z * s2l.x + d1z * s2h.x;
      acc.y += d0z * s2l.y + d1z * s2h.y;
      acc.z += d0z * s2l.z + d1z * s2h.z;
      acc.w += d0z * s2l.w + d1z * s2h.w;
      if (z == 0) {
        const float4 s1 = FS[(0 * CPB + cs) * 4 + y];
        acc.x += s1.x; acc.y += s1.y; acc.z += s1.z; acc.w += s1.w;
      }
      if (z == N - 1) {
        const float4 s1 = FS[(2 * CPB + cs) * 4 + y];
        acc.x += s1.x; acc.y += s1.y; acc.z += s1.z; acc.w += s1.w;
      }
      Zp[y][0] = acc.x; Zp[y][1] = acc.y; Zp[y][2] = acc.z; Zp[y][3] = acc.w;
    }
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
    float mz[N];
#pragma unroll
    for (int q = 0; q < N; q++) mz[q] = tb.M[z * N + q];
#pragma unroll
    for (int y = 0; y < N; y++) {
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int q = 0; q < N; q++) {
        const float4 v = PS[swz(cs * 16 + q * 4 + y)];
        acc.x += mz[q] * v.x; acc.y += mz[q] * v.y; acc.z += mz[q] * v.z; acc.w += mz[q] * v.w;
      }
#pragma unroll
      for (int r = 0; r < N; r++) {
        const float m = tb.M[y * N + r];
        acc.x += m * T1[r][0]; acc.y += m * T1[r][1]; acc.z += m * T1[r][2]; acc.w += m * T1[r][3];
      }
      out[y][0] = acc.x; out[y][1] = acc.y; out[y][2] = acc.z; out[y][3] = acc.w;
    }
  }

  // ---- coalesced write-back through shared memory (the YL run is free) ----
  __syncthreads();
#pragma unroll
  for (int y = 0; y < N; y++)
    YL[swz(cs * 16 + z * 4 + y)] = make_float4(out[y][0], out[y][1], out[y][2], out[y][3]);
  __syncthreads();
  const long ob = e0 * NB;
  const long ndof = ncell * NB;
  const float alpha = a.alpha;
  const bool yvec = ((reinterpret_cast<uintptr_t>(a.y) | reinterpret_cast<uintptr_t>(a.add)) & 15) == 0;
  float part = 0.f;
  for (int r = threadIdx.x; r < C::RUN; r += C::THREADS) {
    const long g = ob + 4L * r;
    if (g >= ndof) break;
    const float4 o = YL[swz(r)];
    const float4 pin = OWN[swz(16 + r)];
    float4 v = make_float4(alpha * o.x, alpha * o.y, alpha * o.z, alpha * o.w);
    if (yvec) {
      float4 *yp = reinterpret_cast<float4 *>(a.y + g);
      if (a.accumulate) {
        const float4 w = *yp;
        v.x += w.x; v.y += w.y; v.z += w.z; v.w += w.w;
      }
      if (a.add) {
        const float4 w = *reinterpret_cast<const float4 *>(a.add + g);
        v.x += w.x; v.y += w.y; v.z += w.z; v.w += w.w;
      }
      *yp = v;
    } else {
      float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        float rr = vv[j];
        if (a.accumulate) rr += a.y[g + j];
        if (a.add) rr += a.add[g + j];
        a.y[g + j] = rr;
        vv[j] = rr;
      }
      v = make_float4(vv[0], vv[1], vv[2], vv[3]);
    }
    part += pin.x * v.x + pin.y * v.y + pin.z * v.z + pin.w * v.w;
  }
  // block sums in the YH run (its z-face terms were consumed in stage 2): no
  // static shared arrays, six blocks per SM
  if (a.dot_part)
    reduce_tail_grouped<Q3Cfg::THREADS, true>(
        a.dot_part, a.dot_max_blocks, a.dot_cnt, RedCtx{nullptr, a.dot_scal, a.dot_flags},
        (double)part, 0.0, a.dot_fin, -1, -1, reinterpret_cast<double *>(YH));
}

// ---------------------------------------------------------------------------
// Q3 kernel with phase-aliased shared memory (the TMA path of coupled
// applies).  Same staging and the same arithmetic as k_apply32_q3, with the
// address arithmetic and the data exchanges reorganised:
//  * record of 84 floats per cell (A'_x column-major, A'_y, A'_z row-major, the five
//    coupling coefficients of each face, zero where the face has no
//    neighbour, 6 floats of padding) read as 16-byte vectors; the neighbour
//    couplings need no per-face predicates;
//  * the swizzled row of (cell c, plane z, row y) is
//      16c + 8(z>>1) + 4((z&1) ^ ((c>>1)&1)) + ((2(c&1) | (z>>1)) ^ y)
//    (the 128-byte pattern written out), so a thread forms each of its
//    stage-1 addresses once from its cell and plane;
//  * after stage 1 the staged runs are dead and their space holds three
//    unswizzled arrays [cell][plane][row]: the cell values U, the P planes,
//    and the z-face terms already combined per plane (thread y of a cell
//    forms the terms of the face points of row y for all four planes);
//  * the odd strides (21 rows of 16 bytes per cell, in the arrays and the
//    records; 5 rows per plane) put the 8 cells of a warp on 8 different
//    16-byte bank groups: the loads that the 4 threads of a cell share are
//    one wavefront, and the plane-per-thread accesses four;
//  * each thread stores its own plane (64 contiguous bytes) with two 32-byte
//    vector stores, so no staging of the result;
//  * rows are held as pairs (x0, x1), (x2, x3) and every contraction runs as
//    paired FP32 multiply-adds (one instruction for two lanes, the scalar
//    factor broadcast): along x the pair is a column pair of the 1D matrix,
//    along y and z a row pair of the data.  The FP32 instructions per thread
//    fall from about 830 to 430 (ncu instruction counts at 80^3 Q3);
//  * operator direction as a template parameter.
// ---------------------------------------------------------------------------
struct Q3T {
  static constexpr int N = 4, N2 = 16, NB = 64, CPB = 32, THREADS = 128, REC = 84;
  // phase 1 (TMA): own run with one halo cell each side, the y-neighbour
  // runs (128-byte swizzle, 1024-byte aligned), the records
  static constexpr int OWN_B = 0, YL_B = 9216, YH_B = YL_B + CPB * 256,
                       REC_B = YH_B + CPB * 256, P1_END = REC_B + CPB * REC * 4;
  // phase 2: [cell][plane][row] float4 arrays, 21 rows per cell, 5 per plane
  static constexpr int CR = 21, PR = 5, ARR = CPB * CR * 16;
  static constexpr int U_B = 0, PS_B = ARR, FS_B = 2 * ARR, P2_END = 3 * ARR;
  static constexpr int SMEM = 1024 + P1_END;
  static constexpr int LINES_OWN = (CPB + 2) * 2, LINES_RUN = CPB * 2;
  static_assert((CPB + 2) * 256 <= YL_B, "own run overlaps the y runs");
  static_assert(P2_END + 2 * THREADS * 8 <= P1_END,
                "phase-2 arrays and the block-sum scratch must fit the phase-1 space");
  static_assert(LINES_OWN == Q3Cfg::LINES_OWN && LINES_RUN == Q3Cfg::LINES_RUN &&
                    LINES_OWN == (int)kLinesOwn && LINES_RUN == (int)kLinesRun,
                "tensor maps are shared with k_apply32_q3");
};

// byte offset of row y of plane q of cell c in a phase-2 array
__device__ __forceinline__ unsigned q3_pad_row(int c, int q, int y) {
  return 16u * (unsigned)(Q3T::CR * c + Q3T::PR * q + y);
}

// 1D tables of the Q3 kernel (kernel parameter space), with the pairs its
// paired multiply-adds take as operands
struct Q3Tab {
  float M[16];         // Mhat row-major
  float d0[4], d1[4];  // basis derivatives at 0 and 1
  float2 MTp[4][2];    // MTp[c][h] = (Mhat[2h][c], Mhat[2h+1][c])
  float2 d0p[2], d1p[2];
};
static_assert(offsetof(Q3Tab, MTp) % 8 == 0, "pairs must be 8-byte aligned");

// coupling of a neighbour trace (val, dv) on a lower (hi = false) or upper
// face; cf = {hp ke, hp ko, hp pen, th hp ke, th hp ko} (zero without a
// neighbour)
template <bool kTr>
__device__ __forceinline__ void q3_face(const float *cf, bool hi, float val, float dv, float &s1,
                                        float &s2) {
  if constexpr (!kTr) {
    s1 = (hi ? -cf[1] : cf[1]) * dv - cf[2] * val;
    s2 = (hi ? -cf[3] : cf[3]) * val;
  } else {
    s1 = (hi ? cf[4] : -cf[4]) * dv - cf[2] * val;
    s2 = (hi ? cf[0] : -cf[0]) * val;
  }
}

// the same for two face points at once
template <bool kTr>
__device__ __forceinline__ void q3_face2(const float *cf, bool hi, float2 val, float2 dv, float2 &s1,
                                         float2 &s2) {
  if constexpr (!kTr) {
    s1 = ffma2(bc2(hi ? -cf[1] : cf[1]), dv, fmul2(bc2(-cf[2]), val));
    s2 = fmul2(bc2(hi ? -cf[3] : cf[3]), val);
  } else {
    s1 = ffma2(bc2(hi ? cf[4] : -cf[4]), dv, fmul2(bc2(-cf[2]), val));
    s2 = fmul2(bc2(hi ? cf[0] : -cf[0]), val);
  }
}

// records of k_apply32_q3t from the 78-float records (computed in FP64,
// rounded): padded to 84 floats, A'_x transposed (its columns are the pairs
// of the x contraction), the coupling coefficients of faces without a
// neighbour zeroed.  Records built in the kernel from K in FP32 instead cost
// more time than their copy (272 against 217 us at 96^3) and, less
// accurate, took the mixed solve of the 96^3 Q3 problem from 5,533 to 7,885
// inner iterations.
__global__ void k_record_q3t(const OpParams<float> p, const float *__restrict__ rec,
                             float *__restrict__ out) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ncell) return;
  int ix[3];
  coords32(p, (unsigned)e, ix);
  const float *r = rec + e * Q3Cfg::REC;
  float *o = out + e * Q3T::REC;
  for (int i = 0; i < 4; i++)
    for (int q = 0; q < 4; q++) o[q * 4 + i] = r[i * 4 + q];
  for (int i = Q3T::N2; i < 3 * Q3T::N2; i++) o[i] = r[i];
  for (int f = 0; f < 6; f++) {
    const int d = f >> 1;
    const bool has = (f & 1) ? ix[d] + 1 < p.nc[d] : ix[d] > 0;
    for (int j = 0; j < 5; j++) o[3 * Q3T::N2 + 5 * f + j] = has ? r[3 * Q3T::N2 + 5 * f + j] : 0.f;
  }
  for (int i = 78; i < Q3T::REC; i++) o[i] = 0.f;
}

// One run of CPB cells (first cell e0) from a staged phase-1 region `base`
// (own run with halo, y-neighbour runs, records); zl / zh: the thread's
// z-neighbour rows.  Returns the thread's part of <x, y_out>.
template <bool kTr>
__device__ __forceinline__ float q3_run(const OpParams<float> &p, const ApplyArgs<float> &a,
                                        const Q3Tab &tb, unsigned char *base, long e0,
                                        const float4 *zl, const float4 *zh) {
  using C = Q3T;
  constexpr int N = 4, NB = 64, REC = C::REC;
  const long ncell = p.ncell;
  const int cs = threadIdx.x >> 2, z = threadIdx.x & 3;
  const long e = e0 + cs;
  const unsigned char *R = base + C::REC_B + cs * REC * 4;
  auto rec4 = [&](int i) -> float4 { return sh4(R, 16u * i); };
  // coupling coefficients: floats 48..77 of the record
  float cf[32];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const float4 v = rec4(12 + i);
    cf[4 * i] = v.x; cf[4 * i + 1] = v.y; cf[4 * i + 2] = v.z; cf[4 * i + 3] = v.w;
  }
  // row z (column z for the transpose) of A'_z, for stage 2
  float az[N];
  if constexpr (!kTr) {
    const float4 v = sh4(R, 128u + 16u * z);
    az[0] = v.x; az[1] = v.y; az[2] = v.z; az[3] = v.w;
  } else {
#pragma unroll
    for (int q = 0; q < N; q++) az[q] = *reinterpret_cast<const float *>(R + 128u + 16u * q + 4u * z);
  }

  // ---- stage 1: plane z, rows as pairs (x0, x1), (x2, x3) ----
  const unsigned char *OWN = base + C::OWN_B;
  float2 u[N][2];
#pragma unroll
  for (int y = 0; y < N; y++) {
    const float4 v = sh4(OWN, q3_swz_row(cs + 1, z, y));
    u[y][0] = make_float2(v.x, v.y);
    u[y][1] = make_float2(v.z, v.w);
  }
  float2 P[N][2];
  {
    // x: X = A'_x u + x-face terms, P = Mhat_y X
    float2 X[N][2];
    float4 A[N];   // A[i] = column i of A'_x
#pragma unroll
    for (int i = 0; i < N; i++) A[i] = rec4(i);
#pragma unroll
    for (int y = 0; y < N; y++) {
      const float4 l = sh4(OWN, q3_swz_row(cs, z, y));
      const float4 h = sh4(OWN, q3_swz_row(cs + 2, z, y));
      const float dvl = tb.d1[0] * l.x + tb.d1[1] * l.y + tb.d1[2] * l.z + tb.d1[3] * l.w;
      const float dvh = tb.d0[0] * h.x + tb.d0[1] * h.y + tb.d0[2] * h.z + tb.d0[3] * h.w;
      float s1l, s2l, s1h, s2h;
      q3_face<kTr>(cf + 0, false, l.w, dvl, s1l, s2l);
      q3_face<kTr>(cf + 5, true, h.x, dvh, s1h, s2h);
      // [xx = 0] s1l + d0[xx] s2l + [xx = N-1] s1h + d1[xx] s2h
      X[y][0] = ffma2(tb.d1p[0], bc2(s2h), ffma2(tb.d0p[0], bc2(s2l), make_float2(s1l, 0.f)));
      X[y][1] = ffma2(tb.d1p[1], bc2(s2h), ffma2(tb.d0p[1], bc2(s2l), make_float2(0.f, s1h)));
#pragma unroll
      for (int q = 0; q < N; q++) {
        const float uq = q < 2 ? (q == 0 ? u[y][0].x : u[y][0].y) : (q == 2 ? u[y][1].x : u[y][1].y);
        if constexpr (!kTr) {
          X[y][0] = ffma2(make_float2(A[q].x, A[q].y), bc2(uq), X[y][0]);
          X[y][1] = ffma2(make_float2(A[q].z, A[q].w), bc2(uq), X[y][1]);
        } else {
          X[y][0] = ffma2(make_float2(f4c(A[0], q), f4c(A[1], q)), bc2(uq), X[y][0]);
          X[y][1] = ffma2(make_float2(f4c(A[2], q), f4c(A[3], q)), bc2(uq), X[y][1]);
        }
      }
    }
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        float2 s = fmul2(bc2(tb.M[y * N]), X[0][hh]);
#pragma unroll
        for (int r = 1; r < N; r++) s = ffma2(bc2(tb.M[y * N + r]), X[r][hh], s);
        P[y][hh] = s;
      }
  }
  {
    // y: Y = A'_y u + y-face terms, P += Mhat_x Y
    float2 s1l[2], s2l[2], s1h[2], s2h[2];
    {
      float2 yl[N][2], yh[N][2];
#pragma unroll
      for (int y = 0; y < N; y++) {
        const float4 l = sh4(base + C::YL_B, q3_swz_row(cs, z, y));
        const float4 h = sh4(base + C::YH_B, q3_swz_row(cs, z, y));
        yl[y][0] = make_float2(l.x, l.y); yl[y][1] = make_float2(l.z, l.w);
        yh[y][0] = make_float2(h.x, h.y); yh[y][1] = make_float2(h.z, h.w);
      }
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        float2 dvl = fmul2(bc2(tb.d1[0]), yl[0][hh]), dvh = fmul2(bc2(tb.d0[0]), yh[0][hh]);
#pragma unroll
        for (int q = 1; q < N; q++) {
          dvl = ffma2(bc2(tb.d1[q]), yl[q][hh], dvl);
          dvh = ffma2(bc2(tb.d0[q]), yh[q][hh], dvh);
        }
        q3_face2<kTr>(cf + 10, false, yl[N - 1][hh], dvl, s1l[hh], s2l[hh]);
        q3_face2<kTr>(cf + 15, true, yh[0][hh], dvh, s1h[hh], s2h[hh]);
      }
    }
    const float4 A0 = rec4(4), A1 = rec4(5), A2 = rec4(6), A3 = rec4(7);
#pragma unroll
    for (int y = 0; y < N; y++) {
      float2 Y[2];
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        float2 s = ffma2(bc2(tb.d1[y]), s2h[hh], fmul2(bc2(tb.d0[y]), s2l[hh]));
        if (y == 0) s = fadd2(s, s1l[hh]);
        if (y == N - 1) s = fadd2(s, s1h[hh]);
#pragma unroll
        for (int q = 0; q < N; q++) {
          // A'_y(y, q), or A'_y(q, y) for the transpose
          const float4 &Ar = kTr ? (q == 0 ? A0 : q == 1 ? A1 : q == 2 ? A2 : A3)
                                 : (y == 0 ? A0 : y == 1 ? A1 : y == 2 ? A2 : A3);
          s = ffma2(bc2(f4c(Ar, kTr ? y : q)), u[q][hh], s);
        }
        Y[hh] = s;
      }
      // P[y][xx] += sum_r Mhat[xx][r] Y[r]
#pragma unroll
      for (int r = 0; r < N; r++) {
        const float yr = r < 2 ? (r == 0 ? Y[0].x : Y[0].y) : (r == 2 ? Y[1].x : Y[1].y);
        P[y][0] = ffma2(tb.MTp[r][0], bc2(yr), P[y][0]);
        P[y][1] = ffma2(tb.MTp[r][1], bc2(yr), P[y][1]);
      }
    }
  }
  // z faces at the face points of row y = z, combined for each plane w:
  //   F_w = [w = 0] s1 lo + d0[w] s2 lo + [w = N-1] s1 hi + d1[w] s2 hi
  float2 F[N][2];
  {
    float2 s1l[2], s2l[2], s1h[2], s2h[2];
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
      float2 zl2[N], zh2[N];
#pragma unroll
      for (int q = 0; q < N; q++) {
        zl2[q] = hh ? make_float2(zl[q].z, zl[q].w) : make_float2(zl[q].x, zl[q].y);
        zh2[q] = hh ? make_float2(zh[q].z, zh[q].w) : make_float2(zh[q].x, zh[q].y);
      }
      float2 dvl = fmul2(bc2(tb.d1[0]), zl2[0]), dvh = fmul2(bc2(tb.d0[0]), zh2[0]);
#pragma unroll
      for (int q = 1; q < N; q++) {
        dvl = ffma2(bc2(tb.d1[q]), zl2[q], dvl);
        dvh = ffma2(bc2(tb.d0[q]), zh2[q], dvh);
      }
      q3_face2<kTr>(cf + 20, false, zl2[N - 1], dvl, s1l[hh], s2l[hh]);
      q3_face2<kTr>(cf + 25, true, zh2[0], dvh, s1h[hh], s2h[hh]);
    }
#pragma unroll
    for (int w = 0; w < N; w++)
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        float2 s = ffma2(bc2(tb.d1[w]), s2h[hh], fmul2(bc2(tb.d0[w]), s2l[hh]));
        if (w == 0) s = fadd2(s, s1l[hh]);
        if (w == N - 1) s = fadd2(s, s1h[hh]);
        F[w][hh] = s;
      }
  }
  // every thread has read the staged runs and records: phase-2 arrays
  __syncthreads();
  unsigned char *U = base + C::U_B, *PS = base + C::PS_B, *FS = base + C::FS_B;
#pragma unroll
  for (int y = 0; y < N; y++) {
    st4(U, q3_pad_row(cs, z, y), make_float4(u[y][0].x, u[y][0].y, u[y][1].x, u[y][1].y));
    st4(PS, q3_pad_row(cs, z, y), make_float4(P[y][0].x, P[y][0].y, P[y][1].x, P[y][1].y));
  }
#pragma unroll
  for (int w = 0; w < N; w++)
    st4(FS, q3_pad_row(cs, w, z), make_float4(F[w][0].x, F[w][0].y, F[w][1].x, F[w][1].y));
  __syncthreads();

  // ---- stage 2: z contractions of plane z ----
  float2 out[N][2];
  {
    float2 Zp[N][2];
#pragma unroll
    for (int y = 0; y < N; y++) {
      const float4 f = sh4(FS, q3_pad_row(cs, z, y));
      float2 a0 = make_float2(f.x, f.y), a1 = make_float2(f.z, f.w);
#pragma unroll
      for (int q = 0; q < N; q++) {
        const float4 v = sh4(U, q3_pad_row(cs, q, y));
        a0 = ffma2(bc2(az[q]), make_float2(v.x, v.y), a0);
        a1 = ffma2(bc2(az[q]), make_float2(v.z, v.w), a1);
      }
      Zp[y][0] = a0;
      Zp[y][1] = a1;
    }
    float mz[N];
#pragma unroll
    for (int q = 0; q < N; q++) mz[q] = tb.M[z * N + q];
#pragma unroll
    for (int y = 0; y < N; y++) {
      // Mhat_z P
      float2 a0, a1;
      {
        const float4 v = sh4(PS, q3_pad_row(cs, 0, y));
        a0 = fmul2(bc2(mz[0]), make_float2(v.x, v.y));
        a1 = fmul2(bc2(mz[0]), make_float2(v.z, v.w));
      }
#pragma unroll
      for (int q = 1; q < N; q++) {
        const float4 v = sh4(PS, q3_pad_row(cs, q, y));
        a0 = ffma2(bc2(mz[q]), make_float2(v.x, v.y), a0);
        a1 = ffma2(bc2(mz[q]), make_float2(v.z, v.w), a1);
      }
      out[y][0] = a0;
      out[y][1] = a1;
    }
    // (Mhat_y (x) Mhat_x) Zp: T1 = Mhat_x along x, then Mhat_y across rows
#pragma unroll
    for (int r = 0; r < N; r++) {
      float2 t0 = make_float2(0.f, 0.f), t1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int c = 0; c < N; c++) {
        const float zc = c < 2 ? (c == 0 ? Zp[r][0].x : Zp[r][0].y)
                               : (c == 2 ? Zp[r][1].x : Zp[r][1].y);
        t0 = ffma2(tb.MTp[c][0], bc2(zc), t0);
        t1 = ffma2(tb.MTp[c][1], bc2(zc), t1);
      }
#pragma unroll
      for (int y = 0; y < N; y++) {
        out[y][0] = ffma2(bc2(tb.M[y * N + r]), t0, out[y][0]);
        out[y][1] = ffma2(bc2(tb.M[y * N + r]), t1, out[y][1]);
      }
    }
  }

  // ---- write-back: the thread's plane, 64 contiguous bytes ----
  float part = 0.f;
  if (e < ncell) {
    const float alpha = a.alpha;
    float v[NB / N];
#pragma unroll
    for (int y = 0; y < N; y++)
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        const float2 o = fmul2(bc2(alpha), out[y][hh]);
        v[y * N + 2 * hh] = o.x;
        v[y * N + 2 * hh + 1] = o.y;
      }
    float *yp = a.y + e * NB + z * 16;
    const float *ap = a.add ? a.add + e * NB + z * 16 : nullptr;
    if (((reinterpret_cast<uintptr_t>(yp) | reinterpret_cast<uintptr_t>(ap)) & 31) == 0) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float *d = yp + 8 * h;
        if (a.accumulate) {
          float w[8];
          ld8(d, w);
#pragma unroll
          for (int j = 0; j < 8; j++) v[8 * h + j] += w[j];
        }
        if (ap) {
          float w[8];
          ld8(ap + 8 * h, w);
#pragma unroll
          for (int j = 0; j < 8; j++) v[8 * h + j] += w[j];
        }
        st8(d, v + 8 * h);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 16; j++) {
        float r = v[j];
        if (a.accumulate) r += yp[j];
        if (ap) r += ap[j];
        yp[j] = r;
        v[j] = r;
      }
    }
    if (a.dot_part) {
#pragma unroll
      for (int y = 0; y < N; y++) {
        const float4 pin = sh4(U, q3_pad_row(cs, z, y));
        part += pin.x * v[4 * y] + pin.y * v[4 * y + 1] + pin.z * v[4 * y + 2] + pin.w * v[4 * y + 3];
      }
    }
  }
  return part;
}

// 5 blocks per SM (4: the same time at 96^3; 6: 254 against 227 us, spills)
template <bool kTr>
__global__ void __launch_bounds__(Q3T::THREADS, 5)
    k_apply32_q3t(const OpParams<float> p, const ApplyArgs<float> a, const float *__restrict__ rec,
                  const Q3Tab tb, const __grid_constant__ CUtensorMap map_own,
                  const __grid_constant__ CUtensorMap map_run, int *tma_err) {
  using C = Q3T;
  constexpr int N = 4, NB = 64, CPB = C::CPB, REC = C::REC;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) unsigned long long stage_bar;
  if (a.skip && *a.skip) return;
  // 1024-byte aligned base, kept in the shared window
  unsigned char *base = smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u);

  const long e0 = (long)blockIdx.x * CPB;
  const long ncell = p.ncell;
  const long sx = p.nc[0], sxy = (long)p.nc[0] * p.nc[1];
  const float *__restrict__ x = a.x;
  const int t = threadIdx.x, cs = t >> 2, z = t & 3;
  const long e = e0 + cs;
  const long ee = e < ncell ? e : 0;
  int ix[3];
  coords32(p, (unsigned)ee, ix);
  // z-neighbour rows (plane q, row y = z) straight from global memory, issued
  // before the staging wait; zero where the cell has no z neighbour
  float4 zl[N], zh[N];
  {
    const bool lo = ix[2] > 0, hi = ix[2] + 1 < p.nc[2];
    const float4 *pl = reinterpret_cast<const float4 *>(x + (ee - (lo ? sxy : 0)) * NB + z * N);
    const float4 *ph = reinterpret_cast<const float4 *>(x + (ee + (hi ? sxy : 0)) * NB + z * N);
#pragma unroll
    for (int q = 0; q < N; q++) {
      zl[q] = lo ? pl[q * 4] : make_float4(0.f, 0.f, 0.f, 0.f);
      zh[q] = hi ? ph[q * 4] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }

  {
    const unsigned bar = smem_u32(&stage_bar);
    const long ncp = ncell - e0 < CPB ? ncell - e0 : CPB;
    const unsigned rbytes = (unsigned)(ncp * REC * 4);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(bar, (unsigned)(C::LINES_OWN + 2 * C::LINES_RUN) * 128u + rbytes);
      tma_load_2d(smem_u32(base + C::OWN_B), &map_own, 0, (int)((e0 - 1) * 2), bar);
      tma_load_2d(smem_u32(base + C::YL_B), &map_run, 0, (int)((e0 - sx) * 2), bar);
      tma_load_2d(smem_u32(base + C::YH_B), &map_run, 0, (int)((e0 + sx) * 2), bar);
      bulk_load(smem_u32(base + C::REC_B), rec + e0 * REC, rbytes, bar);
    }
    if (!mbar_wait(bar, 0, kTmaPolls)) {
      if (threadIdx.x == 0) atomicExch(tma_err, 1);
      mbar_wait(bar, 0, kTmaPolls);
      return;
    }
  }

  const float part = q3_run<kTr>(p, a, tb, base, e0, zl, zh);
  // block sums in the phase-1 space past the phase-2 arrays (record space,
  // dead since stage 1; other warps may still read the arrays)
  if (a.dot_part)
    reduce_tail_grouped<Q3T::THREADS, true>(
        a.dot_part, a.dot_max_blocks, a.dot_cnt, RedCtx{nullptr, a.dot_scal, a.dot_flags},
        (double)part, 0.0, a.dot_fin, -1, -1, reinterpret_cast<double *>(base + C::P2_END));
}

// Persistent form: a block runs the runs blockIdx.x, + gridDim.x, ... with
// two phase-1 regions; the copies of run i + 2 are issued as soon as run i
// has released its region, and the z-neighbour rows of run i + 1 are loaded
// into registers while run i computes, so the staging latency of a run
// overlaps the computation of the one before.
struct Q3P {
  static constexpr int STAGE = (Q3T::P1_END + 1023) / 1024 * 1024;
  static constexpr int SMEM = 1024 + 2 * STAGE;
};
__device__ __forceinline__ void q3_zrows(const OpParams<float> &p, const float *x, long run,
                                         float4 *zl, float4 *zh) {
  constexpr int N = 4, NB = 64;
  const int cs = threadIdx.x >> 2, z = threadIdx.x & 3;
  const long e = run * Q3T::CPB + cs;
  const long ee = e < p.ncell ? e : 0;
  const long sxy = (long)p.nc[0] * p.nc[1];
  int ix[3];
  coords32(p, (unsigned)ee, ix);
  const bool lo = ix[2] > 0, hi = ix[2] + 1 < p.nc[2];
  const float4 *pl = reinterpret_cast<const float4 *>(x + (ee - (lo ? sxy : 0)) * NB + z * N);
  const float4 *ph = reinterpret_cast<const float4 *>(x + (ee + (hi ? sxy : 0)) * NB + z * N);
#pragma unroll
  for (int q = 0; q < N; q++) {
    zl[q] = lo ? pl[q * 4] : make_float4(0.f, 0.f, 0.f, 0.f);
    zh[q] = hi ? ph[q * 4] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

template <bool kTr>
__global__ void __launch_bounds__(Q3T::THREADS, 3)
    k_apply32_q3p(const OpParams<float> p, const ApplyArgs<float> a, const float *__restrict__ rec,
                  const Q3Tab tb, const __grid_constant__ CUtensorMap map_own,
                  const __grid_constant__ CUtensorMap map_run, int *tma_err) {
  using C = Q3T;
  constexpr int N = 4, CPB = C::CPB, REC = C::REC;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) unsigned long long stage_bar[2];
  if (a.skip && *a.skip) return;
  unsigned char *base = smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u);
  const long ncell = p.ncell;
  const long nruns = (ncell + CPB - 1) / CPB;
  const long sx = p.nc[0];
  const long G = gridDim.x;
  const unsigned bar0 = smem_u32(&stage_bar[0]), bar1 = smem_u32(&stage_bar[1]);
  // thread 0: the copies of run r into region b
  auto issue = [&](long r, int b) {
    const long e0 = r * CPB;
    const long ncp = ncell - e0 < CPB ? ncell - e0 : CPB;
    const unsigned rbytes = (unsigned)(ncp * REC * 4);
    unsigned char *st = base + b * Q3P::STAGE;
    const unsigned bar = b ? bar1 : bar0;
    // the region was last written by ordinary stores (phase-2 arrays)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, (unsigned)(C::LINES_OWN + 2 * C::LINES_RUN) * 128u + rbytes);
    tma_load_2d(smem_u32(st + C::OWN_B), &map_own, 0, (int)((e0 - 1) * 2), bar);
    tma_load_2d(smem_u32(st + C::YL_B), &map_run, 0, (int)((e0 - sx) * 2), bar);
    tma_load_2d(smem_u32(st + C::YH_B), &map_run, 0, (int)((e0 + sx) * 2), bar);
    bulk_load(smem_u32(st + C::REC_B), rec + e0 * REC, rbytes, bar);
  };
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
  }
  __syncthreads();
  const long r0 = blockIdx.x;
  if (threadIdx.x == 0) {
    if (r0 < nruns) issue(r0, 0);
    if (r0 + G < nruns) issue(r0 + G, 1);
  }
  float4 zl[N], zh[N];
  if (r0 < nruns) q3_zrows(p, a.x, r0, zl, zh);
  double part = 0.0;   // a block runs up to nruns / gridDim.x runs
  int it = 0;
  for (long r = r0; r < nruns; r += G, it++) {
    const int b = it & 1;
    float4 nzl[N], nzh[N];
    if (r + G < nruns) q3_zrows(p, a.x, r + G, nzl, nzh);
    if (!mbar_wait(b ? bar1 : bar0, (unsigned)((it >> 1) & 1), kTmaPolls)) {
      if (threadIdx.x == 0) atomicExch(tma_err, 1);
      mbar_wait(b ? bar1 : bar0, (unsigned)((it >> 1) & 1), kTmaPolls);
      return;
    }
    part += (double)q3_run<kTr>(p, a, tb, base + b * Q3P::STAGE, r * CPB, zl, zh);
    // every thread is done with region b: stage run r + 2G there
    __syncthreads();
    if (threadIdx.x == 0 && r + 2 * G < nruns) issue(r + 2 * G, b);
#pragma unroll
    for (int q = 0; q < N; q++) {
      zl[q] = nzl[q];
      zh[q] = nzh[q];
    }
  }
  // block sums in region 0's scratch space (free: the last sync above, or
  // no run at all)
  if (a.dot_part)
    reduce_tail_grouped<Q3T::THREADS, true>(
        a.dot_part, a.dot_max_blocks, a.dot_cnt, RedCtx{nullptr, a.dot_scal, a.dot_flags},
        part, 0.0, a.dot_fin, -1, -1, reinterpret_cast<double *>(base + C::P2_END));
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

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    cudaGetLastError();
  });
  return fn;
}

// A FP32 vector of ndof values as a 2D tensor of 128-byte lines (32 floats),
// boxes of `lines` lines, the 128-byte swizzle, zeros outside
static bool encode_lines(CUtensorMap *m, const float *x, long ndof, unsigned lines) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t dims[2] = {32, (cuuint64_t)(ndof / 32)};
  const cuuint64_t strides[1] = {128};
  const cuuint32_t box[2] = {32, lines};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(x), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the maps of the last few input vectors (a Krylov solve applies the
// operator to the same few buffers); per host thread, so no locking
struct LinesMaps {
  const float *x;
  long ndof;
  CUtensorMap own, run;
};
bool q3_lines_maps(const float *x, long ndof, const CUtensorMap **own,
                   const CUtensorMap **run) {
  constexpr int kSlots = 8;
  thread_local LinesMaps cache[kSlots];
  thread_local int next = 0;
  for (int i = 0; i < kSlots; i++)
    if (cache[i].x == x && cache[i].ndof == ndof) {
      *own = &cache[i].own;
      *run = &cache[i].run;
      return true;
    }
  LinesMaps &c = cache[next];
  if (!encode_lines(&c.own, x, ndof, kLinesOwn) || !encode_lines(&c.run, x, ndof, kLinesRun)) {
    c.x = nullptr;
    return false;
  }
  c.x = x;
  c.ndof = ndof;
  next = (next + 1) % kSlots;
  *own = &c.own;
  *run = &c.run;
  return true;
}

static int launch32_q3(pdg_context *ctx, const ApplyArgs<float> &a, const OpParams<float> &p,
                       const float *rec) {
  const size_t smem = Q3Cfg::SMEM;
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32_q3<true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32_q3<false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_dev = ctx->device;
  }
  const EdgeTab &tb = edge_tab(ctx);
  const unsigned blocks = (unsigned)((ctx->ncell + Q3Cfg::CPB - 1) / Q3Cfg::CPB);
  int *err = ctx->d_flag + F_TMA;
  const CUtensorMap *own = nullptr, *run = nullptr;
  // TMA needs a 16-byte aligned vector (and records, from cudaMalloc)
  if ((reinterpret_cast<uintptr_t>(a.x) & 15) == 0 && (reinterpret_cast<uintptr_t>(rec) & 15) == 0 &&
      q3_lines_maps(a.x, ctx->ndof, &own, &run)) {
    if (!a.diag_only) {
      static_assert(Q3T::CPB == Q3Cfg::CPB, "one block per run of CPB cells");
      if (!ctx->rec32q_valid) {
        if (!ctx->rec32q)
          PDG_CUDA_TRY(cudaMalloc(&ctx->rec32q, sizeof(float) * Q3T::REC * ctx->ncell));
        k_record_q3t<<<(unsigned)((ctx->ncell + 127) / 128), 128, 0, ctx->stream>>>(p, rec,
                                                                                   ctx->rec32q);
        PDG_CUDA_TRY(cudaGetLastError());
        ctx->rec32q_valid = 1;
      }
      static int attr_t = -1, sms = 0;
      if (attr_t != ctx->device) {
        PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32_q3t<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, Q3T::SMEM));
        PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32_q3t<true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, Q3T::SMEM));
        PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32_q3p<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, Q3P::SMEM));
        PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply32_q3p<true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, Q3P::SMEM));
        PDG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
        attr_t = ctx->device;
      }
      Q3Tab qt;
      for (int i = 0; i < 16; i++) qt.M[i] = tb.M[i];
      for (int i = 0; i < 4; i++) {
        qt.d0[i] = tb.d0[i];
        qt.d1[i] = tb.d1[i];
      }
      for (int c = 0; c < 4; c++)
        for (int h = 0; h < 2; h++) qt.MTp[c][h] = make_float2(qt.M[2 * h * 4 + c], qt.M[(2 * h + 1) * 4 + c]);
      for (int h = 0; h < 2; h++) {
        qt.d0p[h] = make_float2(qt.d0[2 * h], qt.d0[2 * h + 1]);
        qt.d1p[h] = make_float2(qt.d1[2 * h], qt.d1[2 * h + 1]);
      }
      if (!a.accumulate && !a.add) {
        // three resident blocks per SM (two phase-1 regions each); the
        // accumulating forms stay with one run per block, whose read of y
        // other resident blocks cover (96^3 Q3, y += J x: 220 us against 253)
        const unsigned pblocks = (unsigned)std::min<long>(blocks, 3L * sms);
        if (a.transpose)
          k_apply32_q3p<true><<<pblocks, Q3T::THREADS, Q3P::SMEM, ctx->stream>>>(
              p, a, ctx->rec32q, qt, *own, *run, err);
        else
          k_apply32_q3p<false><<<pblocks, Q3T::THREADS, Q3P::SMEM, ctx->stream>>>(
              p, a, ctx->rec32q, qt, *own, *run, err);
      } else if (a.transpose) {
        k_apply32_q3t<true><<<blocks, Q3T::THREADS, Q3T::SMEM, ctx->stream>>>(
            p, a, ctx->rec32q, qt, *own, *run, err);
      } else {
        k_apply32_q3t<false><<<blocks, Q3T::THREADS, Q3T::SMEM, ctx->stream>>>(
            p, a, ctx->rec32q, qt, *own, *run, err);
      }
      PDG_CUDA_TRY(cudaGetLastError());
      return PDG_OK;
    }
    k_apply32_q3<true><<<blocks, Q3Cfg::THREADS, smem, ctx->stream>>>(p, a, rec, tb, *own, *run,
                                                                      err);
  } else {
    CUtensorMap none;
    std::memset(&none, 0, sizeof(none));
    k_apply32_q3<false><<<blocks, Q3Cfg::THREADS, smem, ctx->stream>>>(p, a, rec, tb, none, none,
                                                                       err);
  }
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int launch_apply32_3d(pdg_context *ctx, const ApplyArgs<float> &a0, const OpParams<float> &p,
                      const float *rec) {
  ApplyArgs<float> a = a0;
  if (ctx->fuse_fin) {
    a.dot_part = ctx->fuse_part;
    a.dot_max_blocks = ctx->fuse_max_blocks;
    a.dot_cnt = ctx->fuse_cnt;
    a.dot_scal = ctx->red_out;
    a.dot_flags = ctx->d_flag;
    a.dot_fin = ctx->fuse_fin;
  }
  switch (ctx->N) {
    case 2: return launch32_n<2>(ctx, a, p, rec);
    case 3: return launch32_n<3>(ctx, a, p, rec);
    case 4: return launch32_q3(ctx, a, p, rec);
    default: return set_error(PDG_EUNSUPPORTED, "staged FP32 kernel: degrees 1 to 3");
  }
}

}  // namespace pdg
