// pdg_apply_fp.cu -- the 3D FP64 cell operator in float-pair arithmetic.
//
// Same operator and thread mapping as k_apply<double, 3, N> (pdg_apply.cu;
// reference: ConvectionDiffusionDG::jacobian_apply_volume / _skeleton /
// _boundary, localoperator/convectiondiffusiondg.hh:191-195, 474-481,
// 892-899), with every FP64 value carried as an unevaluated sum of two floats
// (hi + lo, the "double-float" representation of Dekker 1971).  GB300 runs
// FP64 at about 1/74 of its FP32 rate, and the FP64 operator is bound by its
// FP64 pipe; here the arithmetic runs on the FP32 pipe:
//   * a multiply-add acc += a b is the exact product of the leading parts
//     (p = ah bh and its rounding error fma(ah, bh, -p), Ogita-Rump-Oishi
//     TwoProdFMA), the cross terms ah bl + al bh in FP32, and Knuth's TwoSum
//     of acc.hi and p; the errors collect in acc.lo (12 FP32 operations);
//   * inputs are split with integer operations on the FP64 bit pattern (hi:
//     sign, exponent, top 23 mantissa bits; lo: the next 24 bits), so no
//     FP64 instruction runs per input value; the output is joined in FP64.
// A float pair holds 48 significant bits (FP64: 53), so results agree with
// the FP64 operator to a few units in the 14th digit.  The per-cell records
// and the 1D tables are converted to pairs once.
//
// Selected by pdg_set_f64_arithmetic(ctx, PDG_F64_FLOAT_PAIR) for the applies
// of the 3D scalar-K operator; every other kernel keeps FP64.
#include "pdg_ops.cuh"
#include "pdg_vec.cuh"

namespace pdg {

// ---- float-pair primitives ---------------------------------------------------
struct __align__(8) fpair {
  float hi, lo;
};

// hi + lo = d to 48 bits, from the bit pattern (no FP64 arithmetic).  Values
// whose float exponent would leave the normal range are flushed to zero
// (|d| < 2^-126) or saturate (never met by the operator's data).
__device__ __forceinline__ fpair split_bits(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7FF);
  fpair r{0.f, 0.f};
  const int ef = e - 1023 + 127;
  if (e == 0 || ef < 1) return r;
  if (ef > 254) {
    r.hi = __int_as_float((int)(sign | 0x7F7FFFFFu));
    return r;
  }
  r.hi = __int_as_float((int)(sign | ((unsigned)ef << 23) | (unsigned)((b >> 29) & 0x7FFFFF)));
  // the low 29 mantissa bits, value L 2^(e - 1075), as a normalised float
  const unsigned L = (unsigned)(b & 0x1FFFFFFFu);
  if (L == 0) return r;
  const int p = 31 - __clz((int)L);                 // highest set bit, 0..28
  const int el = e - 1075 + p + 127;                // biased exponent of lo
  if (el < 1) return r;
  const unsigned m = p >= 23 ? (L >> (p - 23)) : (L << (23 - p));
  r.lo = __int_as_float((int)(sign | ((unsigned)el << 23) | (m & 0x7FFFFF)));
  return r;
}

__device__ __forceinline__ double join(fpair a) { return (double)a.hi + (double)a.lo; }

// acc += a * b
__device__ __forceinline__ void pmac(fpair &acc, fpair a, fpair b) {
  const float p = a.hi * b.hi;
  const float e = fmaf(a.hi, b.hi, -p);
  const float c = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  const float t = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += t + c;
}

// a * b as a pair: the exact product of the leading parts plus the cross
// terms (the first term of a chain, 4 FP32 operations)
__device__ __forceinline__ fpair pmul(fpair a, fpair b) {
  const float p = a.hi * b.hi;
  const float e = fmaf(a.hi, b.hi, -p);
  return fpair{p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e))};
}

// acc += a
__device__ __forceinline__ void padd(fpair &acc, fpair a) {
  const float s = acc.hi + a.hi;
  const float bb = s - acc.hi;
  const float t = (acc.hi - (s - bb)) + (a.hi - bb);
  acc.hi = s;
  acc.lo += t + a.lo;
}

// |lo| <= ulp(hi) / 2 again (Fast2Sum)
__device__ __forceinline__ fpair norm(fpair a) {
  const float s = a.hi + a.lo;
  return fpair{s, a.lo - (s - a.hi)};
}

// ---- conversion of the FP64 records and tables --------------------------------
__global__ void k_to_pairs(long n, const double *__restrict__ src, fpair *__restrict__ dst) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = split_bits(src[i]);
}

template <int N>
struct FpCfg {
  static constexpr int N2 = N * N, NB = N * N * N, TPC = N * N, NF = 6;
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  static constexpr int NW = NF * (N + 1);               // neighbour-line coefficients
  static constexpr int RECW = 3 * N2 + 2 * NW;          // FP64 record (both forms)
  static constexpr int RECU = 3 * N2 + NW;              // the part one launch uses
  static constexpr int TAB = 2 * N2 + 2 * N;            // Mhat, Shat, d0, d1
  // ue, Xs, Ys, Zs, face data (12 TPC), record part; padding per cell
  static constexpr int PER_CELL = 4 * NB + 12 * TPC + RECU + 1;
  // blocks per SM the register allocation must allow: 6 for Q2 (at most 86
  // registers; 0.262 against 0.287 ms per 64^3 apply with the compiler's 96),
  // the compiler's choice otherwise (0: no bound; Q4 bounded to 6 blocks:
  // 0.416 against 0.374 ms at 40^3)
  static constexpr int MINB = N == 3 ? 6 : 0;
};

template <int N>
__global__ void __launch_bounds__(FpCfg<N>::THREADS, FpCfg<N>::MINB)
    k_apply_fp(const OpParams<double> p, const ApplyArgs<double> a, const fpair *__restrict__ rec,
               const fpair *__restrict__ tab) {
  using C = FpCfg<N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB, NF = C::NF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fpair *tM = reinterpret_cast<fpair *>(smem_raw);
  fpair *td0 = tM + 2 * N2;          // (Shat is not needed: it is folded into the record)
  fpair *td1 = td0 + N;
  const int t = threadIdx.x;
  const int cs = t / TPC;
  const int l = t - cs * TPC;
  fpair *cellmem = tM + C::TAB + cs * C::PER_CELL;
  fpair *ue = cellmem;
  fpair *Xs = ue + NB, *Ys = Xs + NB, *Zs = Ys + NB;
  fpair *fa = Zs + NB;               // [2 NF][TPC]
  fpair *Am = fa + 2 * NF * TPC;     // A'_dir [3][N2], then the line coefficients [NF][N+1]
  fpair *W = Am + 3 * N2;

  if (a.skip && *a.skip) return;
  for (int i = t; i < C::TAB; i += blockDim.x) tM[i] = tab[i];

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
  const int stride[3] = {1, p.nc[0], p.nc[0] * p.nc[1]};
  int nbr[NF];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    if (f & 1) nbr[f] = ix[dir] + 1 < p.nc[dir] ? ee + stride[dir] : -1;
    else nbr[f] = ix[dir] > 0 ? ee - stride[dir] : -1;
  }

  // ---- all global loads first: own column, neighbour lines, record ----
  double cold[N];
  const double *xe = a.x + (size_t)ee * NB;
#pragma unroll
  for (int z = 0; z < N; z++) cold[z] = xe[z * TPC + l];
  double vd[NF][N];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    const int nb = (nbr[f] >= 0 && !a.diag_only) ? nbr[f] : ee;
    const double *xn = a.x + (size_t)nb * NB;
#pragma unroll
    for (int q = 0; q < N; q++) {
      const int off =
          dir == 0 ? l * N + q : (dir == 1 ? (l / N) * N2 + q * N + (l % N) : q * N2 + l);
      vd[f][q] = xn[off];
    }
  }
  {
    const fpair *r = rec + (size_t)ee * C::RECW;
    const int woff = a.transpose ? C::NW : 0;
    for (int i = l; i < C::RECU; i += TPC) Am[i] = r[i < 3 * N2 ? i : i + woff];
  }
  fpair col[N];
#pragma unroll
  for (int z = 0; z < N; z++) {
    col[z] = split_bits(cold[z]);
    ue[z * TPC + l] = col[z];
  }
  __syncthreads();

  // ---- neighbour face data: one line per thread per face ----
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int hi = f & 1;
    fpair s1{0.f, 0.f}, s2{0.f, 0.f};
    if (nbr[f] >= 0 && !a.diag_only) {
      const fpair *w = W + f * (N + 1);
      fpair vf[N];
#pragma unroll
      for (int q = 0; q < N; q++) vf[q] = split_bits(vd[f][q]);
      s1 = pmul(w[0], vf[0]);
#pragma unroll
      for (int q = 1; q < N; q++) pmac(s1, w[q], vf[q]);
      s2 = pmul(w[N], vf[hi ? 0 : N - 1]);
    }
    fa[(2 * f) * TPC + l] = norm(s1);
    fa[(2 * f + 1) * TPC + l] = norm(s2);
  }
  __syncthreads();

  const int tr = a.transpose;
  auto Aat = [&](int dir, int i, int q) -> fpair {
    return Am[dir * N2 + (tr ? q * N + i : i * N + q)];
  };
  const int tx = l % N, ty = l / N;
  fpair Arx[N], Ary[N], Mtx[N], Mty[N];
#pragma unroll
  for (int q = 0; q < N; q++) {
    Arx[q] = Aat(0, tx, q);
    Ary[q] = Aat(1, ty, q);
    Mtx[q] = tM[tx * N + q];
    Mty[q] = tM[ty * N + q];
  }
  const fpair d0x = td0[tx], d1x = td1[tx], d0y = td0[ty], d1y = td1[ty];
  const fpair zf0 = fa[8 * TPC + l], zf1 = fa[9 * TPC + l];
  const fpair zf2 = fa[10 * TPC + l], zf3 = fa[11 * TPC + l];
  fpair X[N], Y[N], Z[N];
#pragma unroll
  for (int z = 0; z < N; z++) {
    fpair sx = pmul(Arx[0], ue[z * N2 + ty * N]);
    fpair sy = pmul(Ary[0], ue[z * N2 + tx]);
    fpair sz = pmul(Aat(2, z, 0), col[0]);
#pragma unroll
    for (int q = 1; q < N; q++) {
      pmac(sx, Arx[q], ue[z * N2 + ty * N + q]);
      pmac(sy, Ary[q], ue[z * N2 + q * N + tx]);
      pmac(sz, Aat(2, z, q), col[q]);
    }
    const int lx = z * N + ty, ly = z * N + tx;
    if (tx == 0) padd(sx, fa[0 * TPC + lx]);
    pmac(sx, d0x, fa[1 * TPC + lx]);
    if (tx == N - 1) padd(sx, fa[2 * TPC + lx]);
    pmac(sx, d1x, fa[3 * TPC + lx]);
    if (ty == 0) padd(sy, fa[4 * TPC + ly]);
    pmac(sy, d0y, fa[5 * TPC + ly]);
    if (ty == N - 1) padd(sy, fa[6 * TPC + ly]);
    pmac(sy, d1y, fa[7 * TPC + ly]);
    if (z == 0) padd(sz, zf0);
    pmac(sz, td0[z], zf1);
    if (z == N - 1) padd(sz, zf2);
    pmac(sz, td1[z], zf3);
    X[z] = norm(sx);
    Y[z] = norm(sy);
    Z[z] = norm(sz);
  }
#pragma unroll
  for (int z = 0; z < N; z++) {
    Xs[z * N2 + l] = X[z];
    Ys[z * N2 + l] = Y[z];
    Zs[z * N2 + l] = Z[z];
  }
  __syncthreads();
  // W = M_y X + M_x Y ; T1 = M_x Z   (tangential masses; scales are in A')
  fpair Wv[N];
#pragma unroll
  for (int z = 0; z < N; z++) {
    fpair w = pmul(Mty[0], Xs[z * N2 + tx]);
    fpair t1 = pmul(Mtx[0], Zs[z * N2 + ty * N]);
    pmac(w, Mtx[0], Ys[z * N2 + ty * N]);
#pragma unroll
    for (int q = 1; q < N; q++) {
      pmac(w, Mty[q], Xs[z * N2 + q * N + tx]);
      pmac(w, Mtx[q], Ys[z * N2 + ty * N + q]);
      pmac(t1, Mtx[q], Zs[z * N2 + ty * N + q]);
    }
    Wv[z] = norm(w);
    ue[z * N2 + l] = norm(t1);   // ue is free: all reads finished before the sync
  }
  __syncthreads();
  // out = M_z W + M_y T1, joined to FP64
  if (active) {
    double *ye = a.y + (size_t)e * NB;
    const double *ad = a.add ? a.add + (size_t)e * NB : nullptr;
    const bool scale = a.alpha != 1.0;
#pragma unroll
    for (int z = 0; z < N; z++) {
      fpair s = pmul(tM[z * N], Wv[0]);
      pmac(s, Mty[0], ue[z * N2 + tx]);
#pragma unroll
      for (int q = 1; q < N; q++) {
        pmac(s, tM[z * N + q], Wv[q]);
        pmac(s, Mty[q], ue[z * N2 + q * N + tx]);
      }
      const int idx = z * TPC + l;
      double r = join(s);
      if (scale) r *= a.alpha;
      if (a.accumulate) r += ye[idx];
      if (ad) r += ad[idx];
      ye[idx] = r;
    }
  }
}

template <int N>
static int launch_fp_n(pdg_context *ctx, const ApplyArgs<double> &a, const OpParams<double> &p) {
  using C = FpCfg<N>;
  const size_t smem = sizeof(fpair) * (C::TAB + C::CPB * C::PER_CELL);
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply_fp<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_dev = ctx->device;
  }
  const long work = (a.cells || a.ncells > 0) ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  k_apply_fp<N><<<blocks, C::THREADS, smem, ctx->stream>>>(
      p, a, reinterpret_cast<const fpair *>(ctx->recfp),
      reinterpret_cast<const fpair *>(ctx->tabfp));
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// ---- the mass-factored form in float pairs, two z-columns per instruction ----
// Same arithmetic as k_apply_m (pdg_apply_m.cu): y = (Mhat x Mhat x Mhat) S,
// S = sum_dir (Mhat^-1 A'_dir) u + the face terms lifted by Mhat^-1, with
// every value a float pair.  The chains of two z-levels of a thread's column
// run in the two lanes of paired FP32 instructions (FFMA2 / FADD2 / FMUL2, one
// issue for two lanes); a factor common to both levels is broadcast.  The
// shared arrays hold, per z-pair, (hi_z0, hi_z1, lo_z0, lo_z1) as one 16-byte
// vector, so one load gives both lanes of a pair.  With N odd the last pair's
// second lane duplicates the first and is not stored.
struct f2p {
  float2 hi, lo;
};
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 bcf(float s) { return make_float2(s, s); }
// acc += a * b (lane-wise pmac)
__device__ __forceinline__ void pmac2(f2p &acc, const f2p &a, const f2p &b) {
  const float2 p = __fmul2_rn(a.hi, b.hi);
  const float2 e = __ffma2_rn(a.hi, b.hi, neg2(p));
  const float2 c = __ffma2_rn(a.hi, b.lo, __ffma2_rn(a.lo, b.hi, e));
  const float2 s = __fadd2_rn(acc.hi, p);
  const float2 bb = sub2(s, acc.hi);
  const float2 t = __fadd2_rn(sub2(acc.hi, sub2(s, bb)), sub2(p, bb));
  acc.hi = s;
  acc.lo = __fadd2_rn(acc.lo, __fadd2_rn(t, c));
}
__device__ __forceinline__ f2p pmul2(const f2p &a, const f2p &b) {
  const float2 p = __fmul2_rn(a.hi, b.hi);
  const float2 e = __ffma2_rn(a.hi, b.hi, neg2(p));
  return f2p{p, __ffma2_rn(a.hi, b.lo, __ffma2_rn(a.lo, b.hi, e))};
}
__device__ __forceinline__ f2p norm2(const f2p &a) {
  const float2 s = __fadd2_rn(a.hi, a.lo);
  return f2p{s, sub2(a.lo, sub2(s, a.hi))};
}
__device__ __forceinline__ f2p bcp(fpair a) { return f2p{bcf(a.hi), bcf(a.lo)}; }
__device__ __forceinline__ f2p from4(float4 v) {
  return f2p{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ float4 to4(const f2p &a) {
  return make_float4(a.hi.x, a.hi.y, a.lo.x, a.lo.y);
}
// lane k of a pair as a float pair
__device__ __forceinline__ fpair lane(const f2p &a, int k) {
  return k ? fpair{a.hi.y, a.lo.y} : fpair{a.hi.x, a.lo.x};
}

template <int N>
struct FpmCfg {
  static constexpr int N2 = N * N, NB = N * N * N, TPC = N * N, NF = 6, NZP = (N + 1) / 2;
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  static constexpr int NW = NF * (N + 1);
  static constexpr int RECM = 3 * N2 + NW;          // Mhat^-1 A'_dir, the operator's lines
  static constexpr int TAB = N2 + 4 * N;            // Mhat, m0, m1, md0, md1
  // per cell, in 16-byte units: U (NZP N2), S (NZP N2), face data as fpairs
  // (2 NF TPC / 2), record as fpairs (RECM / 2, rounded up); one unit of padding
  static constexpr int PER_CELL = 2 * NZP * N2 + NF * TPC + (RECM + 1) / 2 + 1;
  static constexpr int TAB16 = (TAB + 1) / 2;
  static constexpr int MINB = N == 3 ? 6 : 0;
};

template <int N>
__global__ void __launch_bounds__(FpmCfg<N>::THREADS, FpmCfg<N>::MINB)
    k_apply_fpm(const OpParams<double> p, const ApplyArgs<double> a,
                const fpair *__restrict__ rec, const fpair *__restrict__ tab) {
  using C = FpmCfg<N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB, NF = C::NF, NZP = C::NZP;
  extern __shared__ __align__(16) float4 fpm_raw[];
  fpair *T = reinterpret_cast<fpair *>(fpm_raw);                 // tables
  const fpair *tM = T, *tm0 = T + N2, *tm1 = tm0 + N, *tmd0 = tm1 + N, *tmd1 = tmd0 + N;
  const int t = threadIdx.x;
  const int cs = t / TPC;
  const int l = t - cs * TPC;
  float4 *UP = fpm_raw + C::TAB16 + cs * C::PER_CELL;   // [NZP][N2] z-pairs
  float4 *SP = UP + NZP * N2;                           // [NZP][N2]
  fpair *fa = reinterpret_cast<fpair *>(SP + NZP * N2);  // [2 NF][TPC]
  fpair *R = fa + 2 * NF * TPC;                          // record
  const fpair *W = R + 3 * N2;

  if (a.skip && *a.skip) return;
  for (int i = t; i < C::TAB; i += blockDim.x) T[i] = tab[i];

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
  double cold[N];
  const double *xe = a.x + (size_t)ee * NB;
#pragma unroll
  for (int z = 0; z < N; z++) cold[z] = xe[z * TPC + l];
  double vd[NF][N];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int dir = f >> 1;
    const int nb = nbr[f] >= 0 ? nbr[f] : ee;
    const double *xn = a.x + (size_t)nb * NB;
#pragma unroll
    for (int q = 0; q < N; q++) {
      const int off =
          dir == 0 ? l * N + q : (dir == 1 ? (l / N) * N2 + q * N + (l % N) : q * N2 + l);
      vd[f][q] = xn[off];
    }
  }
  {
    const fpair *r = rec + (size_t)ee * C::RECM;
    for (int i = l; i < C::RECM; i += TPC) R[i] = r[i];
  }
  fpair col[N];
#pragma unroll
  for (int z = 0; z < N; z++) col[z] = split_bits(cold[z]);
#pragma unroll
  for (int zp = 0; zp < NZP; zp++) {
    const fpair c0 = col[2 * zp], c1 = col[2 * zp + 1 < N ? 2 * zp + 1 : 2 * zp];
    UP[zp * N2 + l] = make_float4(c0.hi, c1.hi, c0.lo, c1.lo);
  }
  __syncthreads();

  // ---- neighbour face data: one line per thread per face ----
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int hi = f & 1;
    fpair s1{0.f, 0.f}, s2{0.f, 0.f};
    if (nbr[f] >= 0) {
      const fpair *w = W + f * (N + 1);
      fpair vf[N];
#pragma unroll
      for (int q = 0; q < N; q++) vf[q] = split_bits(vd[f][q]);
      s1 = pmul(w[0], vf[0]);
#pragma unroll
      for (int q = 1; q < N; q++) pmac(s1, w[q], vf[q]);
      s2 = pmul(w[N], vf[hi ? 0 : N - 1]);
    }
    fa[(2 * f) * TPC + l] = norm(s1);
    fa[(2 * f + 1) * TPC + l] = norm(s2);
  }
  __syncthreads();

  const int tx = l % N, ty = l / N;
  // ---- S = sum_dir B_dir u + lifted face terms, two z-levels per chain ----
  {
    const f2p m0x = bcp(tm0[tx]), m1x = bcp(tm1[tx]), md0x = bcp(tmd0[tx]), md1x = bcp(tmd1[tx]);
    const f2p m0y = bcp(tm0[ty]), m1y = bcp(tm1[ty]), md0y = bcp(tmd0[ty]), md1y = bcp(tmd1[ty]);
    const f2p zf0 = bcp(fa[8 * TPC + l]), zf1 = bcp(fa[9 * TPC + l]);
    const f2p zf2 = bcp(fa[10 * TPC + l]), zf3 = bcp(fa[11 * TPC + l]);
#pragma unroll
    for (int zp = 0; zp < NZP; zp++) {
      const int z0 = 2 * zp, z1 = 2 * zp + 1 < N ? 2 * zp + 1 : 2 * zp;
      f2p s = pmul2(bcp(R[tx * N]), from4(UP[zp * N2 + ty * N]));
      pmac2(s, bcp(R[N2 + ty * N]), from4(UP[zp * N2 + tx]));
#pragma unroll
      for (int q = 1; q < N; q++) {
        pmac2(s, bcp(R[tx * N + q]), from4(UP[zp * N2 + ty * N + q]));
        pmac2(s, bcp(R[N2 + ty * N + q]), from4(UP[zp * N2 + q * N + tx]));
      }
#pragma unroll
      for (int q = 0; q < N; q++) {
        const fpair b0 = R[2 * N2 + z0 * N + q], b1 = R[2 * N2 + z1 * N + q];
        pmac2(s, f2p{make_float2(b0.hi, b1.hi), make_float2(b0.lo, b1.lo)}, bcp(col[q]));
      }
      auto fp2 = [&](int arr, int i0, int i1) -> f2p {
        const fpair u0 = fa[arr * TPC + i0], u1 = fa[arr * TPC + i1];
        return f2p{make_float2(u0.hi, u1.hi), make_float2(u0.lo, u1.lo)};
      };
      const int lx0 = z0 * N + ty, lx1 = z1 * N + ty, ly0 = z0 * N + tx, ly1 = z1 * N + tx;
      pmac2(s, m0x, fp2(0, lx0, lx1));
      pmac2(s, md0x, fp2(1, lx0, lx1));
      pmac2(s, m1x, fp2(2, lx0, lx1));
      pmac2(s, md1x, fp2(3, lx0, lx1));
      pmac2(s, m0y, fp2(4, ly0, ly1));
      pmac2(s, md0y, fp2(5, ly0, ly1));
      pmac2(s, m1y, fp2(6, ly0, ly1));
      pmac2(s, md1y, fp2(7, ly0, ly1));
      auto tp2 = [&](const fpair *tb) -> f2p {
        return f2p{make_float2(tb[z0].hi, tb[z1].hi), make_float2(tb[z0].lo, tb[z1].lo)};
      };
      pmac2(s, tp2(tm0), zf0);
      pmac2(s, tp2(tmd0), zf1);
      pmac2(s, tp2(tm1), zf2);
      pmac2(s, tp2(tmd1), zf3);
      SP[zp * N2 + l] = to4(norm2(s));
    }
  }
  __syncthreads();
  // ---- S1 = Mhat_x S (into UP: its reads finished before the sync) ----
#pragma unroll
  for (int zp = 0; zp < NZP; zp++) {
    f2p s = pmul2(bcp(tM[tx * N]), from4(SP[zp * N2 + ty * N]));
#pragma unroll
    for (int q = 1; q < N; q++) pmac2(s, bcp(tM[tx * N + q]), from4(SP[zp * N2 + ty * N + q]));
    UP[zp * N2 + l] = to4(norm2(s));
  }
  __syncthreads();
  // ---- S2 = Mhat_y S1 (own column), out = Mhat_z S2 ----
  f2p s2c[NZP];
#pragma unroll
  for (int zp = 0; zp < NZP; zp++) {
    f2p s = pmul2(bcp(tM[ty * N]), from4(UP[zp * N2 + tx]));
#pragma unroll
    for (int q = 1; q < N; q++) pmac2(s, bcp(tM[ty * N + q]), from4(UP[zp * N2 + q * N + tx]));
    s2c[zp] = norm2(s);
  }
  if (active) {
    double *ye = a.y + (size_t)e * NB;
    const double *ad = a.add ? a.add + (size_t)e * NB : nullptr;
    const bool scale = a.alpha != 1.0;
#pragma unroll
    for (int zp = 0; zp < NZP; zp++) {
      const int z0 = 2 * zp, z1 = 2 * zp + 1 < N ? 2 * zp + 1 : 2 * zp;
      f2p o = pmul2(f2p{make_float2(tM[z0 * N].hi, tM[z1 * N].hi),
                        make_float2(tM[z0 * N].lo, tM[z1 * N].lo)},
                    bcp(lane(s2c[0], 0)));
#pragma unroll
      for (int q = 1; q < N; q++)
        pmac2(o, f2p{make_float2(tM[z0 * N + q].hi, tM[z1 * N + q].hi),
                     make_float2(tM[z0 * N + q].lo, tM[z1 * N + q].lo)},
              bcp(lane(s2c[q >> 1], q & 1)));
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const int z = 2 * zp + k;
        if (z >= N) break;
        const int idx = z * TPC + l;
        double r = join(lane(o, k));
        if (scale) r *= a.alpha;
        if (a.accumulate) r += ye[idx];
        if (ad) r += ad[idx];
        ye[idx] = r;
      }
    }
  }
}

template <int N>
static int launch_fpm_n(pdg_context *ctx, const ApplyArgs<double> &a, const OpParams<double> &p) {
  using C = FpmCfg<N>;
  const size_t smem = 16 * (C::TAB16 + C::CPB * C::PER_CELL);
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply_fpm<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_dev = ctx->device;
  }
  const long work = a.ncells > 0 ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  k_apply_fpm<N><<<blocks, C::THREADS, smem, ctx->stream>>>(
      p, a, reinterpret_cast<const fpair *>(ctx->recfpm),
      reinterpret_cast<const fpair *>(ctx->tabfpm));
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

// Float-pair copies of the FP64 records (rec64, built before this call) and
// of the 1D tables
static int ensure_pairs(pdg_context *ctx, long rec_doubles) {
  if (ctx->recfp_valid) return PDG_OK;
  if (!ctx->recfp) PDG_CUDA_TRY(cudaMalloc(&ctx->recfp, sizeof(fpair) * rec_doubles));
  const long ntab = 2 * ctx->N * ctx->N + 2 * ctx->N;
  if (!ctx->tabfp) {
    PDG_CUDA_TRY(cudaMalloc(&ctx->tabfp, sizeof(fpair) * ntab));
    k_to_pairs<<<1, 128, 0, ctx->stream>>>(ntab, ctx->tab64, (fpair *)ctx->tabfp);
    PDG_CUDA_TRY(cudaGetLastError());
  }
  k_to_pairs<<<(unsigned)((rec_doubles + 255) / 256), 256, 0, ctx->stream>>>(
      rec_doubles, ctx->rec64, (fpair *)ctx->recfp);
  PDG_CUDA_TRY(cudaGetLastError());
  ctx->recfp_valid = 1;
  return PDG_OK;
}

// float-pair copies of the mass-factored records and tables (rec64m)
static int ensure_pairs_m(pdg_context *ctx, long rec_doubles, int ntab) {
  if (ctx->recfpm_valid) return PDG_OK;
  PDG_TRY(prepare_apply_m(ctx));
  if (!ctx->recfpm) PDG_CUDA_TRY(cudaMalloc(&ctx->recfpm, sizeof(fpair) * rec_doubles));
  if (!ctx->tabfpm) {
    PDG_CUDA_TRY(cudaMalloc(&ctx->tabfpm, sizeof(fpair) * ntab));
    k_to_pairs<<<1, 128, 0, ctx->stream>>>(ntab, ctx->tabm64, (fpair *)ctx->tabfpm);
    PDG_CUDA_TRY(cudaGetLastError());
  }
  k_to_pairs<<<(unsigned)((rec_doubles + 255) / 256), 256, 0, ctx->stream>>>(
      rec_doubles, ctx->rec64m, (fpair *)ctx->recfpm);
  PDG_CUDA_TRY(cudaGetLastError());
  ctx->recfpm_valid = 1;
  return PDG_OK;
}

template <int N>
static int prepare_fp_n(pdg_context *ctx) {
  PDG_TRY(ensure_pairs(ctx, (long)FpCfg<N>::RECW * ctx->ncell));
  if (ctx->tabm64) PDG_TRY(ensure_pairs_m(ctx, (long)FpmCfg<N>::RECM * ctx->ncell, FpmCfg<N>::TAB));
  return PDG_OK;
}

// the float-pair copies, built on the context stream (before a launch is
// spread over several streams)
int prepare_float_pair(pdg_context *ctx) {
  switch (ctx->N) {
    case 2: return prepare_fp_n<2>(ctx);
    case 3: return prepare_fp_n<3>(ctx);
    case 4: return prepare_fp_n<4>(ctx);
    case 5: return prepare_fp_n<5>(ctx);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

int launch_apply_float_pair(pdg_context *ctx, const ApplyArgs<double> &a) {
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  PDG_TRY(prepare_float_pair(ctx));
#ifndef PDG_FPM
#define PDG_FPM 1
#endif
  if (PDG_FPM && ctx->tabm64 && !a.transpose && !a.diag_only && !a.cells) {
    // the mass-factored form, two z-levels per paired instruction
    switch (ctx->N) {
      case 2: return launch_fpm_n<2>(ctx, a, p);
      case 3: return launch_fpm_n<3>(ctx, a, p);
      case 4: return launch_fpm_n<4>(ctx, a, p);
      case 5: return launch_fpm_n<5>(ctx, a, p);
      default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
    }
  }
  switch (ctx->N) {
    case 2: return launch_fp_n<2>(ctx, a, p);
    case 3: return launch_fp_n<3>(ctx, a, p);
    case 4: return launch_fp_n<4>(ctx, a, p);
    case 5: return launch_fp_n<5>(ctx, a, p);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

}  // namespace pdg
