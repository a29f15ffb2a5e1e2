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
  static constexpr int N2 = N * N, NF = 6;
  static constexpr int NW = NF * (N + 1);               // neighbour-line coefficients
  static constexpr int RECW = 3 * N2 + 2 * NW;          // FP64 record (both forms)
  // blocks per SM the register allocation must allow: 6 for Q2 (0.262 against
  // 0.287 ms per 64^3 apply with the compiler's free choice, one z-level per
  // instruction), the compiler's choice otherwise (Q4 bounded to 6 blocks:
  // 0.416 against 0.374 ms at 40^3)
  static constexpr int MINB = N == 3 ? 6 : 0;
};

// ---- the kernel: two z-levels per paired FP32 instruction ---------------------
// Thread mapping and records of k_apply<double, 3, N>: N*N threads per cell,
// each holding a z-column.  Each thread's chains for the z-levels z0 = 2 zp and
// z1 = 2 zp + 1 run in the two lanes of FFMA2 / FADD2 / FMUL2 (one issue for
// two lanes; a factor common to both levels is broadcast); every lane performs
// the scalar float-pair operations (pmul / pmac / padd / norm) on its chain in
// the scalar order, a lane-wise condition as the addition of an exact zero.
// The shared arrays hold per z-pair (hi_z0, hi_z1, lo_z0, lo_z1) as one
// 16-byte vector; with N odd the second lane of the last pair repeats the
// first and is not stored.  (0.252 against 0.262 ms per 64^3 Q2 apply for the
// same arithmetic one level per instruction, identical results.)
struct f2p {
  float2 hi, lo;
};
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 bcf(float s) { return make_float2(s, s); }
// acc += a * b, lane-wise pmac
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
// acc += a, lane-wise padd
__device__ __forceinline__ void padd2(f2p &acc, const f2p &a) {
  const float2 s = __fadd2_rn(acc.hi, a.hi);
  const float2 bb = sub2(s, acc.hi);
  const float2 t = __fadd2_rn(sub2(acc.hi, sub2(s, bb)), sub2(a.hi, bb));
  acc.hi = s;
  acc.lo = __fadd2_rn(acc.lo, __fadd2_rn(t, a.lo));
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
__device__ __forceinline__ f2p two(fpair a, fpair b) {
  return f2p{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)};
}
__device__ __forceinline__ f2p from4(float4 v) {
  return f2p{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ float4 to4(const f2p &a) {
  return make_float4(a.hi.x, a.hi.y, a.lo.x, a.lo.y);
}
__device__ __forceinline__ fpair lane(const f2p &a, int k) {
  return k ? fpair{a.hi.y, a.lo.y} : fpair{a.hi.x, a.lo.x};
}

template <int N>
struct Fp2Cfg {
  static constexpr int N2 = N * N, NB = N * N * N, TPC = N * N, NF = 6, NZP = (N + 1) / 2;
  static constexpr int CPB = (128 / TPC) > 0 ? (128 / TPC) : 1;
  static constexpr int THREADS = CPB * TPC;
  static constexpr int NW = NF * (N + 1);
  static constexpr int RECW = 3 * N2 + 2 * NW;
  static constexpr int RECU = 3 * N2 + NW;
  static constexpr int TAB = 2 * N2 + 2 * N;            // Mhat, Shat, d0, d1
  // per cell in 16-byte units: U, X, Y, Z as z-pairs (4 NZP N2), face data
  // (12 TPC fpairs), record part (RECU fpairs); one unit of padding
  static constexpr int PER_CELL = 4 * NZP * N2 + 6 * TPC + (RECU + 1) / 2 + 1;
  static constexpr int TAB16 = (TAB + 1) / 2;
  static constexpr int MINB = FpCfg<N>::MINB;
};

template <int N>
__global__ void __launch_bounds__(Fp2Cfg<N>::THREADS, Fp2Cfg<N>::MINB)
    k_apply_fp2(const OpParams<double> p, const ApplyArgs<double> a,
                const fpair *__restrict__ rec, const fpair *__restrict__ tab) {
  using C = Fp2Cfg<N>;
  constexpr int N2 = C::N2, NB = C::NB, TPC = C::TPC, CPB = C::CPB, NF = C::NF, NZP = C::NZP;
  extern __shared__ __align__(16) float4 fp2_raw[];
  fpair *tM = reinterpret_cast<fpair *>(fp2_raw);
  fpair *td0 = tM + 2 * N2;          // (Shat is not needed: it is folded into the record)
  fpair *td1 = td0 + N;
  const int t = threadIdx.x;
  const int cs = t / TPC;
  const int l = t - cs * TPC;
  float4 *UP = fp2_raw + C::TAB16 + cs * C::PER_CELL;   // [NZP][N2]
  float4 *XP = UP + NZP * N2, *YP = XP + NZP * N2, *ZP = YP + NZP * N2;
  fpair *fa = reinterpret_cast<fpair *>(ZP + NZP * N2);  // [2 NF][TPC]
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
  const f2p d0x = bcp(td0[tx]), d1x = bcp(td1[tx]), d0y = bcp(td0[ty]), d1y = bcp(td1[ty]);
  const fpair zf0 = fa[8 * TPC + l], zf1 = fa[9 * TPC + l];
  const fpair zf2 = fa[10 * TPC + l], zf3 = fa[11 * TPC + l];
  const fpair zero{0.f, 0.f};
  // ---- X, Y, Z: the directional operators with the face terms ----
#pragma unroll
  for (int zp = 0; zp < NZP; zp++) {
    const int z0 = 2 * zp, z1 = 2 * zp + 1 < N ? 2 * zp + 1 : 2 * zp;
    f2p sx = pmul2(bcp(Arx[0]), from4(UP[zp * N2 + ty * N]));
    f2p sy = pmul2(bcp(Ary[0]), from4(UP[zp * N2 + tx]));
    f2p sz = pmul2(two(Aat(2, z0, 0), Aat(2, z1, 0)), bcp(col[0]));
#pragma unroll
    for (int q = 1; q < N; q++) {
      pmac2(sx, bcp(Arx[q]), from4(UP[zp * N2 + ty * N + q]));
      pmac2(sy, bcp(Ary[q]), from4(UP[zp * N2 + q * N + tx]));
      pmac2(sz, two(Aat(2, z0, q), Aat(2, z1, q)), bcp(col[q]));
    }
    const int lx0 = z0 * N + ty, lx1 = z1 * N + ty, ly0 = z0 * N + tx, ly1 = z1 * N + tx;
    auto fp2 = [&](int arr, int i0, int i1) -> f2p {
      return two(fa[arr * TPC + i0], fa[arr * TPC + i1]);
    };
    if (tx == 0) padd2(sx, fp2(0, lx0, lx1));
    pmac2(sx, d0x, fp2(1, lx0, lx1));
    if (tx == N - 1) padd2(sx, fp2(2, lx0, lx1));
    pmac2(sx, d1x, fp2(3, lx0, lx1));
    if (ty == 0) padd2(sy, fp2(4, ly0, ly1));
    pmac2(sy, d0y, fp2(5, ly0, ly1));
    if (ty == N - 1) padd2(sy, fp2(6, ly0, ly1));
    pmac2(sy, d1y, fp2(7, ly0, ly1));
    // z faces: the lower-face value enters level 0 only, the upper one level N-1
    padd2(sz, two(z0 == 0 ? zf0 : zero, z1 == 0 ? zf0 : zero));
    pmac2(sz, two(td0[z0], td0[z1]), bcp(zf1));
    padd2(sz, two(z0 == N - 1 ? zf2 : zero, z1 == N - 1 ? zf2 : zero));
    pmac2(sz, two(td1[z0], td1[z1]), bcp(zf3));
    XP[zp * N2 + l] = to4(norm2(sx));
    YP[zp * N2 + l] = to4(norm2(sy));
    ZP[zp * N2 + l] = to4(norm2(sz));
  }
  __syncthreads();
  // W = M_y X + M_x Y ; T1 = M_x Z   (tangential masses; scales are in A')
  f2p Wv[NZP];
#pragma unroll
  for (int zp = 0; zp < NZP; zp++) {
    f2p w = pmul2(bcp(Mty[0]), from4(XP[zp * N2 + tx]));
    f2p t1 = pmul2(bcp(Mtx[0]), from4(ZP[zp * N2 + ty * N]));
    pmac2(w, bcp(Mtx[0]), from4(YP[zp * N2 + ty * N]));
#pragma unroll
    for (int q = 1; q < N; q++) {
      pmac2(w, bcp(Mty[q]), from4(XP[zp * N2 + q * N + tx]));
      pmac2(w, bcp(Mtx[q]), from4(YP[zp * N2 + ty * N + q]));
      pmac2(t1, bcp(Mtx[q]), from4(ZP[zp * N2 + ty * N + q]));
    }
    Wv[zp] = norm2(w);
    UP[zp * N2 + l] = to4(norm2(t1));   // UP is free: all reads finished before the sync
  }
  __syncthreads();
  // out = M_z W + M_y T1, joined to FP64
  if (active) {
    double *ye = a.y + (size_t)e * NB;
    const double *ad = a.add ? a.add + (size_t)e * NB : nullptr;
    const bool scale = a.alpha != 1.0;
#pragma unroll
    for (int zp = 0; zp < NZP; zp++) {
      const int z0 = 2 * zp, z1 = 2 * zp + 1 < N ? 2 * zp + 1 : 2 * zp;
      f2p s = pmul2(two(tM[z0 * N], tM[z1 * N]), bcp(lane(Wv[0], 0)));
      pmac2(s, bcp(Mty[0]), from4(UP[zp * N2 + tx]));
#pragma unroll
      for (int q = 1; q < N; q++) {
        pmac2(s, two(tM[z0 * N + q], tM[z1 * N + q]), bcp(lane(Wv[q >> 1], q & 1)));
        pmac2(s, bcp(Mty[q]), from4(UP[zp * N2 + q * N + tx]));
      }
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const int z = 2 * zp + k;
        if (z >= N) break;
        const int idx = z * TPC + l;
        double r = join(lane(s, k));
        if (scale) r *= a.alpha;
        if (a.accumulate) r += ye[idx];
        if (ad) r += ad[idx];
        ye[idx] = r;
      }
    }
  }
}

template <int N>
static int launch_fp2_n(pdg_context *ctx, const ApplyArgs<double> &a, const OpParams<double> &p) {
  using C = Fp2Cfg<N>;
  const size_t smem = 16 * (C::TAB16 + C::CPB * C::PER_CELL);
  static int attr_dev = -1;
  if (attr_dev != ctx->device) {
    PDG_CUDA_TRY(cudaFuncSetAttribute(k_apply_fp2<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr_dev = ctx->device;
  }
  const long work = (a.cells || a.ncells > 0) ? a.ncells : ctx->ncell;
  if (work <= 0) return PDG_OK;
  const unsigned blocks = (unsigned)((work + C::CPB - 1) / C::CPB);
  k_apply_fp2<N><<<blocks, C::THREADS, smem, ctx->stream>>>(
      p, a, reinterpret_cast<const fpair *>(ctx->recfp),
      reinterpret_cast<const fpair *>(ctx->tabfp));
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

// the float-pair copies, built on the context stream (before a launch is
// spread over several streams)
int prepare_float_pair(pdg_context *ctx) {
  switch (ctx->N) {
    case 2: return ensure_pairs(ctx, (long)FpCfg<2>::RECW * ctx->ncell);
    case 3: return ensure_pairs(ctx, (long)FpCfg<3>::RECW * ctx->ncell);
    case 4: return ensure_pairs(ctx, (long)FpCfg<4>::RECW * ctx->ncell);
    case 5: return ensure_pairs(ctx, (long)FpCfg<5>::RECW * ctx->ncell);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

int launch_apply_float_pair(pdg_context *ctx, const ApplyArgs<double> &a) {
  OpParams<double> p = make_params<double>(ctx, ctx->K64, ctx->c64, ctx->tab64);
  PDG_TRY(prepare_float_pair(ctx));
  switch (ctx->N) {
    case 2: return launch_fp2_n<2>(ctx, a, p);
    case 3: return launch_fp2_n<3>(ctx, a, p);
    case 4: return launch_fp2_n<4>(ctx, a, p);
    case 5: return launch_fp2_n<5>(ctx, a, p);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

}  // namespace pdg
