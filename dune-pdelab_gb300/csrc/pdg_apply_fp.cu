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
    case 2: return launch_fp_n<2>(ctx, a, p);
    case 3: return launch_fp_n<3>(ctx, a, p);
    case 4: return launch_fp_n<4>(ctx, a, p);
    case 5: return launch_fp_n<5>(ctx, a, p);
    default: return set_error(PDG_EUNSUPPORTED, "degree not compiled in");
  }
}

}  // namespace pdg
