// pdg_tma.cuh -- tensor-memory-accelerator staging, mbarrier waits and the
// shared-memory / paired-FP32 helpers of the plane-per-thread Q3 kernels (the
// FP32 operator and the FP32 FDM block Jacobi).
#pragma once

#include <cuda.h>

#include "pdg_internal.cuh"

namespace pdg {

// ---- TMA / mbarrier helpers (inline PTX) ------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
// true once phase `parity` of the barrier completed; at most `limit` polls
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit) {
  for (int it = 0; it < limit; it++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, int c0, int c1,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_load(unsigned dst, const void *src, unsigned bytes,
                                          unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst), "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
// polls of the staging barrier before a launch gives up (far above any
// real copy time); the kernel then records the failure and returns
constexpr int kTmaPolls = 1 << 22;

// byte offset of row y of plane z of cell c in a swizzled run buffer
__device__ __forceinline__ unsigned q3_swz_row(int c, int z, int y) {
  return 16u * (unsigned)(16 * c + 8 * (z >> 1) + 4 * ((z & 1) ^ ((c >> 1) & 1)) +
                          ((2 * (c & 1) | (z >> 1)) ^ y));
}
__device__ __forceinline__ float4 sh4(const unsigned char *b, unsigned off) {
  return *reinterpret_cast<const float4 *>(b + off);
}
__device__ __forceinline__ void st4(unsigned char *b, unsigned off, float4 v) {
  *reinterpret_cast<float4 *>(b + off) = v;
}
__device__ __forceinline__ float f4c(const float4 &v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}
// 32-byte global vector accesses (32-byte aligned addresses)
__device__ __forceinline__ void ld8(const float *p, float *w) {
  asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(w[0]), "=f"(w[1]), "=f"(w[2]), "=f"(w[3]), "=f"(w[4]), "=f"(w[5]),
                 "=f"(w[6]), "=f"(w[7])
               : "l"(p));
}
__device__ __forceinline__ void st8(float *p, const float *w) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(w[0]),
               "f"(w[1]), "f"(w[2]), "f"(w[3]), "f"(w[4]), "f"(w[5]), "f"(w[6]), "f"(w[7])
               : "memory");
}

// paired FP32 arithmetic (one instruction for two lanes; a scalar operand
// is broadcast to both)
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// Tensor maps of an FP32 vector as 128-byte lines (32 floats, the 128-byte
// swizzle, zeros outside): boxes of kLinesOwn lines (a run of 32 cells with
// one halo cell each side) and of kLinesRun lines (a run of 32 cells).
// Cached per host thread for the last few vectors; false if the vector
// cannot be described (the caller then takes its per-thread copy path).
constexpr unsigned kLinesOwn = 68, kLinesRun = 64;
bool q3_lines_maps(const float *x, long ndof, const CUtensorMap **own, const CUtensorMap **run);

}  // namespace pdg
