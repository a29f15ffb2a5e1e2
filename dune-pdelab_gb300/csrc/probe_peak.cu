// probe_peak.cu -- measurement helper for bench.py: sustained FP64 / FP32
// fused-multiply-add throughput of this GPU's CUDA cores (not the product
// path).  The operator kernels run on the FP64 / FP32 pipes, so these are
// the roofline denominators for their arithmetic.  A second probe measures
// the FP64 tensor-core path (warp-level mma.sync of f64 operands), the only
// FP64 matrix instruction sm_103a has, to decide whether the FP64 operator's
// small contractions could move there.
//
// Each thread runs 8 independent FMA chains for `iters` steps; the result
// is written out so the compiler keeps the work.
#include <cuda_runtime.h>

template <typename T>
__global__ void k_fma(int iters, T a, T b, T *out) {
  T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
static int run(int iters, double *tflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * threads * blocks) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma<T><<<blocks, threads>>>(iters / 10, T(0.999999), T(1e-7), out);   // warm-up
  cudaEventRecord(e0);
  k_fma<T><<<blocks, threads>>>(iters, T(0.999999), T(1e-7), out);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Each warp keeps 8 independent m8n8k4 accumulators (D = A B + D, 512 flops
// per warp instruction); A and B stay in registers.
__global__ void k_dmma(int iters, double a, double b, double *out) {
  double c[8][2];
#pragma unroll
  for (int u = 0; u < 8; u++) { c[u][0] = 0.0; c[u][1] = 0.0; }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
          : "+d"(c[u][0]), "+d"(c[u][1])
          : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int u = 0; u < 8; u++) s += c[u][0] + c[u][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int pdg_probe_dmma_peak(int iters, double *tflops) {
  if (!tflops || iters < 10) return 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dmma<<<blocks, threads>>>(iters / 10, 1e-3, 1e-3, out);   // warm-up
  cudaEventRecord(e0);
  k_dmma<<<blocks, threads>>>(iters, 1e-3, 1e-3, out);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const double warps = (double)threads / 32 * blocks;
  const double flops = 512.0 * 8 * (double)iters * warps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Whether the FP64 tensor path is a second FP64 unit: per iteration 8
// mma.sync m8n8k4 f64 per warp and 64 FP64 FMAs per thread (equal flops),
// interleaved; the rate of both together against each alone.
__global__ void k_fp64_mix(int iters, double a, double b, double *out) {
  double c[8][2], x[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    c[u][0] = 0.0;
    c[u][1] = 0.0;
    x[u] = threadIdx.x * 1e-3 + u;
  }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
          : "+d"(c[u][0]), "+d"(c[u][1])
          : "d"(a), "d"(b));
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int u = 0; u < 8; u++) x[u] = x[u] * a + b;
  }
  double s = 0.0;
#pragma unroll
  for (int u = 0; u < 8; u++) s += c[u][0] + c[u][1] + x[u];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int pdg_probe_fp64_mixed(int iters, double *tflops) {
  if (!tflops || iters < 10) return 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_mix<<<blocks, threads>>>(iters / 10, 0.999, 1e-7, out);   // warm-up
  cudaEventRecord(e0);
  k_fp64_mix<<<blocks, threads>>>(iters, 0.999, 1e-7, out);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const double warps = (double)threads / 32 * blocks;
  const double flops = 512.0 * 8 * (double)iters * warps + 2.0 * 64 * (double)iters * threads * blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

extern "C" int pdg_probe_fma_peak(int precision, int iters, double *tflops) {
  if (!tflops || iters < 10) return 1;
  return precision == 0 ? run<double>(iters, tflops) : run<float>(iters, tflops);
}
