// pdg_noalloc.cu -- a dot product that allocates nothing.
//
// Who needs it: callers that cannot allocate device memory at the point of
// the call.  Work recorded into a CUDA graph by stream capture cannot call
// cudaMalloc while capturing; host solvers that own every buffer (for
// example a dune-istl Krylov loop over device vectors, which asks for a dot
// product or a norm in every iteration) may forbid library allocations
// after set-up; memory-budgeted embeddings must not see hidden
// allocations.  pdg_dot needs a context, and a context owns allocated
// scratch; pdg_dot_noalloc needs neither.
//
// How: the same deterministic two-stage reduction as the context-based dot
// (block partial sums, the last block adds them in block order), with the
// partial sums and the completion ticket kept in one file-scope device array
// of fixed size instead of context memory.  Every GPU that loads the
// library holds this array (8 KiB + 256 B) until the process exits.
#include <mutex>

#include "pdg_internal.cuh"

namespace pdg {
namespace {

constexpr int kNAChunks = 1024;                               // partial sums
constexpr int kNAThreads = 256;
constexpr int kNAPerThread = 256;                             // elements per thread
constexpr long kNAChunk = (long)kNAThreads * kNAPerThread;    // 65,536 elements per block
static_assert(kNAChunk * kNAChunks == PDG_DOT_NOALLOC_MAX_N, "limit in pdg.h");

// [0, kNAChunks): per-block partial sums; word kNAChunks: completion ticket
// (an unsigned int, zero at module load and reset to zero by the last block
// of every call).  Partial slots need no clearing: each call writes every
// slot it reads.
static __device__ __align__(256) double g_noalloc_scratch[kNAChunks + 32];

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double na_block_sum(double v, double *sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = na_warp_sum(v);
  if (lane == 0) sm[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sm[lane] : 0.0;
  if (w == 0) v = na_warp_sum(v);
  __syncthreads();
  return v;   // valid in thread 0
}

__global__ void __launch_bounds__(kNAThreads)
    k_dot_noalloc(long n, const double *__restrict__ a, const double *__restrict__ b,
                  double *__restrict__ result, double *__restrict__ scratch) {
  __shared__ double sm[kNAThreads / 32];
  __shared__ bool last;
  const long base = (long)blockIdx.x * kNAChunk;
  double s = 0.0;
  for (int j = 0; j < kNAPerThread; j++) {
    const long i = base + (long)j * kNAThreads + threadIdx.x;
    if (i < n) s += a[i] * b[i];
  }
  s = na_block_sum(s, sm);
  unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch + kNAChunks);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double t = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
    t += ((volatile double *)scratch)[i];
  t = na_block_sum(t, sm);
  if (threadIdx.x == 0) {
    *result = t;
    *ticket = 0u;
  }
}

// Device address of the scratch array per device, looked up once per device
// with that device current (a host-side use of the symbol itself would name
// host memory, not the device array).
constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
double *g_na_ptr[kMaxDevices] = {};

int scratch_address(int dev, double **out) {
  if (dev < 0 || dev >= kMaxDevices) return set_error(PDG_EINVAL, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return set_error(PDG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_na_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_na_ptr[dev];
  return PDG_OK;
}

bool on_device(const void *p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

}  // namespace
}  // namespace pdg

extern "C" int pdg_dot_noalloc(long n, const double *a, const double *b, double *result,
                               void *stream) {
  using namespace pdg;
  if (n < 0) return set_error(PDG_EINVAL, "pdg_dot_noalloc: n must be >= 0");
  if (n > PDG_DOT_NOALLOC_MAX_N)
    return set_error(PDG_EINVAL,
                     "pdg_dot_noalloc: n exceeds PDG_DOT_NOALLOC_MAX_N (67,108,864 = 1024 "
                     "partial sums of 65,536 elements); use pdg_dot");
  if (!result || (n > 0 && (!a || !b)))
    return set_error(PDG_EINVAL, "pdg_dot_noalloc: null pointer");
  if (!on_device(result) || (n > 0 && (!on_device(a) || !on_device(b))))
    return set_error(PDG_EINVAL, "pdg_dot_noalloc: a, b and result must be device pointers");
  int dev = 0;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_error(PDG_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  double *scratch = nullptr;
  const int st = scratch_address(dev, &scratch);
  if (st != PDG_OK) return st;
  const unsigned blocks = n > 0 ? (unsigned)((n + kNAChunk - 1) / kNAChunk) : 1u;
  k_dot_noalloc<<<blocks, kNAThreads, 0, (cudaStream_t)stream>>>(n, a, b, result, scratch);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess)
    return set_error(PDG_ECUDA, std::string("pdg_dot_noalloc launch: ") + cudaGetErrorString(le));
  return PDG_OK;
}
