// pdg_noalloc.cu -- a dot product that allocates nothing.
//
// Who needs it: callers that cannot allocate device memory at the point of
// the call.  Host solvers that own every buffer (for example a dune-istl
// Krylov loop over device vectors, which asks for a dot product or a norm in
// every iteration) may forbid library allocations after set-up, and
// memory-budgeted embeddings must not see hidden allocations or the
// synchronisation that cudaMalloc and cudaFree bring.  pdg_dot needs a
// context, and a context owns allocated scratch; pdg_dot_noalloc needs
// neither.
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

// Device address of the scratch array per device, looked up with that device
// current (a host-side use of the symbol itself would name host memory, not
// the device array).  The address belongs to the device's current context:
// after cudaDeviceReset the runtime makes a new context, loads the module
// again and the old address is gone, so the cache also keeps the unique id
// of the context the address was taken in and looks the address up again
// when that id changes.
constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
double *g_na_ptr[kMaxDevices] = {};
unsigned long long g_na_ctx[kMaxDevices] = {};

typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

// The unique id of the calling thread's current context (cuCtxGetId through
// the runtime's driver entry point, no link against the driver library);
// 0 if it cannot be had, which forces a fresh lookup on every call.
unsigned long long current_context_id() {
  static std::once_flag once;
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

int scratch_address(int dev, double **out) {
  if (dev < 0 || dev >= kMaxDevices) return set_error(PDG_EINVAL, "device ordinal out of range");
  const unsigned long long ctx_id = current_context_id();
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev] || ctx_id == 0 || g_na_ctx[dev] != ctx_id) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return set_error(PDG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_na_ptr[dev] = static_cast<double *>(p);
    g_na_ctx[dev] = ctx_id;
  }
  *out = g_na_ptr[dev];
  return PDG_OK;
}

// The device that owns p (device or managed memory), else -1.
int owning_device(const void *p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) return -1;
  return attr.device;
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
  int dev = 0;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_error(PDG_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  // every pointer must live on the current device, where the kernel runs
  const int dr = owning_device(result);
  if (dr < 0 || (n > 0 && (owning_device(a) < 0 || owning_device(b) < 0)))
    return set_error(PDG_EINVAL, "pdg_dot_noalloc: a, b and result must be device pointers");
  if (dr != dev || (n > 0 && (owning_device(a) != dev || owning_device(b) != dev)))
    return set_error(PDG_EINVAL,
                     "pdg_dot_noalloc: a, b and result must be on the current device");
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
