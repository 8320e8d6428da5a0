// Conservation sums for callers that cannot allocate device memory.
//
// fvgpu_conservation() keeps its block partial sums in a buffer the context
// allocates.  Some host codes cannot make that allocation: a solver that
// reserves all the device memory it will ever use at start-up and forbids any
// allocation inside its time loop (allocation can synchronise the device and
// fragments a pool the host manages itself), or a process whose device
// memory is capped by its job scheduler and already fully committed.  For
// them, fvgpu_conservation_noalloc() computes the same sums from device
// arrays they own, with its scratch in a fixed file-scope device array:
//
//   scratch   g_noalloc_partial, kNoallocBlocks x (kNoallocMaxVars) doubles
//             = 1024 x 6 x 8 B = 48 KiB, held on every device that loads the
//             library until the process exits;
//   limits    1 <= neq <= 5 (so neq + 1 <= 6 sums) and 1 <= ncells < 2^31;
//             anything else is rejected with FVGPU_ERR_ARG before any launch.
//
// The array is shared by every call on a device and keeps the last call's
// contents.  Each call rewrites every slot it later reads (each of the 1024
// blocks stores its partial sum for every variable, empty blocks store 0), so
// nothing has to be cleared between calls.  Calls whose kernels overlap on
// the GPU (different streams, or different host threads without ordering)
// race on the array; callers must order them.
//
// Host code cannot use the array's name as a device address (it is a host-side
// stand-in), so the first call on each device looks up the real address with
// cudaGetSymbolAddress while that device is current, checks the result and
// caches it together with the device's current context.  A call that finds a
// different context (the old one was destroyed, e.g. by cudaDeviceReset, and
// the array now lives in the new one) looks the address up again.  Those calls
// therefore perform a runtime query: make them before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "fvgpu.h"

namespace {

constexpr int kNoallocBlocks = 1024;
constexpr int kNoallocThreads = 256;
constexpr int kNoallocMaxVars = 6;  // neq <= 5 conserved variables + the volume
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partial[kNoallocBlocks * kNoallocMaxVars];

double *g_partial_addr[kMaxDevices] = {nullptr};
void *g_partial_ctx[kMaxDevices] = {nullptr};  // the context the cached address belongs to
std::mutex g_setup_mutex;

// The calling thread's current driver context (cuCtxGetCurrent, fetched from
// the driver through the runtime so the library needs no link to libcuda).
typedef int (*CtxGetCurrentFn)(void **);
void *current_context() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  void *ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

// Same partition and reduction order as fvgpu_conservation: cells split into
// kNoallocBlocks contiguous ranges, fixed in-block tree, fixed final tree.
__global__ void k_noalloc_partial(int neq, int64_t n, const double *__restrict__ S, const double *__restrict__ vol,
                                  double *__restrict__ partial) {
  __shared__ double red[kNoallocThreads];
  const int64_t per = (n + kNoallocBlocks - 1) / kNoallocBlocks;
  const int64_t lo = int64_t(blockIdx.x) * per;
  const int64_t hi = lo + per < n ? lo + per : n;
  for (int v = 0; v <= neq; ++v) {
    double acc = 0.0;
    for (int64_t c = lo + threadIdx.x; c < hi; c += kNoallocThreads) acc += v < neq ? S[v * n + c] * vol[c] : vol[c];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kNoallocThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[v * kNoallocBlocks + blockIdx.x] = red[0];
    __syncthreads();
  }
}

__global__ void k_noalloc_final(int neq, const double *__restrict__ partial, double *__restrict__ sums) {
  __shared__ double red[kNoallocThreads];
  for (int v = 0; v <= neq; ++v) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < kNoallocBlocks; b += kNoallocThreads) acc += partial[v * kNoallocBlocks + b];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kNoallocThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) sums[v] = red[0];
    __syncthreads();
  }
}

// Device address of the scratch array on the current device (looked up once).
int scratch_on_current_device(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FVGPU_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  void *ctx = current_context();
  if (!g_partial_addr[dev] || ctx == nullptr || ctx != g_partial_ctx[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
    if (e != cudaSuccess || p == nullptr) return FVGPU_ERR_CUDA;
    g_partial_addr[dev] = static_cast<double *>(p);
    g_partial_ctx[dev] = current_context();  // the runtime made the primary context current if none was
  }
  *out = g_partial_addr[dev];
  return FVGPU_OK;
}

}  // namespace

extern "C" int fvgpu_conservation_noalloc(const double *S, const double *vol, int64_t ncells, int neq,
                                          double *sums, void *stream) {
  if (!S || !vol || !sums) return FVGPU_ERR_ARG;
  if (neq < 1 || neq + 1 > kNoallocMaxVars) return FVGPU_ERR_ARG;          // scratch holds 6 rows
  if (ncells < 1 || ncells >= (int64_t(1) << 31)) return FVGPU_ERR_ARG;
  double *partial = nullptr;
  const int rc = scratch_on_current_device(&partial);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_noalloc_partial<<<kNoallocBlocks, kNoallocThreads, 0, st>>>(neq, ncells, S, vol, partial);
  if (cudaGetLastError() != cudaSuccess) return FVGPU_ERR_CUDA;
  k_noalloc_final<<<1, kNoallocThreads, 0, st>>>(neq, partial, sums);
  if (cudaGetLastError() != cudaSuccess) return FVGPU_ERR_CUDA;
  return FVGPU_OK;
}
