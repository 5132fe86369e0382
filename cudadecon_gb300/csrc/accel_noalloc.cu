// Allocation-free variant of the Biggs-Andrews acceleration factor.
//
// cdx_accel_factor_device keeps its per-block partial sums in scratch that
// the library allocates with cudaMalloc the first time it is needed.  Some
// callers cannot let a library allocate device memory while they run:
//   * acquisition pipelines that overlap camera transfers and deconvolution
//     on several streams, because cudaMalloc and cudaFree synchronise the
//     whole device and would stall every stream at an unpredictable moment;
//   * processes that reserve the GPU's memory up front (ring buffers for a
//     timelapse, pools of their own), where a late allocation can fail with
//     out-of-memory in the middle of an acquisition.
// For them, cdx_accel_factor_device_noalloc computes the same result with
// its scratch in a fixed array in device memory that exists as long as the
// library is loaded, so a call allocates nothing.
//
// The array holds the partials of at most kNoAllocMaxBlocks blocks of
// kDotElemsPerBlock elements (33,554,432 elements per array) plus the
// last-block counter: 64 KB + 8 bytes on every GPU that loads the library.
// Larger arrays are rejected.  All calls share the array, so calls that may
// overlap on the GPU (different streams, or other threads) race with each
// other and must be serialised by the caller.
#include <mutex>

#include "../../include/cudadecon.h"
#include "accel.cuh"

namespace cdx {

constexpr int kNoAllocMaxBlocks = 4096;
constexpr long long kNoAllocMaxElems = (long long)kNoAllocMaxBlocks * kDotElemsPerBlock;

// partials in [0, 2 * kNoAllocMaxBlocks), the last-block counter in the
// final element (used as an unsigned).
static __device__ __align__(256) double g_accel_scratch[2 * kNoAllocMaxBlocks + 1];

// Device address of g_accel_scratch per device ordinal.  In host code the
// name g_accel_scratch is only a host-side stand-in, so the address is asked
// from the runtime once per device, with that device current.
constexpr int kMaxDevices = 64;
static double* g_scratch_addr[kMaxDevices] = {nullptr};
static std::mutex g_scratch_mu;

static int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_cuda_error("cdx_accel_factor_device_noalloc: cudaGetDevice", e);
    return e;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("cdx_accel_factor_device_noalloc", "device ordinal out of range");
    return cudaErrorInvalidDevice;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_accel_scratch);
    if (e != cudaSuccess || !p) {
      set_cuda_error("cdx_accel_factor_device_noalloc: cudaGetSymbolAddress", e);
      return e != cudaSuccess ? e : cudaErrorInvalidSymbol;
    }
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return 0;
}

__global__ void __launch_bounds__(kDotThreads)
k_accel_factor_noalloc(const float* __restrict__ g_new, const float* __restrict__ g_old,
                       long long n, double* scratch, float eps, double* out, float* lam) {
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + 2 * kNoAllocMaxBlocks);
  accel_factor_block(g_new, g_old, n, scratch, counter, eps, out, lam);
}

}  // namespace cdx

using namespace cdx;

extern "C" int cdx_accel_factor_device_noalloc(const float* g_new, const float* g_old,
                                               long long n, double* out, float* lam,
                                               void* stream) {
  if (!g_new || !g_old || n < 1) {
    set_error("cdx_accel_factor_device_noalloc", "null pointer or empty array");
    return 0;
  }
  if (n > kNoAllocMaxElems) {
    set_error("cdx_accel_factor_device_noalloc",
              "array longer than the 33554432 elements the fixed scratch supports; "
              "use cdx_accel_factor_device");
    return 0;
  }
  double* scratch = nullptr;
  if (scratch_for_current_device(&scratch)) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  // the counter must start at zero (a failed earlier call may have left it set)
  cudaError_t e = cudaMemsetAsync(scratch + 2 * kNoAllocMaxBlocks, 0, sizeof(double), st);
  if (e != cudaSuccess) {
    set_cuda_error("cdx_accel_factor_device_noalloc: cudaMemsetAsync", e);
    return 0;
  }
  const float eps = 1.1920928955078125e-07f;  // FLT_EPSILON, as the reference's eps
  k_accel_factor_noalloc<<<accel_blocks(n), kDotThreads, 0, st>>>(g_new, g_old, n, scratch, eps,
                                                                   out, lam);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_cuda_error("cdx_accel_factor_device_noalloc: launch", e);
    return 0;
  }
  return 1;
}
