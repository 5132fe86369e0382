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

// Device address of g_accel_scratch, looked up once per device and context.
// In host code the name g_accel_scratch is only a host-side stand-in, so the
// address is asked from the runtime (cudaGetSymbolAddress) with the device
// current.  The array lives in the context's copy of the module: after
// cudaDeviceReset (cuda_reset) or under another context of the same device
// it may sit at another address, so each cached address is tagged with the
// id of the context it was looked up in and looked up again when the
// current context's id differs.  The context id comes from the driver
// (cuCtxGetCurrent, cuCtxGetId), reached through the runtime's entry-point
// query so that the library does not link libcuda.
constexpr int kMaxDevices = 64;
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  double* addr = nullptr;
};
static ScratchAddr g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

typedef int (*PfnCtxGetCurrent)(void** ctx);
typedef int (*PfnCtxGetId)(void* ctx, unsigned long long* id);
static PfnCtxGetCurrent g_ctx_get_current = nullptr;
static PfnCtxGetId g_ctx_get_id = nullptr;
static bool g_ctx_fns_queried = false;

// Id of the current context (0 when there is none or the driver cannot say).
static unsigned long long current_context_id() {
  if (!g_ctx_fns_queried) {
    g_ctx_fns_queried = true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) ==
            cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) ==
            cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
      g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(f2);
    }
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != 0 || !ctx) return 0;
  if (g_ctx_get_id(ctx, &id) != 0) return 0;
  return id;
}

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
  const unsigned long long id = current_context_id();
  ScratchAddr& c = g_scratch_addr[dev];
  // id 0: no context yet (the lookup below creates the primary context) or
  // no driver answer; then the address is looked up on every call
  if (!c.addr || id == 0 || c.ctx_id != id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_accel_scratch);
    if (e != cudaSuccess || !p) {
      set_cuda_error("cdx_accel_factor_device_noalloc: cudaGetSymbolAddress", e);
      c = ScratchAddr{};
      return e != cudaSuccess ? e : cudaErrorInvalidSymbol;
    }
    c.addr = static_cast<double*>(p);
    c.ctx_id = id ? id : current_context_id();
  }
  *out = c.addr;
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
