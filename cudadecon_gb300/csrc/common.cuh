// Shared helpers for the cudadecon_gb300 CUDA sources: complex arithmetic on
// float2, status handling without exit()/throw across the C ABI, and the
// small integer utilities the launchers use.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace cdx {

// ---------------------------------------------------------------- status
// Every internal routine returns a cudaError_t-compatible int; the C ABI
// converts it to the reference's 1 (ok) / 0 (failure) convention.  The last
// failure message is kept for cdx_last_error().
void set_error(const char* where, const char* what);
void set_cuda_error(const char* where, cudaError_t err);

#define CDX_CHECK(call)                                                     \
  do {                                                                      \
    cudaError_t _e = (call);                                                \
    if (_e != cudaSuccess) {                                                \
      ::cdx::set_cuda_error(#call, _e);                                     \
      return _e;                                                            \
    }                                                                       \
  } while (0)

#define CDX_LAUNCH_CHECK(name)                                              \
  do {                                                                      \
    cudaError_t _e = cudaGetLastError();                                    \
    if (_e != cudaSuccess) {                                                \
      ::cdx::set_cuda_error(name, _e);                                      \
      return _e;                                                            \
    }                                                                       \
  } while (0)

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------- complex
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a * b
// On the device the roundings are written out (one product rounded, the
// other fused), so that a product computes the same value whether its
// operands come from memory or from registers of a fused neighbouring stage.
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)),
                     __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
#else
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
#endif
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulconj(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return make_float2(__fmaf_rn(a.x, b.x, __fmul_rn(a.y, b.y)),
                     __fmaf_rn(a.y, b.x, -__fmul_rn(a.x, b.y)));
#else
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
#endif
}
__host__ __device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i and +i
__host__ __device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }
__host__ __device__ __forceinline__ float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }

}  // namespace cdx
