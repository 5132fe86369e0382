// Biggs-Andrews acceleration factor on device arrays.
//
// The reference computes it in calcAccelFactor (src/RLgpuImpl.cu:510-569):
// two inner products of the last two RL changes, G_new.G_old and
// G_old.G_old, with products rounded to float and sums accumulated in double
// (innerProduct_kernel, :571-633), per-block partials copied to the host and
// summed there, then lambda = num / (den + eps); the caller clamps lambda to
// [0, 1] (src/RL-Biggs-Andrews.cpp:298).  Here the partials are reduced on
// the device by the last block to finish (fixed order, deterministic) and
// the results stay in device memory: out[0] = num, out[1] = den,
// out[2] = unclamped lambda (double), lam = clamped lambda as float.
#include "accel.cuh"

namespace cdx {

int accel_blocks(long long n) { return (int)((n + kDotElemsPerBlock - 1) / kDotElemsPerBlock); }

__global__ void __launch_bounds__(kDotThreads)
k_accel_factor(const float* __restrict__ g_new, const float* __restrict__ g_old, long long n,
               double* partials, unsigned* counter, float eps, double* out, float* lam) {
  accel_factor_block(g_new, g_old, n, partials, counter, eps, out, lam);
}

int launch_accel_factor(const float* g_new, const float* g_old, long long n, double* partials,
                        unsigned* counter, float eps, double* out, float* lam, cudaStream_t st) {
  const int nblk = accel_blocks(n);
  k_accel_factor<<<nblk, kDotThreads, 0, st>>>(g_new, g_old, n, partials, counter, eps, out, lam);
  CDX_LAUNCH_CHECK("k_accel_factor");
  return 0;
}

}  // namespace cdx
