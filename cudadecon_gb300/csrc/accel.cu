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
#include "kernels.h"

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

// ---------------------------------------------------------------- convergence norm
// The reference computes no convergence measure; this one is for tracing
// (cdx_change_trace) and runs only then, after an iteration's update:
// ||X_{k+1} - X_k||_2 / ||X_k||_2 with the squares summed in FP64, per block
// in a fixed order, then the blocks' sums in a fixed order by one block.
constexpr int kChangeThreads = 256;

__device__ __forceinline__ void block_sum2_d(double& a, double& b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[2 * warp] = a;
    red[2 * warp + 1] = b;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? red[2 * lane] : 0.0;
    b = lane < nw ? red[2 * lane + 1] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
  }
}

__global__ void __launch_bounds__(kChangeThreads)
k_change_partials(const float* __restrict__ x_new, const float* __restrict__ x_old, long long n,
                  double* part) {
  __shared__ double red[2 * (kChangeThreads / 32)];
  double d2 = 0.0, o2 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double o = x_old[i];
    const double d = (double)x_new[i] - o;
    d2 = fma(d, d, d2);
    o2 = fma(o, o, o2);
  }
  block_sum2_d(d2, o2, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = d2;
    part[2 * blockIdx.x + 1] = o2;
  }
}

__global__ void __launch_bounds__(kChangeThreads)
k_change_final(const double* __restrict__ part, int nblk, double* out) {
  __shared__ double red[2 * (kChangeThreads / 32)];
  double d2 = 0.0, o2 = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    d2 += part[2 * i];
    o2 += part[2 * i + 1];
  }
  block_sum2_d(d2, o2, red);
  if (threadIdx.x == 0) *out = o2 > 0.0 ? sqrt(d2 / o2) : 0.0;
}

int launch_change_norm(const float* x_new, const float* x_old, long long n, double* part,
                       double* out, cudaStream_t st) {
  k_change_partials<<<kChangeBlocks, kChangeThreads, 0, st>>>(x_new, x_old, n, part);
  CDX_LAUNCH_CHECK("k_change_partials");
  k_change_final<<<1, kChangeThreads, 0, st>>>(part, kChangeBlocks, out);
  CDX_LAUNCH_CHECK("k_change_final");
  return 0;
}

}  // namespace cdx
