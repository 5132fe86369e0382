// Device code of the Biggs-Andrews acceleration factor (see accel.cu).
#pragma once

#include "common.cuh"

namespace cdx {

constexpr int kDotThreads = 256;
constexpr int kDotPerThread = 32;
constexpr int kDotElemsPerBlock = kDotThreads * kDotPerThread;  // 8192

// Blocks (= partial pairs) for n elements.
int accel_blocks(long long n);

// One block of the two inner products: elements [b*8192, (b+1)*8192) of
// g_new.g_old and g_old.g_old (float products, double sums), the block
// partials to partials[b] / partials[nblk + b], and the last block to finish
// reduces all partials in index order and writes the results.  *counter
// must be 0 at launch; the last block sets it back to 0.
__device__ __forceinline__ void accel_factor_block(const float* __restrict__ g_new,
                                                   const float* __restrict__ g_old, long long n,
                                                   double* partials, unsigned* counter, float eps,
                                                   double* out, float* lam) {
  __shared__ double red[2][kDotThreads / 32];
  __shared__ bool last;
  const int nblk = gridDim.x;
  const long long b0 = (long long)blockIdx.x * kDotElemsPerBlock;
  double s1 = 0.0, s2 = 0.0;
#pragma unroll 4
  for (int i = 0; i < kDotPerThread; ++i) {
    const long long e = b0 + (long long)i * kDotThreads + threadIdx.x;
    if (e < n) {
      const float a = g_new[e], b = g_old[e];
      s1 += (double)__fmul_rn(a, b);
      s2 += (double)__fmul_rn(b, b);
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if (lane == 0) {
    red[0][warp] = s1;
    red[1][warp] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kDotThreads / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    partials[blockIdx.x] = a;
    partials[nblk + blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(counter, 1u) == (unsigned)nblk - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblk; i += kDotThreads) {
    a += __ldcg(partials + i);
    b += __ldcg(partials + nblk + i);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[0][warp] = a;
    red[1][warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double num = 0.0, den = 0.0;
    for (int w = 0; w < kDotThreads / 32; ++w) {
      num += red[0][w];
      den += red[1][w];
    }
    const double l = num / (den + (double)eps);
    double c = (1.0 < l) ? 1.0 : l;
    c = (c < 0.0) ? 0.0 : c;
    if (out) {
      out[0] = num;
      out[1] = den;
      out[2] = l;
    }
    if (lam) *lam = (float)c;
    *counter = 0u;
  }
}

int launch_accel_factor(const float* g_new, const float* g_old, long long n, double* partials,
                        unsigned* counter, float eps, double* out, float* lam, cudaStream_t st);

}  // namespace cdx
