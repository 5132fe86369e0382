// Inverse x pass of the second convolution: C2R, estimate update and the
// acceleration-factor dot products (last block finishes lambda).
#include "decon_common.cuh"

namespace cdx {

// Block-wide sum of two doubles; result valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < nw ? red[lane] : 0.0;
    b = lane < nw ? red[32 + lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
  }
}

template <class Run>
__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_inv_update(Geom g, FftDev fx, const float2* __restrict__ S, const float* __restrict__ X,
               const float* Xm1, const float* __restrict__ lamp, int predict, float* Xout,
               float* __restrict__ G, int dots, double* partials, unsigned* counter,
               float* lam_next, float eps, int P) {
  extern __shared__ float2 smem[];
  __shared__ double red[64];
  __shared__ bool last;
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  // prefetch rows of X, X_{k-1} (when predicting) and G (when the dots are
  // needed) into shared memory; they are read by the epilogue
  float* Xs = reinterpret_cast<float*>(smem + x_rows_offset(nx, P));
  float* Xm1s = Xs + 2 * P * nx;
  float* Gs = Xm1s + 2 * P * nx;
  const int nr = min(2 * P, g.ny - y0);
  const long long roff = ((long long)z * g.ny + y0) * nx;
  prefetch_floats(Xs, X + roff, nr * nx);
  if (predict) prefetch_floats(Xm1s, Xm1 + roff, nr * nx);
  if (dots) prefetch_floats(Gs, G + roff, nr * nx);
  cp_async_commit();
  load_twiddles(fx, stw);
  load_packed_spectra(g, S, io, P, z, y0);
  cp_async_wait_all();
  __syncthreads();
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const UpdateStore us{Xs, Xm1s, Gs, Xout, G, predict ? __ldg(lamp) : 0.f, predict, dots,
                       (long long)z * g.ny * nx, y0, g.ny, nx, acc};
  Run::template run<true>(fx, P, 1.f, false, stw, io, io, us);
  if (!dots) return;
  double s1 = (double)acc[0] + (double)acc[1], s2 = (double)acc[2] + (double)acc[3];
  block_sum2(s1, s2, red);
  const int nblk = gridDim.x * gridDim.y;
  const int bid = blockIdx.y * gridDim.x + blockIdx.x;
  if (threadIdx.x == 0) {
    partials[bid] = s1;
    partials[nblk + bid] = s2;
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == (unsigned)nblk - 1);
  }
  __syncthreads();
  if (!last) return;
  // Last block: reduce all partials in a fixed order (deterministic).
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += __ldcg(partials + i);
    b += __ldcg(partials + nblk + i);
  }
  block_sum2(a, b, red);
  if (threadIdx.x == 0) {
    // calcAccelFactor (RLgpuImpl.cu:565) then the clamp of RL-Biggs-Andrews.cpp:298
    double l = a / (b + (double)eps);
    l = (1.0 < l) ? 1.0 : l;
    l = (l < 0.0) ? 0.0 : l;
    *lam_next = (float)l;
    *counter = 0u;
  }
}

template <class Run>
static int x_update_go(const Geom& g, const FftDev& f, const float2* S, const float* X,
                       const float* Xm1, const float* lam, int predict, float* Xout, float* G,
                       int dots, RLWork& w, float* lam_next, float eps, int P, int T,
                       cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  const int nblk = grid.x * grid.y;
  if (dots && nblk > w.max_blocks) {
    set_error("launch_x_inv_update", "partials buffer too small");
    return cudaErrorInvalidValue;
  }
  size_t smem = sizeof(float2) * ((size_t)x_rows_offset(g.nx, P) + 3 * (size_t)P * g.nx);
  if (int rc = smem_optin(k_x_inv_update<Run>, smem)) return rc;
  k_x_inv_update<Run><<<grid, T, smem, st>>>(g, f, S, X, Xm1, lam, predict, Xout, G, dots,
                                             w.partials, w.counter, lam_next, eps, P);
  CDX_LAUNCH_CHECK("k_x_inv_update");
  return 0;
}

int launch_x_inv_update(const Geom& g, const FftLen& fx, const float2* S, const float* X,
                        const float* Xm1, const float* lam, int predict, float* Xout, float* G,
                        int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st) {
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP)                                                                         \
  case L:                                                                                       \
    return x_update_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, S, X, Xm1, lam, predict, Xout, \
                                                        G, dots, w, lam_next, eps, PP,             \
                                                        splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  const int P = x_pairs(g.nx);
  return x_update_go<GenericRunner>(g, fx.dev, S, X, Xm1, lam, predict, Xout, G, dots, w, lam_next,
                                    eps, P, threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
