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

// Shared-memory layout (float2 units): [twiddles][tile][Y rows][G rows];
// runners that read the twiddles from global memory have no twiddle copy.
template <class Run>
__host__ __device__ __forceinline__ int upd_tile_offset(int nx) {
  return Run::kGlobalTw ? 0 : x_tile_offset(nx);
}
template <class Run>
__host__ __device__ __forceinline__ int upd_rows_offset(int nx, int P) {
  return upd_tile_offset<Run>(nx) + (Run::kTileF2 > 0 ? Run::kTileF2 : x_tile_size(nx, P));
}

// Last inverse stage: estimate update (currEstimate_kernel +
// currPrevDiff_kernel, RLgpuImpl.cu:462-470, 501-508) from the prediction Y,
// with the Biggs-Andrews dot products of innerProduct_kernel
// (RLgpuImpl.cu:571-633: float products, double sums).
struct UpdateStore {
  static constexpr bool kSmem = false;
  static constexpr bool kGroup = false;
  const float* Ys;  // shared copies of rows y0 .. y0+2P-1 of Y and G
  const float* Gs;
  float* Xout;      // global
  float* G;         // global
  int dots;
  long long zoff;
  int y0, ny, nx;
  float* acc;  // float-float accumulators: s1 (hi, lo), s2 (hi, lo)
  __device__ __forceinline__ void one(int rloc, int e, float cc) const {
    const int l = rloc * nx + e;
    const float yv = Ys[l];
    float xn = __fmul_rn(cc, yv);
    xn = xn > 0.f ? xn : 0.f;
    const float gn = __fsub_rn(xn, yv);
    if (dots) {
      const float go = Gs[l];
      acc_add(acc[0], acc[1], __fmul_rn(gn, go));
      acc_add(acc[2], acc[3], __fmul_rn(go, go));
    }
    const long long o = zoff + (long long)(y0 + rloc) * nx + e;
    Xout[o] = xn;
    G[o] = gn;
  }
  __device__ __forceinline__ void st(int v, int e, float2 c) const {
    const int ya = y0 + 2 * v;
    if (ya < ny) one(2 * v, e, c.x);
    if (ya + 1 < ny) one(2 * v + 1, e, c.y);
  }
};

template <class Run>
__global__ void __launch_bounds__(Run::kThreads, Run::template min_blocks<5>())
k_x_inv_update(Geom g, FftDev fx, const float2* __restrict__ S, const float* Y, float* Xout,
               float* G, int dots, double* partials, unsigned* counter, float* lam_next,
               float eps, int Pa) {
  const int P = tile_vectors<Run>(Pa);
  extern __shared__ __align__(16) float2 smem[];
  __shared__ double red[64];
  __shared__ bool last;
  const int nx = g.nx;
  const float2* stw = Run::kGlobalTw ? fx.tw : smem;
  const auto io = Run::row_tile(smem + upd_tile_offset<Run>(nx), nx);
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  // Copy (cp.async) the half spectra into the tile region, where the first
  // stage rebuilds the packed spectra, and the rows of Y and (when the dots
  // are needed) G, which the epilogue reads.
  float4* stg = reinterpret_cast<float4*>(io.sm);
  float* Ys = reinterpret_cast<float*>(smem + upd_rows_offset<Run>(nx, P));
  float* Gs = Ys + 2 * P * nx;
  const int nr = min(2 * P, g.ny - y0);
  const long long roff = ((long long)z * g.ny + y0) * nx;
  if (!Run::kGlobalTw) load_twiddles(fx, smem);
  grid_dep_wait();
  grid_dep_launch();
  prefetch_packed_spectra<Run::kV>(g, S, stg, P, z, y0);
  prefetch_floats(Ys, Y + roff, nr * nx);
  if (dots) prefetch_floats(Gs, G + roff, nr * nx);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  const PackedSpecLoad ld{stg, g.nxh, nx, (nr + 1) / 2};
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const UpdateStore us{Ys, Gs, Xout, G, dots, (long long)z * g.ny * nx, y0, g.ny, nx, acc};
  Run::template run<true>(fx, P, 1.f, false, stw, io, ld, us);
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
static int x_update_go(const Geom& g, const FftDev& f, const float2* S, const float* Y,
                       float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                       int P, int T, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  const int nblk = grid.x * grid.y;
  if (dots && nblk > w.max_blocks) {
    set_error("launch_x_inv_update", "partials buffer too small");
    return cudaErrorInvalidValue;
  }
  size_t smem = sizeof(float2) * ((size_t)upd_rows_offset<Run>(g.nx, P) + 2 * (size_t)P * g.nx);
  if (int rc = smem_optin(k_x_inv_update<Run>, smem)) return rc;
  CDX_CHECK(launch_pdl(k_x_inv_update<Run>, grid, dim3(T), smem, st, g, f, S, Y, Xout, G, dots, w.partials, w.counter,
                                             lam_next, eps, P));
  CDX_LAUNCH_CHECK("k_x_inv_update");
  return 0;
}

int launch_x_inv_update(const Geom& g, const FftLen& fx, const float2* S, const float* Y,
                        float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                        cudaStream_t st) {
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP)                                                                    \
  case L:                                                                                  \
    return x_update_go<StaticRunner<SP##L, PP, false, true>>(g, fx.sdev, S, Y, Xout, G, dots, \
                                                              w, lam_next, eps, PP,          \
                                                              splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  const int P = x_pairs(g.nx);
  return x_update_go<GenericRunner>(g, fx.dev, S, Y, Xout, G, dots, w, lam_next, eps, P,
                                    threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
