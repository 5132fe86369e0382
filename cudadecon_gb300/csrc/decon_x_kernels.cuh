// The x-pass kernels of the plain form as templates over the transform
// runner (compile-time plan or generic engine) with their launch helpers:
// forward x pass with the prediction prologue, inverse x pass with the RL
// ratio and the forward transform of the ratio, inverse x pass with the
// estimate update and the dot products.  decon_x_fwd.cu, decon_x_ratio.cu and
// decon_x_update.cu dispatch the registered lengths; the generated units
// decon_x_gen_*.cu instantiate the generated plans.
#pragma once

#include <algorithm>

#include "decon_common.cuh"

namespace cdx {

// ---------------------------------------------------------------- x forward
template <class Run>
__global__ void __launch_bounds__(Run::kThreads, Run::template min_blocks<6>())
k_x_fwd(Geom g, FftDev fx, const float* __restrict__ X, float* Xm1, const float* __restrict__ lamp,
        int predict, float2* __restrict__ S, int Pa) {
  const int P = tile_vectors<Run>(Pa);
  extern __shared__ __align__(16) float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const auto io = Run::row_tile(smem + x_tile_offset(nx), nx);
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  // The rows of X (and X_{k-1}) are copied into the tile region with
  // cp.async; the first stage reads them from there before it writes the
  // tile (the two alias).
  float* Xs = reinterpret_cast<float*>(io.sm);
  float* Xm1s = Xs + 2 * P * nx;
  const int nr = min(2 * P, g.ny - y0);
  const long long roff = ((long long)z * g.ny + y0) * nx;
  load_twiddles(fx, stw);
  grid_dep_wait();
  grid_dep_launch();
  prefetch_floats(Xs, X + roff, nr * nx, true);
  if (predict) prefetch_floats(Xm1s, Xm1 + roff, nr * nx, true);
  cp_async_commit();
  const float lam = predict ? __ldg(lamp) : 0.f;
  cp_async_wait_all();
  __syncthreads();
  // prediction of updatePrediction_kernel (RLgpuImpl.cu:658-666), applied
  // by the first stage as it reads the rows and written over the block's
  // rows of X_{k-1}
  const RowPairSmemLoad ld{Xs, Xm1s, predict ? Xm1 + roff : nullptr, lam, predict, nr, nx};
  Run::template run<false>(fx, P, 1.f, false, stw, io, ld, io);
  store_half_spectra<Run::kV>(g, io, P, z, y0, S);
}

template <class Run>
static int x_fwd_go(const Geom& g, const FftDev& f, const float* X, float* Xm1,
                    const float* lam, int predict, float2* S, int P, int T, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  const int region = std::max(x_tile_size(g.nx, P), 2 * P * g.nx);
  size_t smem = sizeof(float2) * ((size_t)x_tile_offset(g.nx) + (size_t)region);
  if (int rc = smem_optin(k_x_fwd<Run>, smem)) return rc;
  CDX_CHECK(launch_pdl(k_x_fwd<Run>, grid, dim3(T), smem, st, g, f, X, Xm1, lam, predict, S, P));
  CDX_LAUNCH_CHECK("k_x_fwd");
  return 0;
}

// ---------------------------------------------------------------- x inverse
template <class Run>
__global__ void __launch_bounds__(Run::kThreads, Run::template min_blocks<6>())
k_x_inv_ratio_fwd(Geom g, FftDev fx, float2* __restrict__ S, const float* __restrict__ raw,
                  float eps, int Pa) {
  const int P = tile_vectors<Run>(Pa);
  extern __shared__ __align__(16) float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const auto io = Run::row_tile(smem + x_tile_offset(nx), nx);
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  // Half spectra (staged in the tile region) and raw rows are copied with
  // cp.async; the first stage rebuilds the packed spectra from the stage.
  float4* stg = reinterpret_cast<float4*>(io.sm);
  float* raws = reinterpret_cast<float*>(smem + x_rows_offset(nx, P));
  const int nr = min(2 * P, g.ny - y0);
  load_twiddles(fx, stw);
  grid_dep_wait();
  grid_dep_launch();
  prefetch_packed_spectra<Run::kV>(g, S, stg, P, z, y0);
  prefetch_floats(raws, raw + ((long long)z * g.ny + y0) * nx, nr * nx, true);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  const RatioStore<typename Run::Tile> rs{io, raws, y0, g.ny, nx, eps};
  if constexpr (Run::kStatic) {
    const PackedSpecLoadS<Run::SPlanT::kL> ld{stg, (nr + 1) / 2};
    Run::template run<true>(fx, P, 1.f, false, stw, io, ld, rs);
  } else {
    const PackedSpecLoad ld{stg, g.nxh, nx, (nr + 1) / 2};
    Run::template run<true>(fx, P, 1.f, false, stw, io, ld, rs);
  }
  Run::template run<false>(fx, P, 1.f, false, stw, io, io, io);
  store_half_spectra<Run::kV>(g, io, P, z, y0, S);
}

template <class Run>
static int x_ratio_go(const Geom& g, const FftDev& f, float2* S, const float* raw, float eps,
                      int P, int T, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  size_t smem = sizeof(float2) * ((size_t)x_rows_offset(g.nx, P) + (size_t)P * g.nx);
  if (int rc = smem_optin(k_x_inv_ratio_fwd<Run>, smem)) return rc;
  CDX_CHECK(launch_pdl(k_x_inv_ratio_fwd<Run>, grid, dim3(T), smem, st, g, f, S, raw, eps, P));
  CDX_LAUNCH_CHECK("k_x_inv_ratio_fwd");
  return 0;
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
// (RLgpuImpl.cu:571-633: float products summed in double there; here in
// float-float, about 48 significant bits).
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
    // X is read next by the x forward pass (kept in L2); G only by the next
    // iteration's update pass (evict-first)
    Xout[o] = xn;
    __stcs(G + o, gn);
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
               float* G, int dots, float4* partials, int Pa) {
  const int P = tile_vectors<Run>(Pa);
  extern __shared__ __align__(16) float2 smem[];
  __shared__ float4 red[32];
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
  // the last read of this iteration's spectrum: evict-first
  prefetch_packed_spectra<Run::kV>(g, S, stg, P, z, y0, true);
  prefetch_floats(Ys, Y + roff, nr * nx, true);
  if (dots) prefetch_floats(Gs, G + roff, nr * nx, true);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const UpdateStore us{Ys, Gs, Xout, G, dots, (long long)z * g.ny * nx, y0, g.ny, nx, acc};
  if constexpr (Run::kStatic) {
    const PackedSpecLoadS<Run::SPlanT::kL> ld{stg, (nr + 1) / 2};
    Run::template run<true>(fx, P, 1.f, false, stw, io, ld, us);
  } else {
    const PackedSpecLoad ld{stg, g.nxh, nx, (nr + 1) / 2};
    Run::template run<true>(fx, P, 1.f, false, stw, io, ld, us);
  }
  if (!dots) return;
  const float4 sum = block_sum2_ff(acc[0], acc[1], acc[2], acc[3], red);
  if (threadIdx.x == 0) partials[blockIdx.y * gridDim.x + blockIdx.x] = sum;
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
  float4* part = reinterpret_cast<float4*>(w.partials);
  CDX_CHECK(launch_pdl(k_x_inv_update<Run>, grid, dim3(T), smem, st, g, f, S, Y, Xout, G, dots,
                       part, P));
  CDX_LAUNCH_CHECK("k_x_inv_update");
  if (dots) return launch_lambda(part, nblk, lam_next, eps, st);
  return 0;
}

}  // namespace cdx
