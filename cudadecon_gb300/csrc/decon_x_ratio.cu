// Inverse x pass of the first convolution: C2R, RL ratio, and R2C of the
// ratio for the second convolution.
#include "decon_common.cuh"

namespace cdx {

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
  const PackedSpecLoad ld{stg, g.nxh, nx, (nr + 1) / 2};
  const RatioStore<typename Run::Tile> rs{io, raws, y0, g.ny, nx, eps};
  Run::template run<true>(fx, P, 1.f, false, stw, io, ld, rs);
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

int launch_x_inv_ratio_fwd(const Geom& g, const FftLen& fx, float2* S, const float* raw,
                           float eps, cudaStream_t st) {
  if (fx.has_tc && dft_form() == 1)
    return launch_xtc_ratio(g, fx.tc, S, raw, eps, fx.tc.d_err, st);
  if (fx.has_xr) switch (g.nx) {
#define CDX_XR_CASE(L, PP, ...)                                                            \
  case L:                                                                                  \
    return x_ratio_go<StaticRunner<SPR##L, PP, false>>(g, fx.xrdev, S, raw, eps, PP,       \
                                                       splan_threads<SPR##L, PP>(), st);
      CDX_XR_PLANS(CDX_XR_CASE)
#undef CDX_XR_CASE
      default:
        break;
    }
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP) \
  case L:               \
    return x_ratio_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, S, raw, eps, PP, splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  const int P = x_pairs(g.nx);
  return x_ratio_go<GenericRunner>(g, fx.dev, S, raw, eps, P, threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
