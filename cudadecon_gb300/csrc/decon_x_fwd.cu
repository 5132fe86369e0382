// Forward x pass of the RL iteration (prediction prologue + R2C along x) and
// the plain inverse x pass used by the convolution test hook.
#include <algorithm>

#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int launch_x_fwd(const Geom& g, const FftLen& fx, const float* X, float* Xm1,
                 const float* lam, int predict, float2* S, cudaStream_t st) {
  if (fx.has_tc && dft_form() == 1)
    return launch_xtc_fwd(g, fx.tc, X, Xm1, lam, predict, S, fx.tc.d_err, st);
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP)                                                                      \
  case L:                                                                                    \
    return x_fwd_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, X, Xm1, lam, predict, S, PP, \
                                                    splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  if (fx.has_gx) {
    bool done = false;
    const int rc = xgen_fwd(g, fx, X, Xm1, lam, predict, S, st, &done);
    if (done || rc) return rc;
  }
  const int P = x_pairs(g.nx);
  return x_fwd_go<GenericRunner>(g, fx.dev, X, Xm1, lam, predict, S, P,
                                 threads_for((long long)P * g.nx), st);
}


template <class Run>
__global__ void __launch_bounds__(Run::kThreads, Run::template min_blocks<6>())
k_x_inv_plain(Geom g, FftDev fx, const float2* __restrict__ S, float* __restrict__ out, int Pa) {
  const int P = tile_vectors<Run>(Pa);
  extern __shared__ __align__(16) float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const auto io = Run::row_tile(smem + x_tile_offset(nx), nx);
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  float4* stg = reinterpret_cast<float4*>(io.sm);
  load_twiddles(fx, stw);
  grid_dep_wait();
  grid_dep_launch();
  prefetch_packed_spectra<Run::kV>(g, S, stg, P, z, y0);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  const PackedSpecLoad ld{stg, g.nxh, nx, min(P, (g.ny - y0 + 1) / 2)};
  const PlainRowStore ps{out, (long long)z * g.ny * nx, y0, g.ny, nx};
  Run::template run<true>(fx, P, 1.f, false, stw, io, ld, ps);
}

template <class Run>
static int x_plain_go(const Geom& g, const FftDev& f, const float2* S, float* out, int P, int T,
                      cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  size_t smem = sizeof(float2) * (size_t)x_rows_offset(g.nx, P);
  if (int rc = smem_optin(k_x_inv_plain<Run>, smem)) return rc;
  CDX_CHECK(launch_pdl(k_x_inv_plain<Run>, grid, dim3(T), smem, st, g, f, S, out, P));
  CDX_LAUNCH_CHECK("k_x_inv_plain");
  return 0;
}

int launch_x_inv_plain(const Geom& g, const FftLen& fx, const float2* S, float* out,
                       cudaStream_t st) {
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP) \
  case L:               \
    return x_plain_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, S, out, PP, splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  const int P = x_pairs(g.nx);
  return x_plain_go<GenericRunner>(g, fx.dev, S, out, P, threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
