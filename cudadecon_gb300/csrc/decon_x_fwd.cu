// Forward x pass of the RL iteration (prediction prologue + R2C along x) and
// the plain inverse x pass used by the convolution test hook.
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
