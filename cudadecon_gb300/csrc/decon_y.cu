// y pass of the 3D transforms: complex FFTs along y of every (kx, z) row.
#include "decon_common.cuh"

namespace cdx {

// ---------------------------------------------------------------- y pass
template <bool INV, class Run>
__global__ void __launch_bounds__(Run::kThreads, Run::template min_blocks<8>())
k_y_pass(Geom g, FftDev fy, float2* __restrict__ S, int V) {
  extern __shared__ __align__(16) float2 smem[];
  const int ny = g.ny;
  float2* stw = smem;
  const auto io = Run::row_tile(smem + ny, ny);
  load_twiddles(fy, stw);
  grid_dep_wait();
  grid_dep_launch();
  __syncthreads();
  const SpecRowIO gio{S, (long long)blockIdx.x * V, (long long)g.nxh * g.nz, g.nyp};
  Run::template run<INV>(fy, V, 1.f, false, stw, io, gio, gio);
}

template <bool INV, class Run>
static int y_go(const Geom& g, const FftDev& f, float2* S, int V, int T, cudaStream_t st) {
  const long long nrows = (long long)g.nxh * g.nz;
  // a two-radix static plan's padded middle layout may exceed the generic
  // padded tile
  size_t tile = spad_size(V * g.ny);
  if (Run::kStatic && (size_t)Run::kTileF2 > tile) tile = Run::kTileF2;
  size_t smem = sizeof(float2) * ((size_t)g.ny + tile);
  dim3 grid((unsigned)((nrows + V - 1) / V));
  if (int rc = smem_optin(k_y_pass<INV, Run>, smem)) return rc;
  CDX_CHECK(launch_pdl(k_y_pass<INV, Run>, grid, dim3(T), smem, st, g, f, S, V));
  CDX_LAUNCH_CHECK("k_y_pass");
  return 0;
}

template <bool INV>
static int y_dispatch(const Geom& g, const FftLen& fy, float2* S, cudaStream_t st) {
  if (fy.has_static) switch (g.ny) {
#define CDX_CASE(L, VV, RR, B0, B1)                                                   \
  case L:                                                                             \
    return y_go<INV, StaticRunner<SP##L, VV, false, false, RR, B0, B1>>(               \
        g, fy.sdev, S, VV, splan_threads<SP##L, VV>(), st);
      CDX_Y_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  int V = 2048 / g.ny;
  if (V < 1) V = 1;
  return y_go<INV, GenericRunner>(g, fy.dev, S, V, threads_for((long long)V * g.ny), st);
}

int launch_y_pass(const Geom& g, const FftLen& fy, float2* S, bool inverse, cudaStream_t st) {
  return inverse ? y_dispatch<true>(g, fy, S, st) : y_dispatch<false>(g, fy, S, st);
}

}  // namespace cdx
