// Inverse x pass of the second convolution: C2R, estimate update and the
// acceleration-factor dot products (per-block partial sums, then a one-block
// kernel finishes lambda).
#include "decon_common.cuh"

namespace cdx {

// The next acceleration factor from the blocks' partial sums (one float4 per
// update block): sums in a fixed order, then calcAccelFactor
// (RLgpuImpl.cu:565) in double and the clamp of RL-Biggs-Andrews.cpp:298.
// One block; launched right after the update pass, so the update blocks need
// no fence or completion ticket.
__global__ void __launch_bounds__(1024) k_lambda(const float4* partials, int nblk,
                                                 float* lam_next, float eps) {
  __shared__ float4 red[32];
  grid_dep_wait();
  grid_dep_launch();
  // each thread sums partials t, t + T, t + 2T, ...; the loads of a batch
  // are issued together (zeros past the end add nothing)
  constexpr int kBatch = 8;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i0 = threadIdx.x; i0 < nblk; i0 += kBatch * blockDim.x) {
    float4 r[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int i = i0 + u * blockDim.x;
      r[u] = i < nblk ? __ldcg(partials + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) ff_add(acc, r[u]);
  }
  const float4 s = block_sum2_ff(acc.x, acc.y, acc.z, acc.w, red);
  if (threadIdx.x == 0) {
    const double a = (double)s.x + (double)s.y, b = (double)s.z + (double)s.w;
    double l = a / (b + (double)eps);
    l = (1.0 < l) ? 1.0 : l;
    l = (l < 0.0) ? 0.0 : l;
    *lam_next = (float)l;
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
  const PackedSpecLoad ld{stg, g.nxh, nx, (nr + 1) / 2};
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const UpdateStore us{Ys, Gs, Xout, G, dots, (long long)z * g.ny * nx, y0, g.ny, nx, acc};
  Run::template run<true>(fx, P, 1.f, false, stw, io, ld, us);
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

int launch_lambda(const float4* partials, int nblk, float* lam_next, float eps, cudaStream_t st) {
  CDX_CHECK(launch_pdl(k_lambda, dim3(1), dim3(1024), 0, st, partials, nblk, lam_next, eps));
  CDX_LAUNCH_CHECK("k_lambda");
  return 0;
}

int launch_x_inv_update(const Geom& g, const FftLen& fx, const float2* S, const float* Y,
                        float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                        cudaStream_t st) {
  if (fx.has_tc && dft_form() == 1)
    return launch_xtc_update(g, fx.tc, S, Y, Xout, G, dots, w, lam_next, eps, fx.tc.d_err, st);
  if (fx.has_xr) switch (g.nx) {
#define CDX_XR_CASE(L, PP, ...)                                                                 \
  case L:                                                                                       \
    return x_update_go<StaticRunner<SPR##L, PP, false>>(g, fx.xrdev, S, Y, Xout, G, dots, w,    \
                                                        lam_next, eps, PP,                      \
                                                        splan_threads<SPR##L, PP>(), st);
      CDX_XR_PLANS(CDX_XR_CASE)
#undef CDX_XR_CASE
      default:
        break;
    }
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP)                                                                    \
  case L:                                                                                  \
    return x_update_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, S, Y, Xout, G, dots, \
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
