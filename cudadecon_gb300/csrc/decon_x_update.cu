// Inverse x pass of the second convolution: C2R, estimate update and the
// acceleration-factor dot products (per-block partial sums, then a one-block
// kernel finishes lambda).
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

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
  if (fx.has_gx) {
    bool done = false;
    const int rc = xgen_update(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, &done);
    if (done || rc) return rc;
  }
  const int P = x_pairs(g.nx);
  return x_update_go<GenericRunner>(g, fx.dev, S, Y, Xout, G, dots, w, lam_next, eps, P,
                                    threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
