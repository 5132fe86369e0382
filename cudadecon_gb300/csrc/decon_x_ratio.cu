// Inverse x pass of the first convolution: C2R, RL ratio, and R2C of the
// ratio for the second convolution.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

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
  if (fx.has_gx) {
    bool done = false;
    const int rc = xgen_ratio(g, fx, S, raw, eps, st, &done);
    if (done || rc) return rc;
  }
  const int P = x_pairs(g.nx);
  return x_ratio_go<GenericRunner>(g, fx.dev, S, raw, eps, P, threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
