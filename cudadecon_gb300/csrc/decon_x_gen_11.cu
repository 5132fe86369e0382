// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 192, 270, 375, 486, 630, 784, 980.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_11(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 192:
      *done = true;
      return x_fwd_go<StaticRunner<SPX192, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX192, 8>(), st);
    case 270:
      *done = true;
      return x_fwd_go<StaticRunner<SPX270, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX270, 4>(), st);
    case 375:
      *done = true;
      return x_fwd_go<StaticRunner<SPX375, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX375, 8>(), st);
    case 486:
      *done = true;
      return x_fwd_go<StaticRunner<SPX486, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX486, 4>(), st);
    case 630:
      *done = true;
      return x_fwd_go<StaticRunner<SPX630, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX630, 4>(), st);
    case 784:
      *done = true;
      return x_fwd_go<StaticRunner<SPX784, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX784, 2>(), st);
    case 980:
      *done = true;
      return x_fwd_go<StaticRunner<SPX980, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX980, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_11(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 192:
      *done = true;
      return x_ratio_go<StaticRunner<SPX192, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX192, 8>(), st);
    case 270:
      *done = true;
      return x_ratio_go<StaticRunner<SPX270, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX270, 4>(), st);
    case 375:
      *done = true;
      return x_ratio_go<StaticRunner<SPX375, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX375, 8>(), st);
    case 486:
      *done = true;
      return x_ratio_go<StaticRunner<SPX486, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX486, 4>(), st);
    case 630:
      *done = true;
      return x_ratio_go<StaticRunner<SPX630, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX630, 4>(), st);
    case 784:
      *done = true;
      return x_ratio_go<StaticRunner<SPX784, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX784, 2>(), st);
    case 980:
      *done = true;
      return x_ratio_go<StaticRunner<SPX980, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX980, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_11(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 192:
      *done = true;
      return x_update_go<StaticRunner<SPX192, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX192, 8>(), st);
    case 270:
      *done = true;
      return x_update_go<StaticRunner<SPX270, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX270, 4>(), st);
    case 375:
      *done = true;
      return x_update_go<StaticRunner<SPX375, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX375, 8>(), st);
    case 486:
      *done = true;
      return x_update_go<StaticRunner<SPX486, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX486, 4>(), st);
    case 630:
      *done = true;
      return x_update_go<StaticRunner<SPX630, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX630, 4>(), st);
    case 784:
      *done = true;
      return x_update_go<StaticRunner<SPX784, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX784, 2>(), st);
    case 980:
      *done = true;
      return x_update_go<StaticRunner<SPX980, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX980, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
