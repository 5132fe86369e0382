// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 180, 250, 350, 450, 600, 750, 960.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_9(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 180:
      *done = true;
      return x_fwd_go<StaticRunner<SPX180, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX180, 8>(), st);
    case 250:
      *done = true;
      return x_fwd_go<StaticRunner<SPX250, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX250, 8>(), st);
    case 350:
      *done = true;
      return x_fwd_go<StaticRunner<SPX350, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX350, 4>(), st);
    case 450:
      *done = true;
      return x_fwd_go<StaticRunner<SPX450, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX450, 4>(), st);
    case 600:
      *done = true;
      return x_fwd_go<StaticRunner<SPX600, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX600, 2>(), st);
    case 750:
      *done = true;
      return x_fwd_go<StaticRunner<SPX750, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX750, 4>(), st);
    case 960:
      *done = true;
      return x_fwd_go<StaticRunner<SPX960, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX960, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_9(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 180:
      *done = true;
      return x_ratio_go<StaticRunner<SPX180, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX180, 8>(), st);
    case 250:
      *done = true;
      return x_ratio_go<StaticRunner<SPX250, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX250, 8>(), st);
    case 350:
      *done = true;
      return x_ratio_go<StaticRunner<SPX350, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX350, 4>(), st);
    case 450:
      *done = true;
      return x_ratio_go<StaticRunner<SPX450, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX450, 4>(), st);
    case 600:
      *done = true;
      return x_ratio_go<StaticRunner<SPX600, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX600, 2>(), st);
    case 750:
      *done = true;
      return x_ratio_go<StaticRunner<SPX750, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX750, 4>(), st);
    case 960:
      *done = true;
      return x_ratio_go<StaticRunner<SPX960, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX960, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_9(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 180:
      *done = true;
      return x_update_go<StaticRunner<SPX180, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX180, 8>(), st);
    case 250:
      *done = true;
      return x_update_go<StaticRunner<SPX250, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX250, 8>(), st);
    case 350:
      *done = true;
      return x_update_go<StaticRunner<SPX350, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX350, 4>(), st);
    case 450:
      *done = true;
      return x_update_go<StaticRunner<SPX450, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX450, 4>(), st);
    case 600:
      *done = true;
      return x_update_go<StaticRunner<SPX600, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX600, 2>(), st);
    case 750:
      *done = true;
      return x_update_go<StaticRunner<SPX750, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX750, 4>(), st);
    case 960:
      *done = true;
      return x_update_go<StaticRunner<SPX960, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX960, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
