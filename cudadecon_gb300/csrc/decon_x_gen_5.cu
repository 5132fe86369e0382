// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 160, 225, 320, 420, 560, 700, 882.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_5(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 160:
      *done = true;
      return x_fwd_go<StaticRunner<SPX160, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX160, 4>(), st);
    case 225:
      *done = true;
      return x_fwd_go<StaticRunner<SPX225, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX225, 2>(), st);
    case 320:
      *done = true;
      return x_fwd_go<StaticRunner<SPX320, 4, false, false, 0, 16, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX320, 4>(), st);
    case 420:
      *done = true;
      return x_fwd_go<StaticRunner<SPX420, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX420, 4>(), st);
    case 560:
      *done = true;
      return x_fwd_go<StaticRunner<SPX560, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX560, 4>(), st);
    case 700:
      *done = true;
      return x_fwd_go<StaticRunner<SPX700, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX700, 4>(), st);
    case 882:
      *done = true;
      return x_fwd_go<StaticRunner<SPX882, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX882, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_5(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 160:
      *done = true;
      return x_ratio_go<StaticRunner<SPX160, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX160, 4>(), st);
    case 225:
      *done = true;
      return x_ratio_go<StaticRunner<SPX225, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX225, 2>(), st);
    case 320:
      *done = true;
      return x_ratio_go<StaticRunner<SPX320, 4, false, false, 0, 16, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX320, 4>(), st);
    case 420:
      *done = true;
      return x_ratio_go<StaticRunner<SPX420, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX420, 4>(), st);
    case 560:
      *done = true;
      return x_ratio_go<StaticRunner<SPX560, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX560, 4>(), st);
    case 700:
      *done = true;
      return x_ratio_go<StaticRunner<SPX700, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX700, 4>(), st);
    case 882:
      *done = true;
      return x_ratio_go<StaticRunner<SPX882, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX882, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_5(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 160:
      *done = true;
      return x_update_go<StaticRunner<SPX160, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX160, 4>(), st);
    case 225:
      *done = true;
      return x_update_go<StaticRunner<SPX225, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX225, 2>(), st);
    case 320:
      *done = true;
      return x_update_go<StaticRunner<SPX320, 4, false, false, 0, 16, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX320, 4>(), st);
    case 420:
      *done = true;
      return x_update_go<StaticRunner<SPX420, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX420, 4>(), st);
    case 560:
      *done = true;
      return x_update_go<StaticRunner<SPX560, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX560, 4>(), st);
    case 700:
      *done = true;
      return x_update_go<StaticRunner<SPX700, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX700, 4>(), st);
    case 882:
      *done = true;
      return x_update_go<StaticRunner<SPX882, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX882, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
