// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 147, 216, 300, 400, 525, 675, 864.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_3(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 147:
      *done = true;
      return x_fwd_go<StaticRunner<SPX147, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX147, 8>(), st);
    case 216:
      *done = true;
      return x_fwd_go<StaticRunner<SPX216, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX216, 4>(), st);
    case 300:
      *done = true;
      return x_fwd_go<StaticRunner<SPX300, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX300, 4>(), st);
    case 400:
      *done = true;
      return x_fwd_go<StaticRunner<SPX400, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX400, 4>(), st);
    case 525:
      *done = true;
      return x_fwd_go<StaticRunner<SPX525, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX525, 2>(), st);
    case 675:
      *done = true;
      return x_fwd_go<StaticRunner<SPX675, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX675, 2>(), st);
    case 864:
      *done = true;
      return x_fwd_go<StaticRunner<SPX864, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX864, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_3(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 147:
      *done = true;
      return x_ratio_go<StaticRunner<SPX147, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX147, 8>(), st);
    case 216:
      *done = true;
      return x_ratio_go<StaticRunner<SPX216, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX216, 4>(), st);
    case 300:
      *done = true;
      return x_ratio_go<StaticRunner<SPX300, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX300, 4>(), st);
    case 400:
      *done = true;
      return x_ratio_go<StaticRunner<SPX400, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX400, 4>(), st);
    case 525:
      *done = true;
      return x_ratio_go<StaticRunner<SPX525, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX525, 2>(), st);
    case 675:
      *done = true;
      return x_ratio_go<StaticRunner<SPX675, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX675, 2>(), st);
    case 864:
      *done = true;
      return x_ratio_go<StaticRunner<SPX864, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX864, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_3(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 147:
      *done = true;
      return x_update_go<StaticRunner<SPX147, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX147, 8>(), st);
    case 216:
      *done = true;
      return x_update_go<StaticRunner<SPX216, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX216, 4>(), st);
    case 300:
      *done = true;
      return x_update_go<StaticRunner<SPX300, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX300, 4>(), st);
    case 400:
      *done = true;
      return x_update_go<StaticRunner<SPX400, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX400, 4>(), st);
    case 525:
      *done = true;
      return x_update_go<StaticRunner<SPX525, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX525, 2>(), st);
    case 675:
      *done = true;
      return x_update_go<StaticRunner<SPX675, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX675, 2>(), st);
    case 864:
      *done = true;
      return x_update_go<StaticRunner<SPX864, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX864, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
