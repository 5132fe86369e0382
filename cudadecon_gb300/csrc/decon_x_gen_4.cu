// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 150, 224, 315, 405, 540, 686, 875.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_4(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 150:
      *done = true;
      return x_fwd_go<StaticRunner<SPX150, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX150, 8>(), st);
    case 224:
      *done = true;
      return x_fwd_go<StaticRunner<SPX224, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX224, 4>(), st);
    case 315:
      *done = true;
      return x_fwd_go<StaticRunner<SPX315, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX315, 4>(), st);
    case 405:
      *done = true;
      return x_fwd_go<StaticRunner<SPX405, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX405, 4>(), st);
    case 540:
      *done = true;
      return x_fwd_go<StaticRunner<SPX540, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX540, 4>(), st);
    case 686:
      *done = true;
      return x_fwd_go<StaticRunner<SPX686, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX686, 4>(), st);
    case 875:
      *done = true;
      return x_fwd_go<StaticRunner<SPX875, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX875, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_4(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 150:
      *done = true;
      return x_ratio_go<StaticRunner<SPX150, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX150, 8>(), st);
    case 224:
      *done = true;
      return x_ratio_go<StaticRunner<SPX224, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX224, 4>(), st);
    case 315:
      *done = true;
      return x_ratio_go<StaticRunner<SPX315, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX315, 4>(), st);
    case 405:
      *done = true;
      return x_ratio_go<StaticRunner<SPX405, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX405, 4>(), st);
    case 540:
      *done = true;
      return x_ratio_go<StaticRunner<SPX540, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX540, 4>(), st);
    case 686:
      *done = true;
      return x_ratio_go<StaticRunner<SPX686, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX686, 4>(), st);
    case 875:
      *done = true;
      return x_ratio_go<StaticRunner<SPX875, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX875, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_4(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 150:
      *done = true;
      return x_update_go<StaticRunner<SPX150, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX150, 8>(), st);
    case 224:
      *done = true;
      return x_update_go<StaticRunner<SPX224, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX224, 4>(), st);
    case 315:
      *done = true;
      return x_update_go<StaticRunner<SPX315, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX315, 4>(), st);
    case 405:
      *done = true;
      return x_update_go<StaticRunner<SPX405, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX405, 4>(), st);
    case 540:
      *done = true;
      return x_update_go<StaticRunner<SPX540, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX540, 4>(), st);
    case 686:
      *done = true;
      return x_update_go<StaticRunner<SPX686, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX686, 4>(), st);
    case 875:
      *done = true;
      return x_update_go<StaticRunner<SPX875, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX875, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
