// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 144, 210, 294, 392, 504, 672, 840.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_2(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 144:
      *done = true;
      return x_fwd_go<StaticRunner<SPX144, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX144, 4>(), st);
    case 210:
      *done = true;
      return x_fwd_go<StaticRunner<SPX210, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX210, 8>(), st);
    case 294:
      *done = true;
      return x_fwd_go<StaticRunner<SPX294, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX294, 4>(), st);
    case 392:
      *done = true;
      return x_fwd_go<StaticRunner<SPX392, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX392, 4>(), st);
    case 504:
      *done = true;
      return x_fwd_go<StaticRunner<SPX504, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX504, 4>(), st);
    case 672:
      *done = true;
      return x_fwd_go<StaticRunner<SPX672, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX672, 4>(), st);
    case 840:
      *done = true;
      return x_fwd_go<StaticRunner<SPX840, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX840, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_2(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 144:
      *done = true;
      return x_ratio_go<StaticRunner<SPX144, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX144, 4>(), st);
    case 210:
      *done = true;
      return x_ratio_go<StaticRunner<SPX210, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX210, 8>(), st);
    case 294:
      *done = true;
      return x_ratio_go<StaticRunner<SPX294, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX294, 4>(), st);
    case 392:
      *done = true;
      return x_ratio_go<StaticRunner<SPX392, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX392, 4>(), st);
    case 504:
      *done = true;
      return x_ratio_go<StaticRunner<SPX504, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX504, 4>(), st);
    case 672:
      *done = true;
      return x_ratio_go<StaticRunner<SPX672, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX672, 4>(), st);
    case 840:
      *done = true;
      return x_ratio_go<StaticRunner<SPX840, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX840, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_2(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 144:
      *done = true;
      return x_update_go<StaticRunner<SPX144, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX144, 4>(), st);
    case 210:
      *done = true;
      return x_update_go<StaticRunner<SPX210, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX210, 8>(), st);
    case 294:
      *done = true;
      return x_update_go<StaticRunner<SPX294, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX294, 4>(), st);
    case 392:
      *done = true;
      return x_update_go<StaticRunner<SPX392, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX392, 4>(), st);
    case 504:
      *done = true;
      return x_update_go<StaticRunner<SPX504, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX504, 4>(), st);
    case 672:
      *done = true;
      return x_update_go<StaticRunner<SPX672, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX672, 4>(), st);
    case 840:
      *done = true;
      return x_update_go<StaticRunner<SPX840, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX840, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
