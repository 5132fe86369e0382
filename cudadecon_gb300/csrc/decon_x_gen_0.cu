// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 135, 196, 280, 378, 490, 640, 800, 1000.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_0(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 135:
      *done = true;
      return x_fwd_go<StaticRunner<SPX135, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX135, 4>(), st);
    case 196:
      *done = true;
      return x_fwd_go<StaticRunner<SPX196, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX196, 8>(), st);
    case 280:
      *done = true;
      return x_fwd_go<StaticRunner<SPX280, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX280, 4>(), st);
    case 378:
      *done = true;
      return x_fwd_go<StaticRunner<SPX378, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX378, 4>(), st);
    case 490:
      *done = true;
      return x_fwd_go<StaticRunner<SPX490, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX490, 4>(), st);
    case 640:
      *done = true;
      return x_fwd_go<StaticRunner<SPX640, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX640, 2>(), st);
    case 800:
      *done = true;
      return x_fwd_go<StaticRunner<SPX800, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX800, 2>(), st);
    case 1000:
      *done = true;
      return x_fwd_go<StaticRunner<SPX1000, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX1000, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_0(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 135:
      *done = true;
      return x_ratio_go<StaticRunner<SPX135, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX135, 4>(), st);
    case 196:
      *done = true;
      return x_ratio_go<StaticRunner<SPX196, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX196, 8>(), st);
    case 280:
      *done = true;
      return x_ratio_go<StaticRunner<SPX280, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX280, 4>(), st);
    case 378:
      *done = true;
      return x_ratio_go<StaticRunner<SPX378, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX378, 4>(), st);
    case 490:
      *done = true;
      return x_ratio_go<StaticRunner<SPX490, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX490, 4>(), st);
    case 640:
      *done = true;
      return x_ratio_go<StaticRunner<SPX640, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX640, 2>(), st);
    case 800:
      *done = true;
      return x_ratio_go<StaticRunner<SPX800, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX800, 2>(), st);
    case 1000:
      *done = true;
      return x_ratio_go<StaticRunner<SPX1000, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX1000, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_0(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 135:
      *done = true;
      return x_update_go<StaticRunner<SPX135, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX135, 4>(), st);
    case 196:
      *done = true;
      return x_update_go<StaticRunner<SPX196, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX196, 8>(), st);
    case 280:
      *done = true;
      return x_update_go<StaticRunner<SPX280, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX280, 4>(), st);
    case 378:
      *done = true;
      return x_update_go<StaticRunner<SPX378, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX378, 4>(), st);
    case 490:
      *done = true;
      return x_update_go<StaticRunner<SPX490, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX490, 4>(), st);
    case 640:
      *done = true;
      return x_update_go<StaticRunner<SPX640, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX640, 2>(), st);
    case 800:
      *done = true;
      return x_update_go<StaticRunner<SPX800, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX800, 2>(), st);
    case 1000:
      *done = true;
      return x_update_go<StaticRunner<SPX1000, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX1000, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
