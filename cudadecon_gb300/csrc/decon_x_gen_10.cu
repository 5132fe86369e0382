// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 189, 252, 360, 480, 625, 768, 972.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_10(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 189:
      *done = true;
      return x_fwd_go<StaticRunner<SPX189, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX189, 8>(), st);
    case 252:
      *done = true;
      return x_fwd_go<StaticRunner<SPX252, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX252, 8>(), st);
    case 360:
      *done = true;
      return x_fwd_go<StaticRunner<SPX360, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX360, 4>(), st);
    case 480:
      *done = true;
      return x_fwd_go<StaticRunner<SPX480, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX480, 4>(), st);
    case 625:
      *done = true;
      return x_fwd_go<StaticRunner<SPX625, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX625, 4>(), st);
    case 768:
      *done = true;
      return x_fwd_go<StaticRunner<SPX768, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX768, 2>(), st);
    case 972:
      *done = true;
      return x_fwd_go<StaticRunner<SPX972, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX972, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_10(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 189:
      *done = true;
      return x_ratio_go<StaticRunner<SPX189, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX189, 8>(), st);
    case 252:
      *done = true;
      return x_ratio_go<StaticRunner<SPX252, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX252, 8>(), st);
    case 360:
      *done = true;
      return x_ratio_go<StaticRunner<SPX360, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX360, 4>(), st);
    case 480:
      *done = true;
      return x_ratio_go<StaticRunner<SPX480, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX480, 4>(), st);
    case 625:
      *done = true;
      return x_ratio_go<StaticRunner<SPX625, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX625, 4>(), st);
    case 768:
      *done = true;
      return x_ratio_go<StaticRunner<SPX768, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX768, 2>(), st);
    case 972:
      *done = true;
      return x_ratio_go<StaticRunner<SPX972, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX972, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_10(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 189:
      *done = true;
      return x_update_go<StaticRunner<SPX189, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX189, 8>(), st);
    case 252:
      *done = true;
      return x_update_go<StaticRunner<SPX252, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX252, 8>(), st);
    case 360:
      *done = true;
      return x_update_go<StaticRunner<SPX360, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX360, 4>(), st);
    case 480:
      *done = true;
      return x_update_go<StaticRunner<SPX480, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX480, 4>(), st);
    case 625:
      *done = true;
      return x_update_go<StaticRunner<SPX625, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX625, 4>(), st);
    case 768:
      *done = true;
      return x_update_go<StaticRunner<SPX768, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX768, 2>(), st);
    case 972:
      *done = true;
      return x_update_go<StaticRunner<SPX972, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX972, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
