// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 168, 243, 336, 441, 576, 729, 900.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_7(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 168:
      *done = true;
      return x_fwd_go<StaticRunner<SPX168, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX168, 8>(), st);
    case 243:
      *done = true;
      return x_fwd_go<StaticRunner<SPX243, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX243, 4>(), st);
    case 336:
      *done = true;
      return x_fwd_go<StaticRunner<SPX336, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX336, 4>(), st);
    case 441:
      *done = true;
      return x_fwd_go<StaticRunner<SPX441, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX441, 4>(), st);
    case 576:
      *done = true;
      return x_fwd_go<StaticRunner<SPX576, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX576, 2>(), st);
    case 729:
      *done = true;
      return x_fwd_go<StaticRunner<SPX729, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX729, 4>(), st);
    case 900:
      *done = true;
      return x_fwd_go<StaticRunner<SPX900, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX900, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_7(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 168:
      *done = true;
      return x_ratio_go<StaticRunner<SPX168, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX168, 8>(), st);
    case 243:
      *done = true;
      return x_ratio_go<StaticRunner<SPX243, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX243, 4>(), st);
    case 336:
      *done = true;
      return x_ratio_go<StaticRunner<SPX336, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX336, 4>(), st);
    case 441:
      *done = true;
      return x_ratio_go<StaticRunner<SPX441, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX441, 4>(), st);
    case 576:
      *done = true;
      return x_ratio_go<StaticRunner<SPX576, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX576, 2>(), st);
    case 729:
      *done = true;
      return x_ratio_go<StaticRunner<SPX729, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX729, 4>(), st);
    case 900:
      *done = true;
      return x_ratio_go<StaticRunner<SPX900, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX900, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_7(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 168:
      *done = true;
      return x_update_go<StaticRunner<SPX168, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX168, 8>(), st);
    case 243:
      *done = true;
      return x_update_go<StaticRunner<SPX243, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX243, 4>(), st);
    case 336:
      *done = true;
      return x_update_go<StaticRunner<SPX336, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX336, 4>(), st);
    case 441:
      *done = true;
      return x_update_go<StaticRunner<SPX441, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX441, 4>(), st);
    case 576:
      *done = true;
      return x_update_go<StaticRunner<SPX576, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX576, 2>(), st);
    case 729:
      *done = true;
      return x_update_go<StaticRunner<SPX729, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX729, 4>(), st);
    case 900:
      *done = true;
      return x_update_go<StaticRunner<SPX900, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX900, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
