// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 175, 245, 343, 448, 588, 735, 945.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_8(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 175:
      *done = true;
      return x_fwd_go<StaticRunner<SPX175, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX175, 8>(), st);
    case 245:
      *done = true;
      return x_fwd_go<StaticRunner<SPX245, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX245, 8>(), st);
    case 343:
      *done = true;
      return x_fwd_go<StaticRunner<SPX343, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX343, 4>(), st);
    case 448:
      *done = true;
      return x_fwd_go<StaticRunner<SPX448, 4, false, false, 0, 16, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX448, 4>(), st);
    case 588:
      *done = true;
      return x_fwd_go<StaticRunner<SPX588, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX588, 4>(), st);
    case 735:
      *done = true;
      return x_fwd_go<StaticRunner<SPX735, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX735, 2>(), st);
    case 945:
      *done = true;
      return x_fwd_go<StaticRunner<SPX945, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX945, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_8(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 175:
      *done = true;
      return x_ratio_go<StaticRunner<SPX175, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX175, 8>(), st);
    case 245:
      *done = true;
      return x_ratio_go<StaticRunner<SPX245, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX245, 8>(), st);
    case 343:
      *done = true;
      return x_ratio_go<StaticRunner<SPX343, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX343, 4>(), st);
    case 448:
      *done = true;
      return x_ratio_go<StaticRunner<SPX448, 4, false, false, 0, 16, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX448, 4>(), st);
    case 588:
      *done = true;
      return x_ratio_go<StaticRunner<SPX588, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX588, 4>(), st);
    case 735:
      *done = true;
      return x_ratio_go<StaticRunner<SPX735, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX735, 2>(), st);
    case 945:
      *done = true;
      return x_ratio_go<StaticRunner<SPX945, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX945, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_8(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 175:
      *done = true;
      return x_update_go<StaticRunner<SPX175, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX175, 8>(), st);
    case 245:
      *done = true;
      return x_update_go<StaticRunner<SPX245, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX245, 8>(), st);
    case 343:
      *done = true;
      return x_update_go<StaticRunner<SPX343, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX343, 4>(), st);
    case 448:
      *done = true;
      return x_update_go<StaticRunner<SPX448, 4, false, false, 0, 16, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX448, 4>(), st);
    case 588:
      *done = true;
      return x_update_go<StaticRunner<SPX588, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX588, 4>(), st);
    case 735:
      *done = true;
      return x_update_go<StaticRunner<SPX735, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX735, 2>(), st);
    case 945:
      *done = true;
      return x_update_go<StaticRunner<SPX945, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX945, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
