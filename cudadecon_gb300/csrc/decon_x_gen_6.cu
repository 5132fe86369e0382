// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 162, 240, 324, 432, 567, 720, 896.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_6(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 162:
      *done = true;
      return x_fwd_go<StaticRunner<SPX162, 8, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 8, splan_threads<SPX162, 8>(), st);
    case 240:
      *done = true;
      return x_fwd_go<StaticRunner<SPX240, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX240, 4>(), st);
    case 324:
      *done = true;
      return x_fwd_go<StaticRunner<SPX324, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX324, 4>(), st);
    case 432:
      *done = true;
      return x_fwd_go<StaticRunner<SPX432, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX432, 4>(), st);
    case 567:
      *done = true;
      return x_fwd_go<StaticRunner<SPX567, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX567, 2>(), st);
    case 720:
      *done = true;
      return x_fwd_go<StaticRunner<SPX720, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX720, 2>(), st);
    case 896:
      *done = true;
      return x_fwd_go<StaticRunner<SPX896, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX896, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_6(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 162:
      *done = true;
      return x_ratio_go<StaticRunner<SPX162, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 8, splan_threads<SPX162, 8>(), st);
    case 240:
      *done = true;
      return x_ratio_go<StaticRunner<SPX240, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX240, 4>(), st);
    case 324:
      *done = true;
      return x_ratio_go<StaticRunner<SPX324, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX324, 4>(), st);
    case 432:
      *done = true;
      return x_ratio_go<StaticRunner<SPX432, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX432, 4>(), st);
    case 567:
      *done = true;
      return x_ratio_go<StaticRunner<SPX567, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX567, 2>(), st);
    case 720:
      *done = true;
      return x_ratio_go<StaticRunner<SPX720, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX720, 2>(), st);
    case 896:
      *done = true;
      return x_ratio_go<StaticRunner<SPX896, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX896, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_6(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 162:
      *done = true;
      return x_update_go<StaticRunner<SPX162, 8, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 8, splan_threads<SPX162, 8>(), st);
    case 240:
      *done = true;
      return x_update_go<StaticRunner<SPX240, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX240, 4>(), st);
    case 324:
      *done = true;
      return x_update_go<StaticRunner<SPX324, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX324, 4>(), st);
    case 432:
      *done = true;
      return x_update_go<StaticRunner<SPX432, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX432, 4>(), st);
    case 567:
      *done = true;
      return x_update_go<StaticRunner<SPX567, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX567, 2>(), st);
    case 720:
      *done = true;
      return x_update_go<StaticRunner<SPX720, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX720, 2>(), st);
    case 896:
      *done = true;
      return x_update_go<StaticRunner<SPX896, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX896, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
