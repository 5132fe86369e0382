// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels
// of the generated x lengths 140, 200, 288, 384, 500, 648, 810, 1008.
#include "decon_x_kernels.cuh"
#include "x_gen_dispatch.h"

namespace cdx {

int xgen_fwd_1(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 140:
      *done = true;
      return x_fwd_go<StaticRunner<SPX140, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX140, 4>(), st);
    case 200:
      *done = true;
      return x_fwd_go<StaticRunner<SPX200, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX200, 4>(), st);
    case 288:
      *done = true;
      return x_fwd_go<StaticRunner<SPX288, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX288, 4>(), st);
    case 384:
      *done = true;
      return x_fwd_go<StaticRunner<SPX384, 4, false, false, 0, 16, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX384, 4>(), st);
    case 500:
      *done = true;
      return x_fwd_go<StaticRunner<SPX500, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX500, 2>(), st);
    case 648:
      *done = true;
      return x_fwd_go<StaticRunner<SPX648, 4, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 4, splan_threads<SPX648, 4>(), st);
    case 810:
      *done = true;
      return x_fwd_go<StaticRunner<SPX810, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX810, 2>(), st);
    case 1008:
      *done = true;
      return x_fwd_go<StaticRunner<SPX1008, 2, false, false, 0, 0, 0>>(g, fx.gxdev, X, Xm1, lam, predict, S, 2, splan_threads<SPX1008, 2>(), st);
    default:
      return 0;
  }
}

int xgen_ratio_1(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 140:
      *done = true;
      return x_ratio_go<StaticRunner<SPX140, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX140, 4>(), st);
    case 200:
      *done = true;
      return x_ratio_go<StaticRunner<SPX200, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX200, 4>(), st);
    case 288:
      *done = true;
      return x_ratio_go<StaticRunner<SPX288, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX288, 4>(), st);
    case 384:
      *done = true;
      return x_ratio_go<StaticRunner<SPX384, 4, false, false, 0, 16, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX384, 4>(), st);
    case 500:
      *done = true;
      return x_ratio_go<StaticRunner<SPX500, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX500, 2>(), st);
    case 648:
      *done = true;
      return x_ratio_go<StaticRunner<SPX648, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 4, splan_threads<SPX648, 4>(), st);
    case 810:
      *done = true;
      return x_ratio_go<StaticRunner<SPX810, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX810, 2>(), st);
    case 1008:
      *done = true;
      return x_ratio_go<StaticRunner<SPX1008, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, raw, eps, 2, splan_threads<SPX1008, 2>(), st);
    default:
      return 0;
  }
}

int xgen_update_1(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  switch (g.nx) {
    case 140:
      *done = true;
      return x_update_go<StaticRunner<SPX140, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX140, 4>(), st);
    case 200:
      *done = true;
      return x_update_go<StaticRunner<SPX200, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX200, 4>(), st);
    case 288:
      *done = true;
      return x_update_go<StaticRunner<SPX288, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX288, 4>(), st);
    case 384:
      *done = true;
      return x_update_go<StaticRunner<SPX384, 4, false, false, 0, 16, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX384, 4>(), st);
    case 500:
      *done = true;
      return x_update_go<StaticRunner<SPX500, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX500, 2>(), st);
    case 648:
      *done = true;
      return x_update_go<StaticRunner<SPX648, 4, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 4, splan_threads<SPX648, 4>(), st);
    case 810:
      *done = true;
      return x_update_go<StaticRunner<SPX810, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX810, 2>(), st);
    case 1008:
      *done = true;
      return x_update_go<StaticRunner<SPX1008, 2, false, false, 0, 0, 0>>(g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, 2, splan_threads<SPX1008, 2>(), st);
    default:
      return 0;
  }
}

}  // namespace cdx
