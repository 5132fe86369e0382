// Generated by cudadecon_gb300/gen_plans.py (do not edit): dispatch of the
// x passes of the generated x lengths to the units decon_x_gen_<k>.cu.
// Each function sets *done when its length has a generated plan.
#pragma once

#include "kernels.h"

namespace cdx {

int xgen_fwd_0(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_1(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_2(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_3(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_4(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_5(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_6(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_7(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_8(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_9(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_10(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_fwd_11(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done);
int xgen_ratio_0(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_1(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_2(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_3(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_4(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_5(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_6(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_7(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_8(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_9(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_10(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_ratio_11(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done);
int xgen_update_0(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_1(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_2(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_3(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_4(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_5(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_6(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_7(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_8(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_9(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_10(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);
int xgen_update_11(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done);

inline int xgen_fwd(const Geom& g, const FftLen& fx, const float* X, float* Xm1, const float* lam, int predict, float2* S, cudaStream_t st, bool* done) {
  int rc = 0;
  *done = false;
  if ((rc = xgen_fwd_0(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_1(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_2(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_3(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_4(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_5(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_6(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_7(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_8(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_9(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_10(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  if ((rc = xgen_fwd_11(g, fx, X, Xm1, lam, predict, S, st, done)) || *done) return rc;
  return 0;
}

inline int xgen_ratio(const Geom& g, const FftLen& fx, float2* S, const float* raw, float eps, cudaStream_t st, bool* done) {
  int rc = 0;
  *done = false;
  if ((rc = xgen_ratio_0(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_1(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_2(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_3(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_4(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_5(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_6(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_7(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_8(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_9(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_10(g, fx, S, raw, eps, st, done)) || *done) return rc;
  if ((rc = xgen_ratio_11(g, fx, S, raw, eps, st, done)) || *done) return rc;
  return 0;
}

inline int xgen_update(const Geom& g, const FftLen& fx, const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st, bool* done) {
  int rc = 0;
  *done = false;
  if ((rc = xgen_update_0(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_1(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_2(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_3(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_4(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_5(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_6(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_7(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_8(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_9(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_10(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  if ((rc = xgen_update_11(g, fx, S, Y, Xout, G, dots, w, lam_next, eps, st, done)) || *done) return rc;
  return 0;
}

}  // namespace cdx
