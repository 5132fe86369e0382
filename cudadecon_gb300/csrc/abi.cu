// C ABI and host orchestration.
//
// Session state mirrors the reference library's globals
// (src/RL-Biggs-Andrews.cpp:459-466 and the bleach statics at :46-47): the
// output sizes, deskew factor and width, rotation matrix and OTF survive from
// RL_interface_init until RL_cleanup.  Device work buffers, FFT twiddle
// tables and OTF tables are allocated once per decon grid and reused across
// RL_interface calls (the reference allocates and frees them on every call).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cudadecon.h"
#include "accel.cuh"
#include "kernels.h"
#include "otf_io.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace cdx {

// ---------------------------------------------------------------- errors
static thread_local std::string g_err;
static std::string g_err_shared;
static std::mutex g_err_mu;

void set_error(const char* where, const char* what) {
  std::string s = std::string(where) + ": " + what;
  g_err = s;
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err_shared = s;
}

void set_cuda_error(const char* where, cudaError_t err) { set_error(where, cudaGetErrorString(err)); }

// ---------------------------------------------------------------- sizes
// Good FFT sizes are products of 2, 3, 5 and 7 (notGoodDimension /
// findOptimalDimension, src/RL-Biggs-Andrews.cpp:18-43).  Sizes below 2 have
// no good size below them (the reference recurses forever); 0 is returned.
static bool not_good_dimension(unsigned num) {
  if (num == 2 || num == 3 || num == 5 || num == 7) return false;
  if (num < 2) return true;
  if (num % 2 == 0) return not_good_dimension(num / 2);
  if (num % 3 == 0) return not_good_dimension(num / 3);
  if (num % 5 == 0) return not_good_dimension(num / 5);
  if (num % 7 == 0) return not_good_dimension(num / 7);
  return true;
}

static unsigned find_optimal_dimension(unsigned in, int step = -1) {
  unsigned out = in;
  while (out >= 2 && not_good_dimension(out)) out += step;
  return out >= 2 ? out : 0;
}

// ---------------------------------------------------------------- device buffers
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  int ensure(size_t count) {
    if (count <= n && p) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) return 0;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * count);
    if (e != cudaSuccess) {
      p = nullptr;
      set_cuda_error("cudaMalloc", e);
      return e;
    }
    n = count;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// FFT plans and OTF table for one decon grid.
struct GridPlan {
  bool valid = false;
  Geom g{};
  FftLen fx, fy, fz;
  OtfDev otf{};
  DevBuf<float4> tz;
  DevBuf<float2> full;
  void release() {
    fft_len_free(fx);
    fft_len_free(fy);
    fft_len_free(fz);
    tz.release();
    full.release();
    valid = false;
  }
};

struct Session {
  // values set by RL_interface_init (reference globals)
  bool inited = false;
  unsigned output_nx = 0, output_ny = 0, output_nz = 0;
  bool bCrop = false;
  double deskewFactor = 0.0;
  unsigned deskewedXdim = 0;
  bool has_rot = false;
  float rot[4] = {0, 0, 0, 0};
  float dr = 0, dz = 0;  // dz after the deskew update
  float dkx_otf = 0, dky_otf = 0, dkz_otf = 0;
  RawOtfDims od{};
  DevBuf<float2> raw_otf;
  // bleach correction statics (RL-Biggs-Andrews.cpp:46-47)
  double intensity_overall0 = 0.0;
  bool bFirstTime = true;
  // work buffers
  GridPlan plan;
  DevBuf<unsigned short> u16in;
  DevBuf<float> pre, Xa, Xb, G, raw, rotbuf, res_stage, desk_stage, conv_tmp;
  // Y tiling (cdx_RL_tiled): the whole raw stack, one tile, the stitched
  // output and its blend weights
  DevBuf<unsigned short> tile_raw, tile_in;
  DevBuf<float> tile_out;
  DevBuf<unsigned char> tile_weight;
  DevBuf<float2> S;
  DevBuf<double> partials, stat_d;
  DevBuf<unsigned> stat_u;
  DevBuf<float> lam;
  // acceleration factors of the last call, per iteration (cdx_lambda_trace)
  DevBuf<float> lam_hist;
  int lam_hist_n = 0;
  // convergence norms of the last call, per iteration (cdx_change_trace)
  DevBuf<double> chg_hist, chg_part;
  int chg_hist_n = 0;
  cudaStream_t stream = nullptr;
  long long launches = 0;
  // acceleration-factor scratch (per-block partials and the last-block ticket)
  DevBuf<double> acc_part;
  DevBuf<unsigned> acc_cnt;
  // camcor context
  int cc_nx = 0, cc_ny = 0, cc_nz = 0;
  DevBuf<float> cc_param;
  DevBuf<unsigned short> cc_in, cc_out;
};

static Session g_s;
static std::mutex g_mu;

// Optional per-pass timing with CUDA events recorded on the launch stream
// (cdx_profile_enable / cdx_profile_read).  Pass p of an iteration is timed
// between the events before and after its launch.
constexpr int kPasses = 9;
static const char* kPassNames[kPasses] = {"x_fwd_predict", "y_fwd",       "z_otf",
                                          "y_inv",         "x_ratio_fwd", "y_fwd2",
                                          "z_otf_conj",    "y_inv2",      "x_inv_update"};
struct Profiler {
  bool on = false;
  std::vector<cudaEvent_t> ev;  // 10 events per recorded iteration
  int used = 0;
  double pass_ms[kPasses] = {0};
  long long pass_n[kPasses] = {0};
  double iter_ms = 0;
  long long iter_n = 0;
};
static Profiler g_prof;

static cudaEvent_t prof_event() {
  Profiler& P = g_prof;
  if (P.used == (int)P.ev.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    P.ev.push_back(e);
  }
  return P.ev[P.used++];
}

// Fold the recorded events into the accumulators (synchronises).
static void prof_collect() {
  Profiler& P = g_prof;
  if (P.used < 10) {
    P.used = 0;
    return;
  }
  cudaEventSynchronize(P.ev[P.used - 1]);
  for (int base = 0; base + 10 <= P.used; base += 10) {
    for (int p = 0; p < kPasses; ++p) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, P.ev[base + p], P.ev[base + p + 1]) == cudaSuccess) {
        P.pass_ms[p] += ms;
        P.pass_n[p] += 1;
      }
    }
    float it = 0.f;
    if (cudaEventElapsedTime(&it, P.ev[base], P.ev[base + kPasses]) == cudaSuccess) {
      P.iter_ms += it;
      P.iter_n += 1;
    }
  }
  P.used = 0;
}

static void release_all(Session& s) {
  s.plan.release();
  s.raw_otf.release();
  s.u16in.release();
  s.pre.release();
  s.Xa.release();
  s.Xb.release();
  s.G.release();
  s.raw.release();
  s.rotbuf.release();
  s.res_stage.release();
  s.desk_stage.release();
  s.conv_tmp.release();
  s.tile_raw.release();
  s.tile_in.release();
  s.tile_out.release();
  s.tile_weight.release();
  s.S.release();
  s.partials.release();
  s.stat_d.release();
  s.stat_u.release();
  s.lam.release();
  s.lam_hist.release();
  s.lam_hist_n = 0;
  s.chg_hist.release();
  s.chg_part.release();
  s.chg_hist_n = 0;
  s.cc_param.release();
  s.cc_in.release();
  s.cc_out.release();
  s.acc_part.release();
  s.acc_cnt.release();
  if (s.stream) cudaStreamDestroy(s.stream);
  s.stream = nullptr;
}

static int ensure_stream(Session& s) {
  if (!s.stream) CDX_CHECK(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
  return 0;
}

// OTF description shared by the session and the batch stacks: the raw table
// on the device, its dimensions and k-steps (determine_OTF_dimensions,
// RL-Biggs-Andrews.cpp:506-529; dk values of RL_interface_init 576-590).
struct OtfSpec {
  RawOtfDims od{};
  float dkx_otf = 0, dky_otf = 0, dkz_otf = 0;
  const float2* raw_otf = nullptr;
};

// OTF dimensions and k-steps from a table of w x h x d floats (width 2*nz_otf
// for radial tables); false when the table is too small.
static bool otf_spec_dims(int w, int h, int d, float dr_psf, float dz_psf, OtfSpec& o) {
  unsigned nx_otf, ny_otf, nz_otf;
  if (d > 1) {
    nx_otf = w / 2;
    ny_otf = h;
    nz_otf = d;
  } else {
    nx_otf = h;
    ny_otf = 1;
    nz_otf = w / 2;
  }
  if (nx_otf < 2 || nz_otf < 1) return false;
  o.dkx_otf = 1 / ((nx_otf - 1) * 2 * dr_psf);
  o.dky_otf = ny_otf > 1 ? 1 / (ny_otf * dr_psf) : o.dkx_otf;
  o.dkz_otf = 1 / (nz_otf * dz_psf);
  o.od.nx_otf = nx_otf;
  o.od.ny_otf = ny_otf;
  o.od.nz_otf = nz_otf;
  return true;
}

// OTF table of a plan from the raw table o.raw_otf: the kz-resampled radial
// table (scaled by 1/N) or, for 3D OTF files, the full spectrum-layout array.
static int fill_otf(GridPlan& p, float dr, float dz, const OtfSpec& o, cudaStream_t st) {
  const int gx = p.g.nx, gy = p.g.ny, gz = p.g.nz;
  const float dkx = 1.0 / (dr * (unsigned)gx);
  const float dky = 1.0 / (dr * (unsigned)gy);
  const float dkz = 1.0 / (dz * (unsigned)gz);
  RawOtfDims od = o.od;
  od.kxscale = dkx / o.dkx_otf;
  od.kyscale = dky / o.dky_otf;
  od.kzscale = dkz / o.dkz_otf;
  const float scale = (float)(1.0 / ((double)gx * gy * gz));
  p.otf.nr = od.nx_otf;
  p.otf.kxscale = od.kxscale;
  p.otf.kyscale = od.kyscale;
  p.otf.tz = nullptr;
  p.otf.full = nullptr;
  int rc;
  if (od.ny_otf == 1) {
    p.otf.mode = 0;
    if ((rc = p.tz.ensure((size_t)od.nx_otf * gz))) return rc;
    if ((rc = launch_otf_tz(p.g, o.raw_otf, od, p.tz.p, scale, st))) return rc;
    p.otf.tz = p.tz.p;
  } else {
    p.otf.mode = 1;
    if ((rc = p.full.ensure((size_t)p.g.spec_elems()))) return rc;
    if ((rc = launch_otf_full(p.g, o.raw_otf, od, p.full.p, scale, st))) return rc;
    p.otf.full = p.full.p;
  }
  p.valid = true;
  return 0;
}

// Build FFT plans and the OTF table for a decon grid (gx, gy, gz).  The OTF
// k-scales follow RL_interface_init (RL-Biggs-Andrews.cpp:634-642): dk =
// 1/(pixel * size) per axis divided by the OTF's dk.  Enqueued on st; the
// caller synchronises before the plan is used from another stream.
static int build_plan(GridPlan& p, int gx, int gy, int gz, float dr, float dz, const OtfSpec& o,
                      cudaStream_t st) {
  p.release();
  if (!fft_len_supported(gx) || !fft_len_supported(gy) || !fft_len_supported(gz)) {
    set_error("plan", "decon grid size is not a product of 2, 3, 5 and 7");
    return cudaErrorInvalidValue;
  }
  p.g = make_geom(gx, gy, gz);
  int rc;
  if ((rc = fft_len_init(p.fx, gx))) return rc;
  if ((rc = fft_len_init(p.fy, gy))) return rc;
  if ((rc = fft_len_init(p.fz, gz))) return rc;
  return fill_otf(p, dr, dz, o, st);
}

// Session plan for a decon grid (reused while the grid does not change).
static int ensure_plan(Session& s, int gx, int gy, int gz) {
  GridPlan& p = s.plan;
  if (p.valid && p.g.nx == gx && p.g.ny == gy && p.g.nz == gz) return 0;
  OtfSpec o;
  o.od = s.od;
  o.dkx_otf = s.dkx_otf;
  o.dky_otf = s.dky_otf;
  o.dkz_otf = s.dkz_otf;
  o.raw_otf = s.raw_otf.p;
  int rc;
  if ((rc = build_plan(p, gx, gy, gz, s.dr, s.dz, o, s.stream))) return rc;
  CDX_CHECK(cudaStreamSynchronize(s.stream));
  return 0;
}

static int ensure_grid_buffers(Session& s, const Geom& g) {
  const size_t n = (size_t)g.nvox();
  int rc;
  if ((rc = s.Xa.ensure(n)) || (rc = s.Xb.ensure(n)) || (rc = s.G.ensure(n)) ||
      (rc = s.raw.ensure(n)) || (rc = s.S.ensure((size_t)g.spec_elems())))
    return rc;
  const int nblk = x_pass_blocks(g);
  if ((rc = s.partials.ensure(2 * (size_t)nblk)) || (rc = s.lam.ensure(2))) return rc;
  CDX_CHECK(cudaMemsetAsync(s.lam.p, 0, 2 * sizeof(float), s.stream));
  return 0;
}

// ---------------------------------------------------------------- RL loop
// The iteration loop of RichardsonLucy_GPU (RL-Biggs-Andrews.cpp:282-367) on
// the grid of s.plan, starting from X0 in s.Xa with raw in s.raw.  Returns
// the buffer that holds the final estimate.
// Device buffers of one RL loop: estimates (X0 in Xa), raw, G, spectrum,
// dot-product partials (16 bytes per x-pass block) and the two lambda slots.
struct LoopBufs {
  float* Xa;
  float* Xb;
  float* G;
  float* raw;
  float2* S;
  double* partials;
  float* lam;
  int max_blocks;
};

static int rl_loop(const GridPlan& p, const LoopBufs& b, int nIter, cudaStream_t st, bool prof,
                   float** final_x, long long* launches, float* lam_hist = nullptr,
                   int hist_n = 0, double* chg_hist = nullptr, int chg_n = 0,
                   double* chg_part = nullptr) {
  const Geom& g = p.g;
  RLWork w;
  w.partials = b.partials;
  w.lam = b.lam;
  w.max_blocks = b.max_blocks;
  const float eps = 1.1920928955078125e-07f;  // std::numeric_limits<float>::epsilon()
  float* X = b.Xa;
  float* Xm1 = b.Xb;
  int rc;
  auto mark = [&]() {
    if (prof) {
      cudaEvent_t e = prof_event();
      if (e) cudaEventRecord(e, st);
    }
  };
  for (int k = 0; k < nIter; ++k) {
    const int predict = k > 1;
    float* lam_k = b.lam + (k & 1);
    float* lam_n = b.lam + ((k + 1) & 1);
    mark();
    if ((rc = launch_x_fwd(g, p.fx, X, Xm1, lam_k, predict, b.S, st))) return rc;
    mark();
    if ((rc = launch_y_pass(g, p.fy, b.S, false, st))) return rc;
    mark();
    if ((rc = launch_z_pass(g, p.fz, b.S, p.otf, false, st))) return rc;
    mark();
    if ((rc = launch_y_pass(g, p.fy, b.S, true, st))) return rc;
    mark();
    if ((rc = launch_x_inv_ratio_fwd(g, p.fx, b.S, b.raw, eps, st))) return rc;
    mark();
    if ((rc = launch_y_pass(g, p.fy, b.S, false, st))) return rc;
    mark();
    if ((rc = launch_z_pass(g, p.fz, b.S, p.otf, true, st))) return rc;
    mark();
    if ((rc = launch_y_pass(g, p.fy, b.S, true, st))) return rc;
    mark();
    // x_fwd wrote the prediction Y over Xm1 when predicting (else Y = X);
    // the new estimate replaces it in place
    const float* Y = predict ? Xm1 : X;
    if ((rc = launch_x_inv_update(g, p.fx, b.S, Y, Xm1, b.G, k >= 1, w, lam_n, eps, st)))
      return rc;
    mark();
    // trace: the factor iteration k+1 uses (computed from G_k and G_{k-1})
    if (lam_hist && k >= 1 && k + 1 < hist_n)
      CDX_CHECK(cudaMemcpyAsync(lam_hist + k + 1, lam_n, sizeof(float), cudaMemcpyDeviceToDevice,
                                st));
    if (prof && g_prof.used >= 10 * 64) prof_collect();
    *launches += k >= 1 ? 10 : 9;  // the update pass adds the lambda kernel
    float* t = X;
    X = Xm1;
    Xm1 = t;
    // trace: X holds X_{k+1} and Xm1 X_k until the next forward pass
    if (chg_hist && k < chg_n) {
      if ((rc = launch_change_norm(X, Xm1, g.nvox(), chg_part, chg_hist + k, st))) return rc;
      *launches += 2;
    }
  }
  *final_x = X;
  return 0;
}

static int rl_iterations(Session& s, int nIter, float** final_x) {
  const LoopBufs b{s.Xa.p, s.Xb.p, s.G.p, s.raw.p, s.S.p, s.partials.p, s.lam.p,
                   (int)(s.partials.n / 2)};
  float* hist = nullptr;
  if (s.lam_hist_n > 0 && s.lam_hist.p) {
    CDX_CHECK(cudaMemsetAsync(s.lam_hist.p, 0, sizeof(float) * s.lam_hist_n, s.stream));
    hist = s.lam_hist.p;
  }
  double* chg = nullptr;
  if (s.chg_hist_n > 0 && s.chg_hist.p && s.chg_part.p) {
    CDX_CHECK(cudaMemsetAsync(s.chg_hist.p, 0, sizeof(double) * s.chg_hist_n, s.stream));
    chg = s.chg_hist.p;
  }
  return rl_loop(s.plan, b, nIter, s.stream, g_prof.on, final_x, &s.launches, hist,
                 s.lam_hist_n, chg, s.chg_hist_n, s.chg_part.p);
}

struct RLArgs {
  int nx, ny, nz;  // caller's raw sizes
  float background;
  bool bDoRescale, bSaveDeskewedRaw;
  int nIters, extraShift, napodize, nZblend;
  float padVal;
  bool bDupRevStack, bSkewedDecon;
};

static void rot_out_dims(const Session& s, int nx, int nz, int* nx_r, int* nz_r) {
  const float* p = s.rot;
  // RichardsonLucy_GPU (RL-Biggs-Andrews.cpp:410-411)
  *nz_r = (int)(nz * p[3] / p[0]);
  *nx_r = (int)(nx * p[3] + nz * p[2] * p[2] / fabsf(p[1]));
}

// The body of RichardsonLucy_GPU (RL-Biggs-Andrews.cpp:56-450) on device
// memory.  d_u16 holds the caller's (nx, ny, nz) raw stack.  On return
// *out_ptr / *out_dims describe the device buffer with the result.
static int rl_pipeline(Session& s, const unsigned short* d_u16, const RLArgs& a, float* d_deskewed,
                       const float** out_ptr, int out_dims[3]) {
  int rc;
  const int nx0 = s.output_nx, ny = s.output_ny, nz0 = s.output_nz;
  if (a.nx < nx0 || a.ny < ny || a.nz < nz0) {
    set_error("RL_interface", "input stack smaller than the RL_interface_init sizes");
    return cudaErrorInvalidValue;
  }
  const size_t n0 = (size_t)nx0 * ny * nz0;
  if ((rc = s.pre.ensure(n0))) return rc;
  const bool save_desk = a.bSaveDeskewedRaw && fabs(s.deskewFactor) > 0.0;
  const bool pre = a.nIters > 0 || save_desk || s.has_rot;
  const bool fuse_bg = pre && a.napodize <= 0;
  if ((rc = launch_u16_to_f32_crop(d_u16, a.nx, a.ny, nx0, ny, nz0, s.pre.p, a.background,
                                   fuse_bg ? 1 : 0, s.stream)))
    return rc;
  ++s.launches;
  const float* cur = s.pre.p;
  int nx = nx0, nz = nz0;
  bool cur_is_x = false;  // whether cur already lives in Xa
  if (pre) {
    if (!fuse_bg) {
      if ((rc = launch_apodize(s.pre.p, nx0, ny, nz0, a.napodize, s.stream))) return rc;
      if ((rc = launch_bgsub(s.pre.p, (long long)n0, a.background, s.stream))) return rc;
      s.launches += 3;
    }
    if (a.bDoRescale) {
      // meanAboveBackground_GPU + rescale (RL-Biggs-Andrews.cpp:124-134)
      if ((rc = s.stat_d.ensure(1216 + 2)) || (rc = s.stat_u.ensure(1216 + 2))) return rc;
      double intensity = 0.0;
      if ((rc = mean_above_background(s.pre.p, (long long)n0, s.stat_d.p, s.stat_u.p, &intensity,
                                      s.stream)))
        return rc;
      s.launches += 4;
      if (s.bFirstTime) {
        s.intensity_overall0 = intensity;
        s.bFirstTime = false;
      } else {
        const float ratio = s.intensity_overall0 / intensity;
        if ((rc = launch_scale(s.pre.p, (long long)n0, (double)ratio, s.stream))) return rc;
        ++s.launches;
      }
    }
    const bool deskew_now =
        (!a.bSkewedDecon || (save_desk && a.nIters == 0)) && fabs(s.deskewFactor) > 0.0;
    if (deskew_now) {
      nx = s.deskewedXdim;
      const size_t nd = (size_t)nx * ny * nz0;
      if ((rc = s.Xa.ensure(nd))) return rc;
      if ((rc = launch_deskew(s.pre.p, nx0, ny, nz0, s.deskewFactor, s.Xa.p, nx, a.extraShift,
                              a.padVal, s.stream)))
        return rc;
      ++s.launches;
      cur = s.Xa.p;
      cur_is_x = true;
      if (save_desk && d_deskewed)
        CDX_CHECK(cudaMemcpyAsync(d_deskewed, cur, nd * sizeof(float), cudaMemcpyDeviceToDevice,
                                  s.stream));
      if (save_desk && a.nIters == 0) {
        // The reference returns an unfilled buffer here; the deskewed stack is
        // returned instead.
        *out_ptr = cur;
        out_dims[0] = nx;
        out_dims[1] = ny;
        out_dims[2] = nz;
        return 0;
      }
    }
    if (a.nZblend > 0) {
      if (!cur_is_x) {
        if ((rc = s.Xa.ensure(n0))) return rc;
        CDX_CHECK(cudaMemcpyAsync(s.Xa.p, cur, n0 * sizeof(float), cudaMemcpyDeviceToDevice,
                                  s.stream));
        cur = s.Xa.p;
        cur_is_x = true;
      }
      if ((rc = launch_zblend(s.Xa.p, nx, ny, nz, a.nZblend, s.stream))) return rc;
      ++s.launches;
    }
    if (a.bDupRevStack) {
      // mirrored stack of 2*nz slices (RL-Biggs-Andrews.cpp:193-205); the FFT
      // grid follows the doubled stack
      const size_t nv = (size_t)nx * ny * nz;
      if ((rc = s.raw.ensure(2 * nv))) return rc;
      CDX_CHECK(cudaMemcpyAsync(s.raw.p, cur, nv * sizeof(float), cudaMemcpyDeviceToDevice,
                                s.stream));
      if ((rc = launch_dup_rev(s.raw.p, nx, ny, nz, s.stream))) return rc;
      ++s.launches;
      if ((rc = s.Xa.ensure(2 * nv))) return rc;
      CDX_CHECK(cudaMemcpyAsync(s.Xa.p, s.raw.p, 2 * nv * sizeof(float), cudaMemcpyDeviceToDevice,
                                s.stream));
      cur = s.Xa.p;
      cur_is_x = true;
      nz *= 2;
    }
  }
  const float* X = cur;
  if (a.nIters > 0) {
    if ((rc = ensure_plan(s, nx, ny, nz))) return rc;
    if ((rc = ensure_grid_buffers(s, s.plan.g))) return rc;
    const size_t nv = (size_t)nx * ny * nz;
    if (cur != s.Xa.p)
      CDX_CHECK(cudaMemcpyAsync(s.Xa.p, cur, nv * sizeof(float), cudaMemcpyDeviceToDevice, s.stream));
    CDX_CHECK(cudaMemcpyAsync(s.raw.p, s.Xa.p, nv * sizeof(float), cudaMemcpyDeviceToDevice,
                              s.stream));
    float* fx = nullptr;
    if ((rc = rl_iterations(s, a.nIters, &fx))) return rc;
    X = fx;
  }
  if (a.bDupRevStack && pre) nz /= 2;
  if (a.bSkewedDecon && fabs(s.deskewFactor) > 0.0) {
    // deskew after decon (RL-Biggs-Andrews.cpp:383-401; padVal defaults to 0)
    const int nxd = s.deskewedXdim;
    if ((rc = s.desk_stage.ensure((size_t)nxd * ny * nz))) return rc;
    if ((rc = launch_deskew(X, nx, ny, nz, s.deskewFactor, s.desk_stage.p, nxd, a.extraShift, 0.f,
                            s.stream)))
      return rc;
    ++s.launches;
    X = s.desk_stage.p;
    nx = nxd;
  }
  if (s.has_rot) {
    int nxr, nzr;
    rot_out_dims(s, nx, nz, &nxr, &nzr);
    if (nxr <= 0 || nzr <= 0) {
      set_error("RL_interface", "rotation gives an empty output");
      return cudaErrorInvalidValue;
    }
    if ((rc = s.rotbuf.ensure((size_t)nxr * ny * nzr))) return rc;
    if ((rc = launch_rotate(X, nx, ny, nz, s.rot, s.rotbuf.p, nxr, nzr, s.stream))) return rc;
    ++s.launches;
    X = s.rotbuf.p;
    nx = nxr;
    nz = nzr;
  }
  *out_ptr = X;
  out_dims[0] = nx;
  out_dims[1] = ny;
  out_dims[2] = nz;
  return 0;
}

static unsigned reported_nx(const Session& s) {
  if (s.has_rot) {
    const float* p = s.rot;
    int nx_afterRot = s.deskewedXdim * p[3] + s.output_nz * p[2] * p[2] / p[1];
    return nx_afterRot;
  }
  return s.deskewedXdim;
}

static unsigned reported_nz(const Session& s) {
  if (s.has_rot) {
    const float* p = s.rot;
    int nz_afterRot = s.output_nz * p[3] / p[0];
    return nz_afterRot;
  }
  return s.output_nz;
}

static int init_session(Session& s, int nx, int ny, int nz, float dr, float dz, float dr_psf,
                        float dz_psf, float deskewAngle, float rotationAngle, int outputWidth,
                        bool bSkewedDecon, const char* otf_file) {
  s.plan.release();
  s.inited = false;
  if (nx < 2 || ny < 2 || nz < 2) {
    set_error("RL_interface_init", "image sizes must be at least 2");
    return cudaErrorInvalidValue;
  }
  // RL-Biggs-Andrews.cpp:543-564
  s.bCrop = false;
  s.output_ny = find_optimal_dimension(ny);
  if (s.output_ny != (unsigned)ny) s.bCrop = true;
  s.output_nz = find_optimal_dimension(nz);
  if (s.output_nz != (unsigned)nz) s.bCrop = true;
  s.output_nx = nx;
  if (!(fabs(deskewAngle) > 0.0)) {
    s.output_nx = find_optimal_dimension(nx);
    if (s.output_nx != (unsigned)nx) s.bCrop = true;
  }
  // OTF (RL-Biggs-Andrews.cpp:566-590)
  HostImage otf;
  std::string err;
  if (!load_image_file(otf_file, otf, err)) {
    set_error("RL_interface_init: OTF", err.c_str());
    return cudaErrorInvalidValue;
  }
  if (bSkewedDecon) dz_psf *= fabs(sin(deskewAngle * M_PI / 180.));
  OtfSpec os;
  if (!otf_spec_dims(otf.w, otf.h, otf.d, dr_psf, dz_psf, os)) {
    set_error("RL_interface_init", "OTF too small");
    return cudaErrorInvalidValue;
  }
  s.dkx_otf = os.dkx_otf;
  s.dky_otf = os.dky_otf;
  s.dkz_otf = os.dkz_otf;
  s.od = os.od;
  const unsigned nx_otf = os.od.nx_otf, ny_otf = os.od.ny_otf, nz_otf = os.od.nz_otf;
  int rc;
  if ((rc = ensure_stream(s))) return rc;
  const size_t notf = (size_t)nx_otf * ny_otf * nz_otf;
  if ((rc = s.raw_otf.ensure(notf))) return rc;
  CDX_CHECK(cudaMemcpy(s.raw_otf.p, otf.data.data(), notf * sizeof(float2), cudaMemcpyHostToDevice));
  // deskew geometry (RL-Biggs-Andrews.cpp:592-607)
  s.deskewFactor = 0.;
  s.deskewedXdim = s.output_nx;
  if (fabs(deskewAngle) > 0.0) {
    if (deskewAngle < 0) deskewAngle += 180.;
    s.deskewFactor = cos(deskewAngle * M_PI / 180.) * dz / dr;
    if (outputWidth == 0)
      s.deskewedXdim += floor(s.output_nz * dz * fabs(cos(deskewAngle * M_PI / 180.)) / dr);
    else
      s.deskewedXdim = outputWidth;
    s.deskewedXdim = find_optimal_dimension(s.deskewedXdim);
    dz *= fabs(sin(deskewAngle * M_PI / 180.));
  }
  // rotation matrix (RL-Biggs-Andrews.cpp:609-619); the float overloads of
  // cos/sin are the ones the reference's C++ resolves to
  s.has_rot = false;
  if (fabs(rotationAngle) > 0.0) {
    s.has_rot = true;
    rotationAngle *= M_PI / 180;
    const float stretch = dr / dz;
    s.rot[0] = cosf(rotationAngle) * stretch;
    s.rot[1] = sinf(rotationAngle) * stretch;
    s.rot[2] = -sinf(rotationAngle);
    s.rot[3] = cosf(rotationAngle);
  }
  s.dr = dr;
  s.dz = dz;
  if (s.output_nx < 2 || s.output_ny < 2 || s.output_nz < 2 || s.deskewedXdim < 2) {
    set_error("RL_interface_init", "no FFT-friendly size below the input size");
    return cudaErrorInvalidValue;
  }
  // decon grid: deskewed width unless the decon runs on the skewed stack
  const int gx = (bSkewedDecon && fabs(deskewAngle) > 0.0) ? (int)s.output_nx : (int)s.deskewedXdim;
  if ((rc = ensure_plan(s, gx, s.output_ny, s.output_nz))) return rc;
  s.inited = true;
  return 0;
}

// ---------------------------------------------------------------- batch
// Independent stacks (timepoints, channels, tiles) of any shapes, each with
// its own OTF.  Per stack: plans, OTF table and work buffers, kept across
// calls.  The iterations of all stacks are captured once into a CUDA graph:
// the stacks, largest first, each go to the least-loaded of K streams forked
// from the origin stream, so the graph holds K independent chains of about
// equal work and small stacks run concurrently.  K is 2 by default
// (cdx_batch_set_streams): on the 64-stack uneven batch, device-resident,
// 1, 2, 3, 4, 6, 8 and 16 streams gave 42.7, 44.6, 43.9, 42.6, 40.2, 39.9 and
// 39.9 G voxel-iter/s (more concurrent stacks share the L2 that holds a
// stack's spectrum between its passes).  The host batch's transfers run on
// an upload and a download stream of their own, so they overlap the chains
// whatever K is: 1, 2, 3, 4 and 6 streams gave 42.7, 44.8, 44.0, 42.6 and
// 39.2 G end to end.
constexpr int kBatchStreams = 16;
static int g_batch_streams[2] = {2, 2};  // device batch, host batch

struct BatchStack {
  int nx = 0, ny = 0, nz = 0;  // caller's stack
  int gx = 0, gy = 0, gz = 0;  // decon grid
  int otf_w = 0, otf_h = 0;
  float dr = 0, dz = 0, dr_psf = 0, dz_psf = 0;
  OtfSpec os;
  GridPlan plan;
  DevBuf<float2> raw_otf;
  DevBuf<float> Xa, Xb, G, raw;
  DevBuf<float2> S;
  DevBuf<double> partials;
  DevBuf<float> lam;
  float* final_x = nullptr;
  // host mode (cdx_RL_batch_host): the stack's device copy of the caller's
  // page-locked raw buffer, and what the captured graph baked in
  DevBuf<unsigned short> u16;
  const unsigned short* h_raw = nullptr;
  float* h_result = nullptr;
  float background = 0.f;
  void release() {
    plan.release();
    raw_otf.release();
    u16.release();
    h_raw = nullptr;
    h_result = nullptr;
    Xa.release();
    Xb.release();
    G.release();
    raw.release();
    S.release();
    partials.release();
    lam.release();
  }
};

struct Batch {
  std::vector<BatchStack> st;
  cudaStream_t origin = nullptr;
  cudaStream_t fan[kBatchStreams] = {};
  cudaEvent_t ev_in = nullptr, ev_out = nullptr, ev_fork = nullptr;
  cudaEvent_t ev_join[kBatchStreams] = {};
  // host batch: uploads and downloads run on streams of their own
  cudaStream_t up = nullptr, dn = nullptr;
  cudaEvent_t ev_up = nullptr, ev_dn = nullptr, ev_jup = nullptr, ev_jdn = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_iters = -1;
  int graph_form = -1;  // DFT form the graph's kernels were captured with
  int graph_host = -1;  // 1 when the graph carries the host transfers
  int graph_streams = -1;  // streams the graph's chains were spread over
  long long graph_launches = 0;
  long long last_launches = 0;
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    graph_iters = -1;
    graph_form = -1;
    graph_host = -1;
    graph_streams = -1;
  }
  void release() {
    drop_graph();
    for (auto& b : st) b.release();
    st.clear();
    for (int i = 0; i < kBatchStreams; ++i) {
      if (fan[i]) cudaStreamDestroy(fan[i]);
      if (ev_join[i]) cudaEventDestroy(ev_join[i]);
      fan[i] = nullptr;
      ev_join[i] = nullptr;
    }
    if (origin) cudaStreamDestroy(origin);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (ev_fork) cudaEventDestroy(ev_fork);
    origin = nullptr;
    ev_in = ev_out = ev_fork = nullptr;
    for (cudaStream_t* q : {&up, &dn}) {
      if (*q) cudaStreamDestroy(*q);
      *q = nullptr;
    }
    for (cudaEvent_t* ev : {&ev_up, &ev_dn, &ev_jup, &ev_jdn}) {
      if (*ev) cudaEventDestroy(*ev);
      *ev = nullptr;
    }
  }
};
static Batch g_b;

static int batch_streams(Batch& b) {
  if (b.origin) return 0;
  CDX_CHECK(cudaStreamCreateWithFlags(&b.origin, cudaStreamNonBlocking));
  CDX_CHECK(cudaEventCreateWithFlags(&b.ev_in, cudaEventDisableTiming));
  CDX_CHECK(cudaEventCreateWithFlags(&b.ev_out, cudaEventDisableTiming));
  CDX_CHECK(cudaEventCreateWithFlags(&b.ev_fork, cudaEventDisableTiming));
  for (int i = 0; i < kBatchStreams; ++i) {
    CDX_CHECK(cudaStreamCreateWithFlags(&b.fan[i], cudaStreamNonBlocking));
    CDX_CHECK(cudaEventCreateWithFlags(&b.ev_join[i], cudaEventDisableTiming));
  }
  CDX_CHECK(cudaStreamCreateWithFlags(&b.up, cudaStreamNonBlocking));
  CDX_CHECK(cudaStreamCreateWithFlags(&b.dn, cudaStreamNonBlocking));
  for (cudaEvent_t* ev : {&b.ev_up, &b.ev_dn, &b.ev_jup, &b.ev_jdn})
    CDX_CHECK(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  return 0;
}

// (Re)build the state of one stack for the caller's description; *changed
// tells whether its shape-dependent state (and so the graph) changed.
static int batch_setup_stack(BatchStack& b, const cdx_batch_stack& d, bool* changed) {
  *changed = true;
  if (d.nx < 2 || d.ny < 2 || d.nz < 2) {
    set_error("cdx_RL_batch_device", "stack sizes must be at least 2");
    return cudaErrorInvalidValue;
  }
  const int gx = (int)find_optimal_dimension(d.nx), gy = (int)find_optimal_dimension(d.ny),
            gz = (int)find_optimal_dimension(d.nz);
  const bool same = b.plan.valid && b.nx == d.nx && b.ny == d.ny && b.nz == d.nz &&
                    b.otf_w == d.otf_w && b.otf_h == d.otf_h && b.dr == d.dr && b.dz == d.dz &&
                    b.dr_psf == d.dr_psf && b.dz_psf == d.dz_psf;
  *changed = !same;
  if (same) return 0;
  b.release();
  if (gx < 2 || gy < 2 || gz < 2) {
    set_error("cdx_RL_batch_device", "no FFT-friendly size below the stack size");
    return cudaErrorInvalidValue;
  }
  if (d.otf_w < 2 || d.otf_h < 2 || (d.otf_w & 1) ||
      !otf_spec_dims(d.otf_w, d.otf_h, 1, d.dr_psf, d.dz_psf, b.os)) {
    set_error("cdx_RL_batch_device", "OTF table too small or of odd width");
    return cudaErrorInvalidValue;
  }
  b.nx = d.nx;
  b.ny = d.ny;
  b.nz = d.nz;
  b.gx = gx;
  b.gy = gy;
  b.gz = gz;
  b.otf_w = d.otf_w;
  b.otf_h = d.otf_h;
  b.dr = d.dr;
  b.dz = d.dz;
  b.dr_psf = d.dr_psf;
  b.dz_psf = d.dz_psf;
  const size_t n = (size_t)gx * gy * gz;
  const Geom g = make_geom(gx, gy, gz);
  int rc;
  if ((rc = b.raw_otf.ensure((size_t)d.otf_w * d.otf_h / 2)) || (rc = b.Xa.ensure(n)) ||
      (rc = b.Xb.ensure(n)) || (rc = b.G.ensure(n)) || (rc = b.raw.ensure(n)) ||
      (rc = b.S.ensure((size_t)g.spec_elems())) ||
      (rc = b.partials.ensure(2 * (size_t)x_pass_blocks(g))) ||
      (rc = b.lam.ensure(2)))
    return rc;
  b.os.raw_otf = b.raw_otf.p;
  return 0;
}

// Capture the iterations of every stack into b.exec; with host, each
// stack's chain also conditions its raw stack first, after its upload on
// the upload stream, and its result is downloaded on the download stream
// after the chain ends, so the transfers overlap the chains.
static int batch_capture(Batch& b, int nIters, bool host) {
  b.drop_graph();
  std::vector<int> order(b.st.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::sort(order.begin(), order.end(), [&](int a, int c) {
    return (long long)b.st[a].gx * b.st[a].gy * b.st[a].gz >
           (long long)b.st[c].gx * b.st[c].gy * b.st[c].gz;
  });
  const int K = std::min<int>(g_batch_streams[host ? 1 : 0], (int)b.st.size());
  CDX_CHECK(cudaStreamBeginCapture(b.origin, cudaStreamCaptureModeRelaxed));
  int rc = 0;
  long long launches = 0;
  cudaError_t e = cudaEventRecord(b.ev_fork, b.origin);
  for (int k = 0; k < K && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b.fan[k], b.ev_fork, 0);
  if (host && e == cudaSuccess) e = cudaStreamWaitEvent(b.up, b.ev_fork, 0);
  if (host && e == cudaSuccess) e = cudaStreamWaitEvent(b.dn, b.ev_fork, 0);
  if (e != cudaSuccess) {
    set_cuda_error("batch capture", e);
    rc = e;
  }
  // largest stack first onto the least-loaded stream (voxels so far): the
  // streams' chains then end together (dealing round-robin left the
  // busiest stream 23% above the mean on a 64-stack uneven batch)
  std::vector<long long> load(K, 0);
  for (size_t j = 0; j < order.size() && !rc; ++j) {
    BatchStack& t = b.st[order[j]];
    const size_t n = (size_t)t.gx * t.gy * t.gz;
    const int ks = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[ks] += (long long)n;
    cudaStream_t s = b.fan[ks];
    if (host) {
      // the stack's upload runs on the upload stream (all uploads back to
      // back, in the order the chains need them); its conditioning heads
      // its chain once the upload is in
      const size_t nin = (size_t)t.nx * t.ny * t.nz;
      if ((e = cudaMemcpyAsync(t.u16.p, t.h_raw, nin * sizeof(unsigned short),
                               cudaMemcpyHostToDevice, b.up)) != cudaSuccess ||
          (e = cudaEventRecord(b.ev_up, b.up)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(s, b.ev_up, 0)) != cudaSuccess) {
        set_cuda_error("batch capture", e);
        rc = e;
        break;
      }
      if ((rc = launch_u16_to_f32_crop(t.u16.p, t.nx, t.ny, t.gx, t.gy, t.gz, t.Xa.p,
                                       t.background, 1, s)))
        break;
      ++launches;
    }
    if ((e = cudaMemsetAsync(t.lam.p, 0, 2 * sizeof(float), s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(t.raw.p, t.Xa.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess) {
      set_cuda_error("batch capture", e);
      rc = e;
      break;
    }
    const LoopBufs lb{t.Xa.p, t.Xb.p, t.G.p, t.raw.p, t.S.p, t.partials.p, t.lam.p,
                      (int)(t.partials.n / 2)};
    rc = rl_loop(t.plan, lb, nIters, s, false, &t.final_x, &launches);
    if (!rc && host) {
      // and its download, on the download stream, follows the chain's end
      // (nIters == 0: the conditioned stack)
      const float* src = nIters > 0 ? t.final_x : t.Xa.p;
      if ((e = cudaEventRecord(b.ev_dn, s)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(b.dn, b.ev_dn, 0)) != cudaSuccess ||
          (e = cudaMemcpyAsync(t.h_result, src, n * sizeof(float), cudaMemcpyDeviceToHost,
                               b.dn)) != cudaSuccess) {
        set_cuda_error("batch capture", e);
        rc = e;
      }
    }
  }
  for (int k = 0; k < K && !rc; ++k) {
    if ((e = cudaEventRecord(b.ev_join[k], b.fan[k])) != cudaSuccess ||
        (e = cudaStreamWaitEvent(b.origin, b.ev_join[k], 0)) != cudaSuccess) {
      set_cuda_error("batch capture", e);
      rc = e;
    }
  }
  if (host && !rc) {
    if ((e = cudaEventRecord(b.ev_jup, b.up)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(b.origin, b.ev_jup, 0)) != cudaSuccess ||
        (e = cudaEventRecord(b.ev_jdn, b.dn)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(b.origin, b.ev_jdn, 0)) != cudaSuccess) {
      set_cuda_error("batch capture", e);
      rc = e;
    }
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(b.origin, &graph);
  if (!rc && e != cudaSuccess) {
    set_cuda_error("batch capture", e);
    rc = e;
  }
  if (!rc) {
    e = cudaGraphInstantiate(&b.exec, graph, 0);
    if (e != cudaSuccess) {
      set_cuda_error("cudaGraphInstantiate", e);
      b.exec = nullptr;
      rc = e;
    }
  }
  if (graph) cudaGraphDestroy(graph);
  if (rc) {
    cudaGetLastError();
    return rc;
  }
  b.graph_iters = nIters;
  b.graph_form = dft_form();
  b.graph_host = host ? 1 : 0;
  b.graph_streams = g_batch_streams[host ? 1 : 0];
  b.graph_launches = launches;
  return 0;
}

// host: raw and result are page-locked host buffers (cdx_RL_batch_host).
static int batch_run(const cdx_batch_stack* stacks, int n, int nIters, cudaStream_t caller,
                     bool host) {
  Batch& b = g_b;
  if (!stacks || n < 1 || nIters < 0) {
    set_error("cdx_RL_batch_device", "need at least one stack and nIters >= 0");
    return cudaErrorInvalidValue;
  }
  for (int i = 0; i < n; ++i) {
    const cdx_batch_stack& d = stacks[i];
    if (!d.raw || !d.result || !d.otf) {
      set_error("cdx_RL_batch_device", "null raw, result or otf pointer");
      return cudaErrorInvalidValue;
    }
    if (d.nx < 2 || d.ny < 2 || d.nz < 2) {
      set_error("cdx_RL_batch_device", "stack sizes must be at least 2");
      return cudaErrorInvalidValue;
    }
    if (d.otf_w < 2 || d.otf_h < 2 || (d.otf_w & 1)) {
      set_error("cdx_RL_batch_device", "OTF table too small or of odd width");
      return cudaErrorInvalidValue;
    }
    if (!(d.dr > 0.f) || !(d.dz > 0.f) || !(d.dr_psf > 0.f) || !(d.dz_psf > 0.f)) {
      set_error("cdx_RL_batch_device", "pixel sizes must be positive");
      return cudaErrorInvalidValue;
    }
  }
  int rc;
  if ((rc = batch_streams(b))) return rc;
  bool changed = (int)b.st.size() != n;
  if (changed) {
    b.drop_graph();
    for (auto& t : b.st) t.release();
    b.st.clear();
    b.st.resize(n);
  }
  for (int i = 0; i < n; ++i) {
    bool c = false;
    if ((rc = batch_setup_stack(b.st[i], stacks[i], &c))) {
      b.drop_graph();
      b.st[i].release();
      return rc;
    }
    changed = changed || c;
  }
  if (changed) b.drop_graph();
  if (host) {
    // the graph bakes in the host buffers and backgrounds
    for (int i = 0; i < n; ++i) {
      BatchStack& t = b.st[i];
      const cdx_batch_stack& d = stacks[i];
      if ((rc = t.u16.ensure((size_t)d.nx * d.ny * d.nz))) return rc;
      if (t.h_raw != d.raw || t.h_result != d.result || t.background != d.background)
        b.drop_graph();
      t.h_raw = d.raw;
      t.h_result = d.result;
      t.background = d.background;
    }
  }
  // after the caller's queued work: the OTF tables, then (device buffers)
  // the cropped, background-subtracted stacks (into each stack's first
  // estimate)
  CDX_CHECK(cudaEventRecord(b.ev_in, caller));
  CDX_CHECK(cudaStreamWaitEvent(b.origin, b.ev_in, 0));
  long long launches = 0;
  for (int i = 0; i < n; ++i) {
    BatchStack& t = b.st[i];
    const cdx_batch_stack& d = stacks[i];
    CDX_CHECK(cudaMemcpyAsync(t.raw_otf.p, d.otf, sizeof(float) * (size_t)d.otf_w * d.otf_h,
                              cudaMemcpyHostToDevice, b.origin));
    if (!t.plan.valid) {
      if ((rc = build_plan(t.plan, t.gx, t.gy, t.gz, t.dr, t.dz, t.os, b.origin))) return rc;
    } else {
      if ((rc = fill_otf(t.plan, t.dr, t.dz, t.os, b.origin))) return rc;
    }
    launches += 1;
    if (host) continue;
    if ((rc = launch_u16_to_f32_crop(d.raw, d.nx, d.ny, t.gx, t.gy, t.gz, t.Xa.p, d.background, 1,
                                     b.origin)))
      return rc;
    launches += 1;
  }
  if (nIters > 0 || host) {
    if (!b.exec || b.graph_iters != nIters || b.graph_form != dft_form() ||
        b.graph_host != (host ? 1 : 0) || b.graph_streams != g_batch_streams[host ? 1 : 0]) {
      // the plans' tables were built on the origin stream
      CDX_CHECK(cudaStreamSynchronize(b.origin));
      if ((rc = batch_capture(b, nIters, host))) return rc;
    }
    CDX_CHECK(cudaGraphLaunch(b.exec, b.origin));
    launches += b.graph_launches;
  }
  if (host) {
    // the results are in the caller's host buffers when this returns
    CDX_CHECK(cudaStreamSynchronize(b.origin));
    b.last_launches = launches;
    return 0;
  }
  for (int i = 0; i < n; ++i) {
    BatchStack& t = b.st[i];
    const float* src = nIters > 0 ? t.final_x : t.Xa.p;
    CDX_CHECK(cudaMemcpyAsync(stacks[i].result, src, sizeof(float) * (size_t)t.gx * t.gy * t.gz,
                              cudaMemcpyDeviceToDevice, b.origin));
  }
  CDX_CHECK(cudaEventRecord(b.ev_out, b.origin));
  CDX_CHECK(cudaStreamWaitEvent(caller, b.ev_out, 0));
  b.last_launches = launches;
  return 0;
}

}  // namespace cdx

using namespace cdx;

extern "C" {

int RL_interface_init(int nx, int ny, int nz, float dr, float dz, float dr_psf, float dz_psf,
                      float deskewAngle, float rotationAngle, int outputWidth, bool bSkewedDecon,
                      char* OTF_file_name) {
  std::lock_guard<std::mutex> lk(g_mu);
  return init_session(g_s, nx, ny, nz, dr, dz, dr_psf, dz_psf, deskewAngle, rotationAngle,
                      outputWidth, bSkewedDecon, OTF_file_name) == 0
             ? 1
             : 0;
}

static int rl_common(const unsigned short* d_raw, const RLArgs& a, float* d_result,
                     float* d_deskewed, float* h_result, float* h_deskewed) {
  Session& s = g_s;
  if (!s.inited) {
    set_error("RL_interface", "RL_interface_init has not succeeded");
    return cudaErrorInvalidValue;
  }
  const float* out = nullptr;
  int dims[3];
  int rc;
  const size_t nd = (size_t)s.deskewedXdim * s.output_ny * s.output_nz;
  float* desk_dev = d_deskewed;
  if (h_deskewed && a.bSaveDeskewedRaw && fabs(s.deskewFactor) > 0.0) {
    if ((rc = s.desk_stage.ensure(nd))) return rc;
    desk_dev = s.desk_stage.p;
  }
  if ((rc = rl_pipeline(s, d_raw, a, desk_dev, &out, dims))) return rc;
  size_t nout = (size_t)dims[0] * dims[1] * dims[2];
  if (s.has_rot) {
    // never write more than the get_output_n* sizes the caller allocated
    const size_t cap = (size_t)reported_nx(s) * s.output_ny * reported_nz(s);
    if (nout > cap) nout = cap;
  }
  if (h_result) {
    CDX_CHECK(cudaMemcpyAsync(h_result, out, nout * sizeof(float), cudaMemcpyDeviceToHost, s.stream));
    if (h_deskewed && a.bSaveDeskewedRaw && fabs(s.deskewFactor) > 0.0 && desk_dev == s.desk_stage.p &&
        !(a.bSkewedDecon && a.nIters > 0))
      CDX_CHECK(cudaMemcpyAsync(h_deskewed, desk_dev, nd * sizeof(float), cudaMemcpyDeviceToHost,
                                s.stream));
    CDX_CHECK(cudaStreamSynchronize(s.stream));
    if (a.nIters > 0 && dft_form() == 1 && (rc = tc_check(s.plan.fx))) return rc;
  } else if (d_result && out != d_result) {
    CDX_CHECK(cudaMemcpyAsync(d_result, out, nout * sizeof(float), cudaMemcpyDeviceToDevice,
                              s.stream));
  }
  return 0;
}

int RL_interface(const unsigned short* const raw_data, int nx, int ny, int nz, float* result,
                 float* raw_deskewed_result, float background, bool bDoRescale,
                 bool bSaveDeskewedRaw, int nIters, int extraShift, int napodize, int nZblend,
                 float padVal, bool bDupRevStack, bool bSkewedDecon) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  s.launches = 0;
  if (!raw_data || !result || nx < 1 || ny < 1 || nz < 1) {
    set_error("RL_interface", "null pointer or empty stack");
    return 0;
  }
  if (ensure_stream(s)) return 0;
  const size_t nin = (size_t)nx * ny * nz;
  if (s.u16in.ensure(nin)) return 0;
  if (cudaMemcpyAsync(s.u16in.p, raw_data, nin * sizeof(unsigned short), cudaMemcpyHostToDevice,
                      s.stream) != cudaSuccess) {
    set_error("RL_interface", "host to device copy failed");
    return 0;
  }
  RLArgs a{nx, ny, nz, background, bDoRescale, bSaveDeskewedRaw, nIters, extraShift,
           napodize, nZblend, padVal, bDupRevStack, bSkewedDecon};
  return rl_common(s.u16in.p, a, nullptr, nullptr, result, raw_deskewed_result) == 0 ? 1 : 0;
}

int cdx_RL_device(const unsigned short* raw_data, int nx, int ny, int nz, float* result,
                  float* raw_deskewed_result, float background, bool bDoRescale,
                  bool bSaveDeskewedRaw, int nIters, int extraShift, int napodize, int nZblend,
                  float padVal, bool bDupRevStack, bool bSkewedDecon, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  s.launches = 0;
  if (!raw_data || !result) {
    set_error("cdx_RL_device", "null pointer");
    return 0;
  }
  if (ensure_stream(s)) return 0;
  // run on the caller's stream
  cudaStream_t own = s.stream;
  s.stream = (cudaStream_t)stream;
  RLArgs a{nx, ny, nz, background, bDoRescale, bSaveDeskewedRaw, nIters, extraShift,
           napodize, nZblend, padVal, bDupRevStack, bSkewedDecon};
  int rc = rl_common(raw_data, a, result, raw_deskewed_result, nullptr, nullptr);
  s.stream = own;
  return rc == 0 ? 1 : 0;
}

long long cdx_last_launch_count(void) { return g_s.launches; }

int cdx_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  prof_collect();
  Profiler& P = g_prof;
  P.on = on != 0;
  for (int p = 0; p < kPasses; ++p) {
    P.pass_ms[p] = 0;
    P.pass_n[p] = 0;
  }
  P.iter_ms = 0;
  P.iter_n = 0;
  return 1;
}

int cdx_profile_read(double* pass_ms, long long* pass_count, int max_passes, double* iter_ms,
                     long long* iter_count) {
  std::lock_guard<std::mutex> lk(g_mu);
  prof_collect();
  Profiler& P = g_prof;
  for (int p = 0; p < kPasses && p < max_passes; ++p) {
    if (pass_ms) pass_ms[p] = P.pass_ms[p];
    if (pass_count) pass_count[p] = P.pass_n[p];
  }
  if (iter_ms) *iter_ms = P.iter_ms;
  if (iter_count) *iter_count = P.iter_n;
  return kPasses;
}

const char* cdx_profile_pass_name(int i) { return (i >= 0 && i < kPasses) ? kPassNames[i] : ""; }

int cdx_set_dft_form(int form) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (form != 0 && form != 1) {
    set_error("cdx_set_dft_form", "form must be 0 (plain FP32) or 1 (mixed precision)");
    return 0;
  }
  set_dft_form(form);
  return 1;
}

int cdx_get_dft_form(void) { return dft_form(); }

int cdx_tc_length_supported(int n) {
  int q0 = 0, q1 = 0;
  return tc_plan_radices(n, q0, q1) ? 1 : 0;
}

int cdx_tc_status(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!s.plan.valid) return 1;
  if (s.stream) cudaStreamSynchronize(s.stream);
  return tc_check(s.plan.fx) == 0 ? 1 : 0;
}

int cdx_lambda_trace(int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (n <= 0) {
    s.lam_hist.release();
    s.lam_hist_n = 0;
    return 1;
  }
  if (s.lam_hist.ensure((size_t)n)) return 0;
  s.lam_hist_n = n;
  return 1;
}

int cdx_change_trace(int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (n <= 0) {
    s.chg_hist.release();
    s.chg_part.release();
    s.chg_hist_n = 0;
    return 1;
  }
  if (s.chg_hist.ensure((size_t)n) || s.chg_part.ensure(2 * (size_t)kChangeBlocks)) return 0;
  s.chg_hist_n = n;
  return 1;
}

int cdx_change_read(double* out, int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!out || s.chg_hist_n <= 0 || !s.chg_hist.p) {
    set_error("cdx_change_read", "no trace enabled (cdx_change_trace)");
    return -1;
  }
  const int m = n < s.chg_hist_n ? n : s.chg_hist_n;
  // the traced call may have run on a caller's stream (cdx_RL_device)
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    e = cudaMemcpy(out, s.chg_hist.p, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_cuda_error("cdx_change_read", e);
    return -1;
  }
  return m;
}

int cdx_lambda_read(float* out, int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!out || s.lam_hist_n <= 0 || !s.lam_hist.p) {
    set_error("cdx_lambda_read", "no trace enabled (cdx_lambda_trace)");
    return -1;
  }
  const int m = n < s.lam_hist_n ? n : s.lam_hist_n;
  cudaError_t e = cudaStreamSynchronize(s.stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(out, s.lam_hist.p, sizeof(float) * (size_t)m, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_cuda_error("cdx_lambda_read", e);
    return -1;
  }
  return m;
}

void RL_cleanup(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  s.intensity_overall0 = 0.;
  s.bFirstTime = true;
  s.plan.release();
  s.raw_otf.release();
  s.has_rot = false;
  s.inited = false;
  // release the large work buffers too (the reference frees them per call)
  s.Xa.release();
  s.Xb.release();
  s.G.release();
  s.raw.release();
  s.S.release();
  s.pre.release();
  s.u16in.release();
  s.rotbuf.release();
  s.desk_stage.release();
  s.res_stage.release();
  s.conv_tmp.release();
  s.tile_raw.release();
  s.tile_in.release();
  s.tile_out.release();
  s.tile_weight.release();
}

void cuda_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_b.origin) cudaStreamSynchronize(g_b.origin);
  g_b.release();
  release_all(g_s);
  g_s.inited = false;
  g_s.intensity_overall0 = 0.;
  g_s.bFirstTime = true;
  cudaDeviceReset();
}

int cdx_decon_grid(int* nx, int* ny, int* nz) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_s.inited || !g_s.plan.valid) {
    set_error("cdx_decon_grid", "RL_interface_init has not succeeded");
    return 0;
  }
  if (nx) *nx = g_s.plan.g.nx;
  if (ny) *ny = g_s.plan.g.ny;
  if (nz) *nz = g_s.plan.g.nz;
  return 1;
}

unsigned get_output_nx(void) { return reported_nx(g_s); }
unsigned get_output_ny(void) { return g_s.output_ny; }
unsigned get_output_nz(void) { return reported_nz(g_s); }

const char* get_version(void) { return "0.7.0-gb300"; }

const char* cdx_last_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_err_shared.c_str();
}

int Deskew_interface(const float* const raw_data, int nx, int ny, int nz, float dz, float dr,
                     float deskewAngle, float* const result, int outputWidth, int extraShift,
                     float padVal) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!raw_data || !result || nx < 1 || ny < 1 || nz < 1) {
    set_error("Deskew_interface", "null pointer or empty stack");
    return 0;
  }
  // RL-Biggs-Andrews.cpp:731-744 (output_nz is the RL_interface_init global)
  double deskewFactor = 0.;
  unsigned deskewedXdim = nx;
  if (fabs(deskewAngle) > 0.0) {
    if (deskewAngle < 0) deskewAngle += 180.;
    deskewFactor = cos(deskewAngle * M_PI / 180.) * dz / dr;
    if (outputWidth == 0)
      deskewedXdim += floor(s.output_nz * dz * fabs(cos(deskewAngle * M_PI / 180.)) / dr) / 4.;
    else
      deskewedXdim = outputWidth;
  }
  if (ensure_stream(s)) return 0;
  DevBuf<float> din, dout;
  const size_t nin = (size_t)nx * ny * nz, nout = (size_t)deskewedXdim * ny * nz;
  if (din.ensure(nin) || dout.ensure(nout)) return 0;
  int ok = 1;
  if (cudaMemcpyAsync(din.p, raw_data, nin * sizeof(float), cudaMemcpyHostToDevice, s.stream) ||
      launch_deskew(din.p, nx, ny, nz, deskewFactor, dout.p, deskewedXdim, extraShift, padVal,
                    s.stream) ||
      cudaMemcpyAsync(result, dout.p, nout * sizeof(float), cudaMemcpyDeviceToHost, s.stream) ||
      cudaStreamSynchronize(s.stream))
    ok = 0;
  din.release();
  dout.release();
  return ok;
}

int cdx_deskew_device(const float* in, int nx, int ny, int nz, double deskewFactor, float* out,
                      int nxOut, int extraShift, float padVal, void* stream) {
  return launch_deskew(in, nx, ny, nz, deskewFactor, out, nxOut, extraShift, padVal,
                       (cudaStream_t)stream) == 0
             ? 1
             : 0;
}

int cdx_rotate_device(const float* in, int nx, int ny, int nz, const float* rot, float* out,
                      int nx_out, int nz_out, void* stream) {
  return launch_rotate(in, nx, ny, nz, rot, out, nx_out, nz_out, (cudaStream_t)stream) == 0 ? 1 : 0;
}

int cdx_camcor_device(const unsigned short* raw, int nx, int ny, int nz, const float* camparam,
                      unsigned short* out, void* stream) {
  return launch_camcor(raw, nx, ny, nz, camparam, out, (cudaStream_t)stream) == 0 ? 1 : 0;
}

int camcor_interface_init(int nx, int ny, int nz, const float* const camparam) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!camparam || nx < 1 || ny < 1 || nz < 1) {
    set_error("camcor_interface_init", "null pointer or empty size");
    return 0;
  }
  if (ensure_stream(s)) return 0;
  const size_t np = (size_t)nx * ny * 3;
  if (s.cc_param.ensure(np)) return 0;
  if (cudaMemcpy(s.cc_param.p, camparam, np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("camcor_interface_init", "copy failed");
    return 0;
  }
  s.cc_nx = nx;
  s.cc_ny = ny;
  s.cc_nz = nz;
  return 1;
}

int camcor_interface(const unsigned short* const raw_data, int nx, int ny, int nz,
                     unsigned short* const result) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!s.cc_param.p) {
    set_error("camcor_interface", "camcor_interface_init has not succeeded");
    return 0;
  }
  if (nx != s.cc_nx || ny != s.cc_ny || nz != s.cc_nz || !raw_data || !result) {
    set_error("camcor_interface", "sizes differ from camcor_interface_init");
    return 0;
  }
  const size_t n = (size_t)nx * ny * nz;
  if (s.cc_in.ensure(n) || s.cc_out.ensure(n)) return 0;
  if (cudaMemcpyAsync(s.cc_in.p, raw_data, n * 2, cudaMemcpyHostToDevice, s.stream) ||
      launch_camcor(s.cc_in.p, nx, ny, nz, s.cc_param.p, s.cc_out.p, s.stream) ||
      cudaMemcpyAsync(result, s.cc_out.p, n * 2, cudaMemcpyDeviceToHost, s.stream) ||
      cudaStreamSynchronize(s.stream)) {
    set_error("camcor_interface", "CUDA failure");
    return 0;
  }
  return 1;
}

int Affine_interface(const float* const raw_data, int nx, int ny, int nz, float* const result,
                     const float* affMat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!raw_data || !result || !affMat || nx < 1 || ny < 1 || nz < 1) {
    set_error("Affine_interface", "null pointer or empty stack");
    return 0;
  }
  if (ensure_stream(g_s)) return 0;
  return affine_host(raw_data, nx, ny, nz, affMat, false, 1.f, 1.f, 1.f, result, g_s.stream) == 0;
}

int Affine_interface_RA(const float* const raw_data, int nx, int ny, int nz, float dx, float dy,
                        float dz, float* const result, const float* affMat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!raw_data || !result || !affMat || nx < 1 || ny < 1 || nz < 1) {
    set_error("Affine_interface_RA", "null pointer or empty stack");
    return 0;
  }
  if (ensure_stream(g_s)) return 0;
  return affine_host(raw_data, nx, ny, nz, affMat, true, dx, dy, dz, result, g_s.stream) == 0;
}

int cdx_fft_length_supported(int n) { return fft_len_supported(n) ? 1 : 0; }

int cdx_accel_factor_device(const float* g_new, const float* g_old, long long n, double* out,
                            float* lam, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!g_new || !g_old || n < 1) {
    set_error("cdx_accel_factor_device", "null pointer or empty array");
    return 0;
  }
  const size_t nblk = (size_t)accel_blocks(n);
  const bool fresh = s.acc_cnt.p == nullptr;
  if (s.acc_part.ensure(2 * nblk) || s.acc_cnt.ensure(1)) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (fresh && cudaMemsetAsync(s.acc_cnt.p, 0, sizeof(unsigned), st) != cudaSuccess) {
    set_error("cdx_accel_factor_device", "memset failed");
    return 0;
  }
  const float eps = 1.1920928955078125e-07f;
  return launch_accel_factor(g_new, g_old, n, s.acc_part.p, s.acc_cnt.p, eps, out, lam, st) == 0;
}

int cdx_load_image(const char* path, int* width, int* height, int* depth, float* out,
                   size_t capacity) {
  HostImage img;
  std::string err;
  if (!load_image_file(path, img, err)) {
    set_error("cdx_load_image", err.c_str());
    return 0;
  }
  if (width) *width = img.w;
  if (height) *height = img.h;
  if (depth) *depth = img.d;
  if (out) {
    if (capacity < img.data.size()) {
      set_error("cdx_load_image", "output buffer too small");
      return 0;
    }
    memcpy(out, img.data.data(), img.data.size() * sizeof(float));
  }
  return 1;
}

int cdx_rfft3d_device(const float* in, void* out_complex, int nx, int ny, int nz, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t st = (cudaStream_t)stream;
  Geom g = make_geom(nx, ny, nz);
  FftLen fx, fy, fz;
  DevBuf<float2> S;
  OtfDev none{};
  int ok = !(fft_len_init(fx, nx) || fft_len_init(fy, ny) || fft_len_init(fz, nz) ||
             S.ensure((size_t)g.spec_elems()) ||
             launch_x_fwd(g, fx, in, nullptr, nullptr, 0, S.p, st) ||
             launch_y_pass(g, fy, S.p, false, st) || launch_z_pass(g, fz, S.p, none, false, st, true) ||
             launch_spec_to_std(g, S.p, (float2*)out_complex, st) || cudaStreamSynchronize(st));
  fft_len_free(fx);
  fft_len_free(fy);
  fft_len_free(fz);
  S.release();
  return ok;
}

int cdx_conv3d_device(const float* in, float* out, int nx, int ny, int nz, int conj, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!s.raw_otf.p) {
    set_error("cdx_conv3d_device", "RL_interface_init has not succeeded");
    return 0;
  }
  if (ensure_stream(s) || ensure_plan(s, nx, ny, nz)) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  const GridPlan& p = s.plan;
  DevBuf<float2> S;
  int ok = !(S.ensure((size_t)p.g.spec_elems()) ||
             launch_x_fwd(p.g, p.fx, in, nullptr, nullptr, 0, S.p, st) ||
             launch_y_pass(p.g, p.fy, S.p, false, st) ||
             launch_z_pass(p.g, p.fz, S.p, p.otf, conj != 0, st) ||
             launch_y_pass(p.g, p.fy, S.p, true, st) || launch_x_inv_plain(p.g, p.fx, S.p, out, st) ||
             cudaStreamSynchronize(st));
  S.release();
  return ok;
}


int cdx_batch_grid(int nx, int ny, int nz, int* gx, int* gy, int* gz) {
  if (gx) *gx = nx >= 2 ? (int)find_optimal_dimension(nx) : 0;
  if (gy) *gy = ny >= 2 ? (int)find_optimal_dimension(ny) : 0;
  if (gz) *gz = nz >= 2 ? (int)find_optimal_dimension(nz) : 0;
  return 1;
}

int cdx_RL_batch_device(const cdx_batch_stack* stacks, int n, int nIters, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  return batch_run(stacks, n, nIters, (cudaStream_t)stream, false) == 0 ? 1 : 0;
}

int cdx_RL_batch_host(const cdx_batch_stack* stacks, int n, int nIters) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!stacks || n < 1) {
    set_error("cdx_RL_batch_host", "need at least one stack and nIters >= 0");
    return 0;
  }
  for (int i = 0; i < n; ++i) {
    const void* ptrs[2] = {stacks[i].raw, stacks[i].result};
    for (const void* ptr : ptrs) {
      cudaPointerAttributes at;
      if (!ptr || cudaPointerGetAttributes(&at, ptr) != cudaSuccess ||
          at.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        set_error("cdx_RL_batch_host",
                  "raw and result must be page-locked host buffers (cudaHostAlloc or "
                  "cudaHostRegister); use RL_interface or cdx_RL_batch_device otherwise");
        return 0;
      }
    }
  }
  return batch_run(stacks, n, nIters, nullptr, true) == 0 ? 1 : 0;
}

long long cdx_batch_last_launch_count(void) { return g_b.last_launches; }

int cdx_batch_set_streams(int device_streams, int host_streams) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (device_streams < 1 || device_streams > kBatchStreams || host_streams < 1 ||
      host_streams > kBatchStreams) {
    set_error("cdx_batch_set_streams", "stream counts must be in [1, 16]");
    return 0;
  }
  g_batch_streams[0] = device_streams;
  g_batch_streams[1] = host_streams;
  return 1;
}

int cdx_batch_get_streams(int* device_streams, int* host_streams) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (device_streams) *device_streams = g_batch_streams[0];
  if (host_streams) *host_streams = g_batch_streams[1];
  return 1;
}

void cdx_batch_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_b.origin) cudaStreamSynchronize(g_b.origin);
  g_b.release();
}


int cdx_wiener_device(const float* in, float* out, int nx, int ny, int nz, float background,
                      float wiener, float NA, float wavelength, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!s.inited || !s.raw_otf.p) {
    set_error("cdx_wiener_device", "RL_interface_init has not succeeded");
    return 0;
  }
  if (s.od.ny_otf != 1) {
    set_error("cdx_wiener_device", "the Wiener filter takes a radially averaged OTF");
    return 0;
  }
  if (!(wiener > 0.f) || !(NA > 0.f) || !(wavelength > 0.f) || !in || !out) {
    set_error("cdx_wiener_device", "wiener, NA and wavelength must be positive");
    return 0;
  }
  if (ensure_stream(s) || ensure_plan(s, nx, ny, nz)) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  const GridPlan& p = s.plan;
  const Geom& g = p.g;
  // wienerfilter's constants (linearDecon.cpp:898-908, 127-130): k steps of
  // the grid, their ratio to the OTF's, cutoff 2 NA / lambda
  const float dkx = 1.0 / (s.dr * nx);
  const float dky = 1.0 / (s.dr * ny);
  const float dkz = 1.0 / (s.dz * nz);
  const float rcutoff = 2 * NA / wavelength;
  const float w = wiener * wiener;
  const float kxscale = dkx / s.dkx_otf, kyscale = dky / s.dkx_otf, kzscale = dkz / s.dkz_otf;
  DevBuf<float2> S, H;
  DevBuf<float> tmp;
  OtfDev hd{};
  int ok = !(S.ensure((size_t)g.spec_elems()) || H.ensure((size_t)g.spec_elems()) ||
             tmp.ensure((size_t)g.nvox()));
  if (ok) {
    hd.mode = 1;
    hd.full = H.p;
    ok = !(launch_minus(in, tmp.p, g.nvox(), background, st) ||
           launch_wiener_h(g, s.raw_otf.p, (int)s.od.nx_otf, (int)s.od.nz_otf, dkx, dky, kxscale,
                           kyscale, kzscale, rcutoff, w, H.p, st) ||
           launch_x_fwd(g, p.fx, tmp.p, nullptr, nullptr, 0, S.p, st) ||
           launch_y_pass(g, p.fy, S.p, false, st) || launch_z_pass(g, p.fz, S.p, hd, false, st) ||
           launch_y_pass(g, p.fy, S.p, true, st) || launch_x_inv_plain(g, p.fx, S.p, out, st) ||
           cudaStreamSynchronize(st));
  }
  S.release();
  H.release();
  tmp.release();
  return ok;
}


int cdx_RL_tiled(const unsigned short* raw, int nx, int ny, int nz, float* result,
                 int tile_requested, int tile_overlap_requested, int blend, float background,
                 int nIters, int napodize, int nZblend, float padVal) {
  std::lock_guard<std::mutex> lk(g_mu);
  Session& s = g_s;
  if (!s.inited) {
    set_error("cdx_RL_tiled", "RL_interface_init has not succeeded");
    return 0;
  }
  if (!raw || !result || nx < 2 || ny < 2 || nz < 2) {
    set_error("cdx_RL_tiled", "null buffer or sizes below 2");
    return 0;
  }
  // tiling setup of the CLI (linearDecon.cpp:498-519)
  int tile_size = ny;
  int ntiles = 1;
  double overlap = 0;
  if (tile_requested != 0) {
    tile_size = tile_requested < 0 ? std::min(128, ny) : std::min(tile_requested, ny);
    if (tile_size - tile_overlap_requested <= 0) {
      set_error("cdx_RL_tiled", "tile overlap must be smaller than the tile");
      return 0;
    }
    ntiles = (int)ceil((double)ny / ((double)tile_size - tile_overlap_requested));
    if (ntiles > 1) overlap = floor(((double)tile_size * ntiles - ny) / (ntiles - 1));
  }
  if ((int)s.output_ny != (int)find_optimal_dimension(tile_size) || s.output_nx == 0) {
    set_error("cdx_RL_tiled", "RL_interface_init must be called with ny = the tile size");
    return 0;
  }
  const int no_zone = (int)ceil((overlap - 4) / 2.0);  // 1175-1245: no zone, blend zone, ...
  const int blend_zone = (int)(overlap - no_zone - no_zone);
  RLArgs a{nx, tile_size, nz, background, false, false, nIters, 0, napodize, nZblend, padVal,
           false, false};
  if (ensure_stream(s)) return 0;
  cudaStream_t st = s.stream;
  const size_t tvox = (size_t)nx * tile_size * nz;
  DevBuf<unsigned short>& d_raw = s.tile_raw;
  DevBuf<unsigned short>& d_tile = s.tile_in;
  DevBuf<float>& stitch = s.tile_out;
  DevBuf<unsigned char>& weight = s.tile_weight;
  int onx = 0, ony_total = 0, onz = 0;
  // the raw stack goes to the device once; each tile's rows are gathered there
  int ok = d_raw.ensure((size_t)nx * ny * nz) == 0 && d_tile.ensure(tvox) == 0 &&
           cudaMemcpyAsync(d_raw.p, raw, sizeof(unsigned short) * (size_t)nx * ny * nz,
                           cudaMemcpyHostToDevice, st) == cudaSuccess;
  if (!ok) set_cuda_error("cdx_RL_tiled", cudaGetLastError());
  for (int t = 0; ok && t < ntiles; ++t) {
    const int yoff = (int)floor((double)t * (tile_size - overlap));
    if (launch_tile_rows(d_raw.p, d_tile.p, nx, ny, nz, tile_size, yoff, st)) {
      ok = 0;
      break;
    }
    const float* out = nullptr;
    int dims[3];
    if (rl_pipeline(s, d_tile.p, a, nullptr, &out, dims)) {
      ok = 0;
      break;
    }
    if (t == 0) {
      onx = dims[0];
      onz = dims[2];
      ony_total = ntiles > 1 ? ny : dims[1];
      const size_t n = (size_t)onx * ony_total * onz;
      if (stitch.ensure(n) || weight.ensure(n) ||
          cudaMemsetAsync(stitch.p, 0, n * sizeof(float), st) != cudaSuccess ||
          cudaMemsetAsync(weight.p, 0, n, st) != cudaSuccess) {
        ok = 0;
        break;
      }
    }
    if (ntiles == 1) {
      if (cudaMemcpyAsync(stitch.p, out, sizeof(float) * (size_t)onx * ony_total * onz,
                          cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        ok = 0;
    } else if (launch_stitch(out, stitch.p, weight.p, onx, dims[1], onz, ony_total, yoff, overlap,
                             no_zone, blend_zone, t == 0, t + 1 >= ntiles, blend != 0, st)) {
      ok = 0;
    }
  }
  if (ok)
    ok = cudaMemcpyAsync(result, stitch.p, sizeof(float) * (size_t)onx * ony_total * onz,
                         cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
  else
    cudaStreamSynchronize(st);
  return ok;
}

int cdx_mip_device(const float* in, int nx, int ny, int nz, int axis, float* out, void* stream) {
  if (!in || !out || nx < 1 || ny < 1 || nz < 1) {
    set_error("cdx_mip_device", "null buffer or empty sizes");
    return 0;
  }
  return launch_mip(in, nx, ny, nz, axis, out, (cudaStream_t)stream) == 0 ? 1 : 0;
}

}  // extern "C"
