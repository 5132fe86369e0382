// Host-side launch interface of the cudadecon_gb300 CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include "fft_engine.cuh"

namespace cdx {

// Geometry of one real volume (x fastest) and of its half spectrum.
//
// The spectrum is an internal buffer and uses kx-plane-major order
// S[kx][z][y] (y fastest, row pitch nyp = ny rounded up to even), unlike
// cuFFT's [z][y][kx].  Each plane holds the (z, y) samples of one kx column,
// so the y pass reads contiguous rows, the z pass reads 128-byte runs, and
// the x passes write and read transposed 16-byte (two-row) groups.
struct Geom {
  int nx, ny, nz;
  int nxh;         // nx/2 + 1
  int nyp;         // ny rounded up to even
  long long plane; // nz * nyp complex elements per kx plane
  long long nvox() const { return (long long)nx * ny * nz; }
  long long spec_elems() const { return (long long)nxh * plane; }
};
Geom make_geom(int nx, int ny, int nz);

// OTF description used by the z pass.
struct OtfDev {
  int mode;           // 0: radially averaged table, 1: full 3D array in spectrum layout
  int nr;             // radial samples of the raw OTF (reference: nx_otf)
  float kxscale, kyscale;
  const float4* tz;   // mode 0: [nz][nr] OTF resampled along kz, scaled by 1/N, as
                      // pairs (value at ir, value at ir + 1; 0 past the table)
  const float2* full; // mode 1: spectrum-layout OTF, scaled by 1/N
};

// Raw OTF as read from file, described like the reference's
// determine_OTF_dimensions() (src/RL-Biggs-Andrews.cpp:506-529).
struct RawOtfDims {
  unsigned nx_otf, ny_otf, nz_otf;
  float kxscale, kyscale, kzscale;
};

// Tables of a tensor-core row plan (mixed-precision form, decon_x_tc.cu):
// the DFT matrices of the two radices as tf32 hi/lo MMA operands, the
// twiddles, and an error word the kernels set when a wait on the tensor
// core runs out.
struct TcTables {
  int q0 = 0, q1 = 0;
  float* d_b = nullptr;
  float2* d_tw = nullptr;
  int* d_err = nullptr;
};
bool tc_plan_radices(int L, int& q0, int& q1);
int tc_tables_init(TcTables& t, int L);
void tc_tables_free(TcTables& t);

// Which form the x passes take: 0 = plain FP32 (CUDA-core FFT), 1 = mixed
// precision (tensor-core DFT stages where the length has a tensor-core plan).
int dft_form();
void set_dft_form(int form);

// FFT plan for one length (host side owns the twiddle table).
// When the length is in the registry of specialised plans (static_plans.cuh),
// sdev holds that plan (its radices and twiddle table) as well.
struct FftLen {
  FftDev dev;
  float2* d_tw = nullptr;
  bool has_static = false;
  FftDev sdev;
  float2* d_tws = nullptr;
  // the x ratio / x update plan where it differs from the registered one
  bool has_xr = false;
  FftDev xrdev;
  float2* d_twxr = nullptr;
  // the generated x-pass plan of the length, if it has one
  bool has_gx = false;
  FftDev gxdev;
  float2* d_twgx = nullptr;
  // the generated z-pass plan of the length, if it has one
  bool has_gz = false;
  FftDev gzdev;
  float2* d_twgz = nullptr;
  // the tensor-core plan of the length, if it has one
  bool has_tc = false;
  TcTables tc;
};
int fft_len_init(FftLen& f, int L);
void fft_len_free(FftLen& f);
bool fft_len_supported(int L);

// Per-session device state for the Biggs-Andrews loop.
struct RLWork {
  double* partials = nullptr;   // 2 * max_blocks (16 bytes per x-pass block)
  float* lam = nullptr;         // two slots: lambda used by iteration k is lam[k & 1]
  int max_blocks = 0;
};

// ---------------------------------------------------------------- passes
// Number of blocks of the x passes (= dot-product partials per iteration).
int x_pass_blocks(const Geom& g);
// Forward x pass: Y (from X, Xm1, lambda when predict != 0, else Y = X) ->
// spectrum after the R2C along x.  When predict != 0, Y = max(X + lam*(X - Xm1), 0)
// is also written over Xm1 (whose old values are not needed afterwards).
int launch_x_fwd(const Geom& g, const FftLen& fx, const float* X, float* Xm1,
                 const float* lam, int predict, float2* S, cudaStream_t st);
// In-place complex FFT along y of every (kx, z) row.
int launch_y_pass(const Geom& g, const FftLen& fy, float2* S, bool inverse, cudaStream_t st);
// z FFT, multiply by OTF (or its conjugate), inverse z FFT, in place.
// fwd_only (test path) stops after the forward z FFT.
int launch_z_pass(const Geom& g, const FftLen& fz, float2* S, const OtfDev& otf, bool conj,
                  cudaStream_t st, bool fwd_only = false);
// Inverse x pass followed by the RL ratio and the forward x pass of the
// second convolution (spectrum updated in place).
int launch_x_inv_ratio_fwd(const Geom& g, const FftLen& fx, float2* S, const float* raw,
                           float eps, cudaStream_t st);
// Inverse x pass followed by the estimate update from the prediction Y:
//   Xnew = max(CC*Y, 0); Gnew = Xnew - Y
// writes Xnew into Xout (may alias Y) and Gnew into G, and when dots != 0
// accumulates (Gnew.Gold, Gold.Gold) per block, then a one-block kernel stores
// the next lambda into lam_next.
int launch_x_inv_update(const Geom& g, const FftLen& fx, const float2* S, const float* Y,
                        float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                        cudaStream_t st);
// The next acceleration factor from nblk float-float partials (one block).
int launch_lambda(const float4* partials, int nblk, float* lam_next, float eps, cudaStream_t st);
// Convergence norm of an RL step, in FP64: *out = ||x_new - x_old|| / ||x_old||
// (0 when x_old is 0).  part: kChangeBlocks * 2 doubles of scratch.
constexpr int kChangeBlocks = 304;
int launch_change_norm(const float* x_new, const float* x_old, long long n, double* part,
                       double* out, cudaStream_t st);
// The x passes in the mixed-precision form (same contracts as the three
// launchers above; err: the plan's error word).
int launch_xtc_fwd(const Geom& g, const TcTables& t, const float* X, float* Xm1, const float* lam,
                   int predict, float2* S, int* err, cudaStream_t st);
int launch_xtc_ratio(const Geom& g, const TcTables& t, float2* S, const float* raw, float eps,
                     int* err, cudaStream_t st);
int launch_xtc_update(const Geom& g, const TcTables& t, const float2* S, const float* Y,
                      float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                      int* err, cudaStream_t st);
// 0 when no tensor-core wait of the plan has run out (reads the error word;
// synchronises the device).
int tc_check(const FftLen& f);

// Plain inverse x pass to a real volume (test path).
int launch_x_inv_plain(const Geom& g, const FftLen& fx, const float2* S, float* out,
                       cudaStream_t st);
// Unpack spectrum S into cuFFT/numpy order [z][y][kx] (test path).
int launch_spec_to_std(const Geom& g, const float2* S, float2* out, cudaStream_t st);

// OTF preparation
int launch_otf_tz(const Geom& g, const float2* raw_otf, const RawOtfDims& od, float4* tz,
                  float scale, cudaStream_t st);
int launch_otf_full(const Geom& g, const float2* raw_otf, const RawOtfDims& od, float2* full,
                    float scale, cudaStream_t st);

// ---------------------------------------------------------------- pre/post
int launch_u16_to_f32_crop(const unsigned short* in, int nx_in, int ny_in, int nx, int ny, int nz,
                           float* out, float background, int subtract_bg, cudaStream_t st);
int launch_bgsub(float* img, long long n, float background, cudaStream_t st);
int launch_apodize(float* img, int nx, int ny, int nz, int napodize, cudaStream_t st);
int launch_zblend(float* img, int nx, int ny, int nz, int nZblend, cudaStream_t st);
int launch_dup_rev(float* img, int nx, int ny, int nz, cudaStream_t st);
int launch_scale(float* img, long long n, double factor, cudaStream_t st);
// Mean of voxels above the mean, as the reference's meanAboveBackground_GPU
// (src/RLgpuImpl.cu:668-718); blocks until the result is on the host.
int mean_above_background(const float* img, long long n, double* d_tmp, unsigned* d_cnt,
                          double* result, cudaStream_t st);
int launch_deskew(const float* in, int nx, int ny, int nz, double deskewFactor, float* out,
                  int nxOut, int extraShift, float padVal, cudaStream_t st);
int launch_rotate(const float* in, int nx_in, int ny, int nz_in, const float* rot_host, float* out,
                  int nx_out, int nz_out, cudaStream_t st);
int launch_camcor(const unsigned short* raw, int nx, int ny, int nz, const float* camparam,
                  unsigned short* out, cudaStream_t st);
int launch_f32_to_u16(const float* in, unsigned short* out, long long n, cudaStream_t st);
// Host-to-host affine transform through a 3D texture (ra: world coordinates).
int affine_host(const float* in, int nx, int ny, int nz, const float* mat16, bool ra, float dx,
                float dy, float dz, float* out, cudaStream_t st);

// Wiener filter factor conj(OTF)(1 - kr/rcutoff)/(|OTF|^2 + w) / N in the
// spectrum layout, from the radial OTF table (nr x nzotf complex).
int launch_wiener_h(const Geom& g, const float2* otf, int nr, int nzotf, float dkx, float dky,
                    float kxscale, float kyscale, float kzscale, float rcutoff, float w,
                    float2* H, cudaStream_t st);
// out = in - bg (no clamp).
int launch_minus(const float* in, float* out, long long n, float bg, cudaStream_t st);

// Stitch a deconvolved y tile into the output (the CLI's tiling rules).
int launch_tile_rows(const unsigned short* raw, unsigned short* tile, int nx, int ny, int nz,
                     int tny, int yoff, cudaStream_t st);
int launch_stitch(const float* tile, float* out, unsigned char* weight, int nx, int tny, int nz,
                  int ny_out, int yoff, double overlap, int no_zone, int blend_zone, bool first,
                  bool last, bool blend, cudaStream_t st);
// Maximum-intensity projection along axis 0 (x), 1 (y) or 2 (z).
int launch_mip(const float* in, int nx, int ny, int nz, int axis, float* out, cudaStream_t st);

}  // namespace cdx
