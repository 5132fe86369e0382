/*
 * cudadecon_gb300 C ABI.
 *
 * The first block keeps the exported entry points of the reference library
 * libcudaDecon (scopetools/cudadecon, src/linearDecon.h:243-317) with the same
 * names, argument order, argument meaning and return convention (1 = success,
 * 0 = failure), so that a ctypes caller such as pycudadecon can load this
 * library in its place.  Unlike the reference, no entry point exits the
 * process or throws across the ABI on a CUDA error: it returns 0 and the
 * reason is available from cdx_last_error().
 *
 * The second block adds entry points with no counterpart in the reference:
 * the same RL pipeline on device pointers and a caller stream, the geometry
 * kernels on device pointers, and FFT test hooks.
 */
#ifndef CUDADECON_GB300_H
#define CUDADECON_GB300_H

#include <stddef.h>

#ifdef __cplusplus
#define CDX_DEFAULT(v) = v
extern "C" {
#else
#include <stdbool.h>
#define CDX_DEFAULT(v)
#endif

/* ------------------------------------------------------------------ *
 * Reference ABI                                                       *
 * ------------------------------------------------------------------ */

/* Replaces RL_interface_init (src/linearDecon.h:260-264, defined at
 * src/RL-Biggs-Andrews.cpp:531-655).  Rounds ny, nz (and nx when there is
 * no deskew) down to 2,3,5,7-smooth sizes, loads the OTF file (TIFF or .cimg),
 * derives the deskew factor / deskewed width / rotation matrix and prepares
 * the FFT plans and the OTF table for the decon grid.  Returns 0 when the OTF
 * cannot be read or a size is unsupported. */
int RL_interface_init(int nx, int ny, int nz, float dr, float dz, float dr_psf, float dz_psf,
                      float deskewAngle, float rotationAngle, int outputWidth, bool bSkewedDecon,
                      char* OTF_file_name);

/* Replaces RL_interface (src/linearDecon.h:278-283, defined at
 * src/RL-Biggs-Andrews.cpp:657-705): crop at the origin to the init sizes,
 * apodize, subtract background, optional bleach rescale, deskew, z blend,
 * optional mirrored stack, nIters Biggs-Andrews RL iterations, optional
 * deskew after decon and rotation.  result must hold
 * get_output_nx()*get_output_ny()*get_output_nz() floats. */
int RL_interface(const unsigned short* const raw_data, int nx, int ny, int nz, float* result,
                 float* raw_deskewed_result, float background, bool bDoRescale,
                 bool bSaveDeskewedRaw, int nIters, int extraShift, int napodize CDX_DEFAULT(0),
                 int nZblend CDX_DEFAULT(0), float padVal CDX_DEFAULT(0),
                 bool bDupRevStack CDX_DEFAULT(false), bool bSkewedDecon CDX_DEFAULT(false));

/* Replaces Deskew_interface (src/linearDecon.h:285-288, defined at
 * src/RL-Biggs-Andrews.cpp:724-773), including its output width rule when
 * outputWidth == 0 (uses the nz of the last RL_interface_init, divided by 4). */
int Deskew_interface(const float* const raw_data, int nx, int ny, int nz, float dz, float dr,
                     float deskewAngle, float* const result, int outputWidth, int extraShift,
                     float padVal CDX_DEFAULT(0));

/* Replaces Affine_interface (src/linearDecon.h:290-292; RL-Biggs-Andrews.cpp:776-814
 * and geometryTransform.cu:183-213,257-301): out(x,y,z) = trilinear sample of
 * the input at M*(x,y,z,1) with border 0; M is a 4x4 row-major matrix. */
int Affine_interface(const float* const raw_data, int nx, int ny, int nz, float* const result,
                     const float* affMat);

/* Replaces Affine_interface_RA (src/linearDecon.h:294-296; RL-Biggs-Andrews.cpp:816-855
 * and geometryTransform.cu:216-253,304-349): the same in world coordinates with
 * voxel size (dx, dy, dz). */
int Affine_interface_RA(const float* const raw_data, int nx, int ny, int nz, float dx, float dy,
                        float dz, float* const result, const float* affMat);

/* Replaces camcor_interface_init (declared at src/linearDecon.h:298-299; the
 * reference's only definition, src/llspy.cpp:70-78, is not built).  camparam
 * holds three nx*ny float planes: a, b, offset (camcor.cu:97-99). */
int camcor_interface_init(int nx, int ny, int nz, const float* const camparam);

/* Replaces camcor_interface (declared at src/linearDecon.h:301-303; semantics
 * of camcor_kernel, src/camcor.cu:80-108). */
int camcor_interface(const unsigned short* const raw_data, int nx, int ny, int nz,
                     unsigned short* const result);

/* Replaces RL_cleanup (src/linearDecon.h:306; RL-Biggs-Andrews.cpp:707-715):
 * frees the OTF, plans and buffers and resets the bleach-correction state. */
void RL_cleanup(void);

/* Replaces cuda_reset (src/linearDecon.h:307; RL-Biggs-Andrews.cpp:717-720). */
void cuda_reset(void);

/* Replace get_output_nx/ny/nz (src/linearDecon.h:311-313;
 * RL-Biggs-Andrews.cpp:474-503), including the reference's use of the signed
 * rotation-matrix entry in get_output_nx. */
unsigned get_output_nx(void);
unsigned get_output_ny(void);
unsigned get_output_nz(void);

/* Replaces get_version (src/linearDecon.h:316). */
const char* get_version(void);

/* ------------------------------------------------------------------ *
 * Extensions (no counterpart in the reference)                        *
 * ------------------------------------------------------------------ */

/* Message of the last failure of any entry point ("" when none). */
const char* cdx_last_error(void);

/* RL_interface on device memory and a caller stream (cudaStream_t, may be
 * NULL for the legacy default stream).  raw_data (u16), result and
 * raw_deskewed_result are device pointers.  Work buffers are owned by the
 * library and reused across calls; the call returns once all work is
 * enqueued (it synchronises only when bDoRescale needs the bleach statistic
 * on the host). */
int cdx_RL_device(const unsigned short* raw_data, int nx, int ny, int nz, float* result,
                  float* raw_deskewed_result, float background, bool bDoRescale,
                  bool bSaveDeskewedRaw, int nIters, int extraShift, int napodize, int nZblend,
                  float padVal, bool bDupRevStack, bool bSkewedDecon, void* stream);

/* Sizes of the decon grid (the volume the RL iterations run on) of the
 * current RL_interface_init session. */
int cdx_decon_grid(int* nx, int* ny, int* nz);

/* Number of kernels the last cdx_RL_device / RL_interface call launched. */
long long cdx_last_launch_count(void);

/* Per-pass timing of the RL iteration with CUDA events recorded on the launch
 * stream.  cdx_profile_enable(1) resets the accumulators and starts
 * recording; cdx_profile_read synchronises and returns the number of passes
 * per iteration (9), the summed milliseconds and counts of each pass, and of
 * whole iterations.  cdx_profile_pass_name(i) names pass i. */
int cdx_profile_enable(int on);
int cdx_profile_read(double* pass_ms, long long* pass_count, int max_passes, double* iter_ms,
                     long long* iter_count);
const char* cdx_profile_pass_name(int i);

/* Form of the DFTs of the x passes (extension; the reference runs cuFFT in
 * FP32): 0 = plain FP32 on the CUDA cores (default); 1 = mixed
 * precision, where rows whose length has a tensor-core plan
 * (cdx_tc_length_supported: 256, 512, 756, 1024) run their DFT stages as
 * tcgen05 MMAs in TF32 with each FP32 operand split into a high and a low
 * part (three products, FP32 accumulation; relative error of the transforms
 * about 1e-6).  Other passes and lengths stay on the CUDA cores.  The form
 * applies to every later RL call of the process.  cdx_set_dft_form returns 0
 * for another value. */
int cdx_set_dft_form(int form);
int cdx_get_dft_form(void);
int cdx_tc_length_supported(int n);
/* 1 when no wait on the tensor core of the current session has run out
 * (the kernels bound every wait to about a second and then give up; the
 * result of such a call is invalid).  Waits for the session's stream.
 * RL_interface checks this itself and returns 0. */
int cdx_tc_status(void);

/* Trace of the Biggs-Andrews acceleration factors (extension; the reference
 * prints them, RL-Biggs-Andrews.cpp:300).  cdx_lambda_trace(n) with n > 0
 * makes every later RL call record, for iteration k < n, the factor lambda_k
 * it applied (0 for k <= 1, which predict nothing); n == 0 stops tracing.
 * cdx_lambda_read waits for the last call and copies min(n, traced) factors
 * to out; it returns their number, or -1 without a trace. */
int cdx_lambda_trace(int n);
int cdx_lambda_read(float* out, int n);

/* Convergence norms (extension; the reference computes none): with
 * cdx_change_trace(n), n > 0, the next RL_interface / cdx_RL_device calls
 * record after each iteration k < n the relative change of the estimate,
 * ||X_{k+1} - X_k||_2 / ||X_k||_2, with the squares summed in FP64 by two
 * extra kernels (none run without the trace); n <= 0 turns the trace off.
 * cdx_change_read waits for the device and copies min(n, traced) values;
 * returns that count, or -1 without a trace.  Returns of cdx_change_trace:
 * 1, or 0 when its buffers cannot be allocated. */
int cdx_change_trace(int n);
int cdx_change_read(double* out, int n);

/* Deskew / rotate / camcor on device pointers (same arithmetic as the
 * reference kernels).  rot is a host pointer to the 4 rotation-matrix floats. */
int cdx_deskew_device(const float* in, int nx, int ny, int nz, double deskewFactor, float* out,
                      int nxOut, int extraShift, float padVal, void* stream);
int cdx_rotate_device(const float* in, int nx, int ny, int nz, const float* rot, float* out,
                      int nx_out, int nz_out, void* stream);
int cdx_camcor_device(const unsigned short* raw, int nx, int ny, int nz, const float* camparam,
                      unsigned short* out, void* stream);

/* FFT test hooks on device pointers: forward 3D real FFT of in (nz, ny, nx)
 * written in numpy/cuFFT order (nz, ny, nx/2+1) complex64; and the
 * convolution out = irfftn(rfftn(in) * H) where H is the OTF of the current
 * RL_interface_init session evaluated on the (nx, ny, nz) grid (conj != 0
 * uses conj(H)). */
int cdx_rfft3d_device(const float* in, void* out_complex, int nx, int ny, int nz, void* stream);
int cdx_conv3d_device(const float* in, float* out, int nx, int ny, int nz, int conj, void* stream);

/* Biggs-Andrews acceleration factor of two device float arrays of n
 * elements, as the reference's calcAccelFactor (src/RLgpuImpl.cu:510-569):
 * num = g_new.g_old, den = g_old.g_old (float products, double sums),
 * lambda = num / (den + FLT_EPSILON).  Results stay on the device: out
 * (3 doubles, may be NULL) receives num, den and lambda; lam (1 float, may be
 * NULL) receives lambda clamped to [0, 1] as RL-Biggs-Andrews.cpp:298 uses it.
 * Scratch for the per-block partials is allocated by the library on first
 * use (cudaMalloc) and reused. */
int cdx_accel_factor_device(const float* g_new, const float* g_old, long long n, double* out,
                            float* lam, void* stream);

/* Same result as cdx_accel_factor_device, but allocates nothing: no entry
 * point of the reference corresponds to it.  For callers that cannot let a
 * library allocate device memory while they run -- pipelines that overlap
 * transfers and deconvolution on several streams (cudaMalloc and cudaFree
 * synchronise the device) and processes that reserve GPU memory up front.
 * The scratch is a fixed 64 KB array in device memory held by every GPU that
 * loads the library; n is limited to 33554432 elements (larger n returns 0
 * with an error message).  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current, so make it
 * before any stream capture; the lookup is repeated when the current context
 * is another one than at the last lookup (after cuda_reset, or under a
 * context the caller made).  All calls share the array and clear its counter
 * on entry: calls that may overlap on the GPU race and must be serialised. */
int cdx_accel_factor_device_noalloc(const float* g_new, const float* g_old, long long n,
                                    double* out, float* lam, void* stream);

/* 1 if n is a product of 2, 3, 5 and 7 (a supported FFT length). */
int cdx_fft_length_supported(int n);

/* Read an image file (TIFF or .cimg) the way RL_interface_init reads the
 * OTF.  Writes the CImg sizes (width, height, depth) and, when out is not
 * NULL and capacity (in floats) suffices, the samples in CImg order.
 * Returns 1 on success.  Host only: usable without a GPU. */
int cdx_load_image(const char* path, int* width, int* height, int* depth, float* out,
                   size_t capacity);

/* One-step Wiener filter instead of RL (the reference's CLI option --wiener,
 * linearDecon.cpp:116-168 and 1116-1127; no ABI entry point there): out =
 * IFFT( FFT(in - background) * conj(OTF) (1 - kr/kc) / (|OTF|^2 + wiener^2) ),
 * kc = 2 NA / wavelength (1/um), zero beyond kc, with the OTF (a radial
 * table) and pixel sizes of the last RL_interface_init.  in and out are
 * device pointers on the (nz, ny, nx) grid (each size a product of 2, 3, 5
 * and 7).  Returns 1 on success, 0 on failure (extension). */
int cdx_wiener_device(const float* in, float* out, int nx, int ny, int nz, float background,
                      float wiener, float NA, float wavelength, void* stream);

/* Y-tiled deconvolution of the CLI (--tile, --TileOverlap, --BlendTileOverlap;
 * linearDecon.cpp:497-566 and 1175-1245), for stacks whose decon buffers do
 * not fit the GPU at once: the (nz, ny, nx) u16 host stack is cut into tiles
 * of tile rows along y (tile < 0: min(128, ny); 0: no tiling) overlapping by
 * about tile_overlap rows (rows past the stack repeat its last row), each tile
 * is processed as RL_interface processes a stack (call RL_interface_init with
 * ny = the tile size first), and the results are stitched back as the CLI
 * does: each overlap is split between the two tiles, or blended over a few
 * rows when blend != 0.  result (host) holds get_output_nx() * ny *
 * get_output_nz() floats.  Returns 1 on success (extension). */
int cdx_RL_tiled(const unsigned short* raw, int nx, int ny, int nz, float* result, int tile,
                 int tile_overlap, int blend, float background, int nIters, int napodize,
                 int nZblend, float padVal);

/* Maximum-intensity projection (the CLI's MIPs, linearDecon.cpp:1434-1473) of a
 * device (nz, ny, nx) float volume along axis 0 (x; out (nz, ny)), 1 (y; out
 * (nz, nx)) or 2 (z; out (ny, nx)).  Returns 1 on success (extension). */
int cdx_mip_device(const float* in, int nx, int ny, int nz, int axis, float* out, void* stream);

/* ---- OTF generation ---------------------------------------------------
 * makeOTF of the reference's libradialft (src/radialft_interface.cpp:52-58,
 * 95-197): reads a PSF stack (TIFF or .cimg), finds the bead (peak and
 * parabola fits) and the background, subtracts it, and writes the
 * radially averaged OTF RL_interface_init reads (float32 TIFF of width
 * 2*nz and height nx/2+1, complex, kz fastest) or, with b3Dout, the 3D OTF
 * (width 2*(nx/2+1), height ny, depth nz).  The transform runs on the GPU
 * with this library's FFT, so each PSF size must be a product of 2, 3, 5
 * and 7 (the reference uses FFTW, which takes any size).  Returns 0 on
 * success and 1 on failure, as the reference does (cdx_last_error()). */
int makeOTF(const char* const ifiles, const char* const ofiles, int lambdanm CDX_DEFAULT(520),
            float dz CDX_DEFAULT(0.102f), int interpkr CDX_DEFAULT(10),
            bool bUserBackground CDX_DEFAULT(false), float background CDX_DEFAULT(90),
            float NA CDX_DEFAULT(1.25f), float NIMM CDX_DEFAULT(1.3f), float dr CDX_DEFAULT(0.102f),
            int krmax CDX_DEFAULT(0), bool bDoCleanup CDX_DEFAULT(false),
            bool b3Dout CDX_DEFAULT(false));

/* makeOTF on a PSF in host memory ((nz, ny, nx) float32, x fastest), with the
 * OTF image returned in `out` (capacity in floats; NULL to query the sizes)
 * instead of a file.  Returns 1 on success, 0 on failure (extension). */
int cdx_make_otf(const float* psf, int nx, int ny, int nz, int lambdanm, float dz, int interpkr,
                 int bUserBackground, float background, float NA, float NIMM, float dr, int krmax,
                 int bDoCleanup, int b3Dout, float* out, size_t capacity, int* out_w, int* out_h,
                 int* out_d);

/* Write a float32 image (width x height x depth, x fastest) as an
 * uncompressed TIFF, one page per z, e.g. an OTF table for
 * RL_interface_init.  Returns 1 on success (extension; host only). */
int cdx_save_image(const char* path, int width, int height, int depth, const float* data);

/* ---- Batched deconvolution of independent stacks (extension) ----------
 * No entry point of the reference corresponds to these: pycudadecon
 * deconvolves timepoints, channels and tiles one RL_interface call at a
 * time, re-initialising for every shape or OTF.  One stack of a batch: */
typedef struct cdx_batch_stack {
  const unsigned short* raw; /* device: (nz, ny, nx) uint16 stack, x fastest */
  int nx, ny, nz;
  float* result;             /* device: (gz, gy, gx) float32 (cdx_batch_grid) */
  const float* otf;          /* host: OTF table as RL_interface_init reads the file:
                                otf_h rows of otf_w floats (radial tables: nr rows of
                                nz_otf complex values, kz fastest) */
  int otf_w, otf_h;
  float dr, dz, dr_psf, dz_psf; /* pixel sizes of the stack and of the PSF (um) */
  float background;
} cdx_batch_stack;

/* Decon grid of a stack: each size rounded down to a product of 2, 3, 5 and
 * 7 (findOptimalDimension, RL-Biggs-Andrews.cpp:18-43).  Returns 1. */
int cdx_batch_grid(int nx, int ny, int nz, int* gx, int* gy, int* gz);

/* Deconvolve n stacks of any shapes, each with its own OTF: every stack is
 * processed as RL_interface processes a stack initialised without deskew or
 * rotation (crop to its decon grid, background subtraction, nIters
 * Biggs-Andrews RL iterations; no rescale, apodize, z-blend or mirrored
 * stack), and the final estimate is written to result.  The iterations of
 * all stacks run as one CUDA graph whose per-stack chains are spread over
 * several streams (small stacks run concurrently); the graph is kept and
 * replayed while the stack shapes, OTF sizes, pixel sizes and nIters stay
 * the same.  Work runs after the work already queued on `stream` (a
 * cudaStream_t, or NULL) and the results are complete when the work queued
 * on `stream` after this call runs.  Returns 1 on success, 0 on failure
 * (cdx_last_error()). */
int cdx_RL_batch_device(const cdx_batch_stack* stacks, int n, int nIters, void* stream);

/* cdx_RL_batch_device with the stacks and results in host memory: raw and
 * result of every stack are page-locked host buffers (cudaHostAlloc or
 * cudaHostRegister; pageable memory is rejected).  The uploads (in the
 * order the chains need them) and the downloads (each after its stack's
 * chain) are nodes of the captured graph on streams of their own, so
 * transfers overlap the stacks' iterations; the graph is also kept
 * while the host buffers and backgrounds stay the same.  Returns 1 once the
 * results are in the host buffers, 0 on failure (extension). */
int cdx_RL_batch_host(const cdx_batch_stack* stacks, int n, int nIters);

/* Streams the batch's per-stack chains are spread over: device_streams for
 * cdx_RL_batch_device, host_streams for cdx_RL_batch_host (whose uploads
 * and downloads run on two more streams of their own); default 2 each, each
 * in [1, 16].  The next batch call recaptures its graph
 * when its count changed.  Results do not depend on the counts.  Returns 1,
 * or 0 for a count out of range (extension). */
int cdx_batch_set_streams(int device_streams, int host_streams);
int cdx_batch_get_streams(int* device_streams, int* host_streams);

/* Number of kernel launches (graph nodes included) of the last batch call. */
long long cdx_batch_last_launch_count(void);

/* Free the batch state (plans, buffers, streams, graph). */
void cdx_batch_release(void);

#ifdef __cplusplus
}
#endif

#endif /* CUDADECON_GB300_H */
