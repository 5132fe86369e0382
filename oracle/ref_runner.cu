// ORACLE — test infrastructure only.  Only tests/ may load the library built
// from this file; the product never does.
//
// Runs the reference's own CUDA kernels (src/RLgpuImpl.cu,
// src/geometryTransform.cu, src/camcor.cu of scopetools/cudadecon, compiled
// to PTX into oracle/_ref/ by oracle/build.py from the reference's sources)
// through the CUDA driver API, with cuFFT for the FFTs, in the launch
// configurations and order of the reference's host code:
//   ref_rl_iterations  <- the loop of RichardsonLucy_GPU
//                         (src/RL-Biggs-Andrews.cpp:282-367) with
//                         transferConstants / makeOTFarray (RLgpuImpl.cu:74-91,
//                         352-381), filterGPU (156-225), calcLRcore (390-414),
//                         updateCurrEstimate (436-460), calcCurrPrevDiff
//                         (472-499), calcAccelFactor (510-569; partial sums
//                         summed on the host), updatePrediction (635-656)
//   ref_deskew / ref_rotate <- deskew_GPU / rotate_GPU (geometryTransform.cu:33-48, 90-106)
//   ref_camcor         <- setupCamCor / setupData / camcor_GPU (camcor.cu:6-122)
//   ref_affine         <- affine_GPU / affine_GPU_RA (geometryTransform.cu:257-349)
//   ref_session_open / ref_session_step / ref_session_close
//                      <- one RL_interface call's device work
//                         (RichardsonLucy_GPU, src/RL-Biggs-Andrews.cpp:56-450:
//                         background subtraction, the bleach statistic,
//                         deskew, the loop, rotate) on buffers and cuFFT plans
//                         made once, as RL_interface_init makes the plans
// Every entry point returns 1 on success, 0 on failure.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <limits>
#include <string>
#include <vector>

namespace {

CUmodule g_rl = nullptr, g_geo = nullptr, g_cc = nullptr;
std::string g_err;

bool ok_drv(CUresult r, const char* what) {
  if (r == CUDA_SUCCESS) return true;
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g_err = std::string(what) + ": " + (s ? s : "?");
  return false;
}

bool ok_rt(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

CUfunction fn(CUmodule m, const char* name) {
  CUfunction f = nullptr;
  if (!ok_drv(cuModuleGetFunction(&f, m, name), name)) return nullptr;
  return f;
}

bool launch(CUfunction f, dim3 g, dim3 b, unsigned smem, void** args) {
  if (!f) return false;
  return ok_drv(cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, smem, nullptr, args, nullptr),
                "cuLaunchKernel");
}

bool set_const(const char* name, const void* v, size_t n) {
  CUdeviceptr p;
  size_t sz;
  if (!ok_drv(cuModuleGetGlobal(&p, &sz, g_rl, name), name)) return false;
  return ok_drv(cuMemcpyHtoD(p, v, n), "cuMemcpyHtoD");
}

// grid of the reference's 1-D elementwise launches (1024 threads per block)
dim3 grid1024(size_t n) {
  unsigned nb = (unsigned)ceil(((float)n) / 1024);
  return dim3(nb, 1, 1);
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

int ref_load(const char* dir) {
  if (!ok_rt(cudaFree(0), "cudaFree(0)")) return 0;
  std::string d(dir);
  if (!g_rl && !ok_drv(cuModuleLoad(&g_rl, (d + "/RLgpuImpl.ptx").c_str()), "load RLgpuImpl.ptx"))
    return 0;
  if (!g_geo &&
      !ok_drv(cuModuleLoad(&g_geo, (d + "/geometryTransform.ptx").c_str()), "load geometry"))
    return 0;
  if (!g_cc && !ok_drv(cuModuleLoad(&g_cc, (d + "/camcor.ptx").c_str()), "load camcor.ptx"))
    return 0;
  return 1;
}

// deskew_GPU: block 128, grid (ceil(newNx/128), ny, nz)
int ref_deskew(float* in, int nx, int ny, int nz, double deskewFactor, float* out, int newNx,
               int extraShift, float padVal) {
  CUfunction f = fn(g_geo, "_Z13deskew_kernelPfiiiS_iidf");
  void* args[] = {&in, &nx, &ny, &nz, &out, &newNx, &extraShift, &deskewFactor, &padVal};
  unsigned nxb = (unsigned)ceil(newNx / (float)128);
  return launch(f, dim3(nxb, ny, nz), dim3(128), 0, args) &&
         ok_rt(cudaDeviceSynchronize(), "sync");
}

// rotate_GPU: the matrix lives in device memory
int ref_rotate(float* in, int nx, int ny, int nz, const float* rot_host, float* out, int nx_out,
               int nz_out) {
  float* d_rot = nullptr;
  if (!ok_rt(cudaMalloc(&d_rot, 4 * sizeof(float)), "cudaMalloc")) return 0;
  cudaMemcpy(d_rot, rot_host, 4 * sizeof(float), cudaMemcpyHostToDevice);
  CUfunction f = fn(g_geo, "_Z13rotate_kernelPfiiiS_iiS_");
  void* args[] = {&in, &nx, &ny, &nz, &out, &nx_out, &nz_out, &d_rot};
  unsigned nxb = (unsigned)ceil(nx_out / (float)128);
  bool ok = launch(f, dim3(nxb, ny, nz_out), dim3(128), 0, args) &&
            ok_rt(cudaDeviceSynchronize(), "sync");
  cudaFree(d_rot);
  return ok;
}

// affine_GPU / affine_GPU_RA with the input in a 3D array and a linear,
// border-addressed texture; host in, host out.
int ref_affine(const float* h_in, int nx, int ny, int nz, const float* mat16, int ra, float dx,
               float dy, float dz, float* h_out) {
  cudaChannelFormatDesc cd = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
  cudaArray* arr = nullptr;
  cudaExtent ext = make_cudaExtent(nx, ny, nz);
  if (!ok_rt(cudaMalloc3DArray(&arr, &cd, ext, cudaArrayDefault), "cudaMalloc3DArray")) return 0;
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof(p));
  p.srcPtr = make_cudaPitchedPtr((void*)h_in, nx * sizeof(float), nx, ny);
  p.dstArray = arr;
  p.extent = ext;
  p.kind = cudaMemcpyHostToDevice;
  cudaMemcpy3D(&p);
  cudaResourceDesc rd;
  memset(&rd, 0, sizeof(rd));
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = arr;
  cudaTextureDesc td;
  memset(&td, 0, sizeof(td));
  td.readMode = cudaReadModeElementType;
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
  td.filterMode = cudaFilterModeLinear;
  td.normalizedCoords = false;
  cudaTextureObject_t tex = 0;
  cudaCreateTextureObject(&tex, &rd, &td, nullptr);
  float *d_out = nullptr, *d_mat = nullptr;
  cudaMalloc(&d_out, (size_t)nx * ny * nz * sizeof(float));
  cudaMalloc(&d_mat, 16 * sizeof(float));
  cudaMemcpy(d_mat, mat16, 16 * sizeof(float), cudaMemcpyHostToDevice);
  dim3 blk(16, 16, 4);
  dim3 grd((nx + blk.x - 1) / blk.x, (ny + blk.y - 1) / blk.y, (nz + blk.z - 1) / blk.z);
  unsigned long long t = tex;
  bool ok;
  if (ra) {
    void* args[] = {&d_out, &nx, &ny, &nz, &dx, &dy, &dz, &d_mat, &t};
    ok = launch(fn(g_geo, "_Z17transformKernelRAPfiiifffS_y"), grd, blk, 0, args);
  } else {
    void* args[] = {&d_out, &nx, &ny, &nz, &d_mat, &t};
    ok = launch(fn(g_geo, "_Z15transformKernelPfiiiS_y"), grd, blk, 0, args);
  }
  ok = ok && ok_rt(cudaMemcpy(h_out, d_out, (size_t)nx * ny * nz * sizeof(float),
                              cudaMemcpyDeviceToHost),
                   "copy back");
  cudaDestroyTextureObject(tex);
  cudaFreeArray(arr);
  cudaFree(d_out);
  cudaFree(d_mat);
  return ok;
}

// setupCamCor + setupData + camcor_GPU (camcor.cu:6-122); raw is widened to
// unsigned on the host as the reference's caller does (llspy.cpp:84).
int ref_camcor(const unsigned short* h_raw, int nx, int ny, int nz, const float* h_camparam,
               unsigned short* h_out) {
  // parameter texture: (nx, ny, 3) float, border, point, unnormalised
  cudaChannelFormatDesc cdf = cudaCreateChannelDesc<float>();
  cudaArray *pa = nullptr, *da = nullptr;
  if (!ok_rt(cudaMalloc3DArray(&pa, &cdf, make_cudaExtent(nx, ny, 3)), "param array")) return 0;
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof(p));
  p.srcPtr = make_cudaPitchedPtr((void*)h_camparam, nx * sizeof(float), nx, ny);
  p.dstArray = pa;
  p.extent = make_cudaExtent(nx, ny, 3);
  p.kind = cudaMemcpyHostToDevice;
  cudaMemcpy3D(&p);
  cudaResourceDesc rd = {};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = pa;
  cudaTextureDesc td;
  memset(&td, 0, sizeof(td));
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
  td.filterMode = cudaFilterModePoint;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 0;
  cudaTextureObject_t tp = 0, tdta = 0;
  cudaCreateTextureObject(&tp, &rd, &td, nullptr);
  // data texture: (nx, ny, nz) unsigned, wrap, point, normalised
  std::vector<unsigned> wide((size_t)nx * ny * nz);
  for (size_t i = 0; i < wide.size(); ++i) wide[i] = h_raw[i];
  cudaChannelFormatDesc cdu = cudaCreateChannelDesc<unsigned>();
  if (!ok_rt(cudaMalloc3DArray(&da, &cdu, make_cudaExtent(nx, ny, nz)), "data array")) return 0;
  memset(&p, 0, sizeof(p));
  p.srcPtr = make_cudaPitchedPtr(wide.data(), nx * sizeof(unsigned), nx, ny);
  p.dstArray = da;
  p.extent = make_cudaExtent(nx, ny, nz);
  p.kind = cudaMemcpyHostToDevice;
  cudaMemcpy3D(&p);
  cudaResourceDesc rd2 = {};
  rd2.resType = cudaResourceTypeArray;
  rd2.res.array.array = da;
  cudaTextureDesc td2 = {};
  td2.addressMode[0] = td2.addressMode[1] = td2.addressMode[2] = cudaAddressModeWrap;
  td2.filterMode = cudaFilterModePoint;
  td2.readMode = cudaReadModeElementType;
  td2.normalizedCoords = 1;
  cudaCreateTextureObject(&tdta, &rd2, &td2, nullptr);
  unsigned short* d_out = nullptr;
  cudaMalloc(&d_out, (size_t)nx * ny * nz * sizeof(unsigned short));
  unsigned unx = nx, uny = ny, unz = nz;
  unsigned long long a = tp, b = tdta;
  void* args[] = {&unx, &uny, &unz, &a, &b, &d_out};
  dim3 blk(16, 16, 1);
  dim3 grd((nx + 15) / 16, (ny + 15) / 16, nz);
  bool ok = launch(fn(g_cc, "_Z13camcor_kerneljjjyyPt"), grd, blk, 0, args) &&
            ok_rt(cudaMemcpy(h_out, d_out, (size_t)nx * ny * nz * 2, cudaMemcpyDeviceToHost),
                  "copy back");
  cudaDestroyTextureObject(tp);
  cudaDestroyTextureObject(tdta);
  cudaFreeArray(pa);
  cudaFreeArray(da);
  cudaFree(d_out);
  return ok;
}

// The RL iteration loop on device arrays: X (in: starting estimate, out:
// result) and raw (the conditioned stack), both (nz, ny, nx) float.  otf is
// the raw OTF (complex) with the reference's dimensions and k-scales.  When
// lambdas is not NULL the nIter acceleration factors are written to it
// (0 for the first two iterations).
int ref_rl_iterations(float* X, const float* raw, int nx, int ny, int nz, const float* otf_host,
                      int nxotf, int nyotf, int nzotf, float kxs, float kys, float kzs, int nIter,
                      double* lambdas) {
  const size_t N = (size_t)nx * ny * nz;
  const size_t M = (size_t)nz * ny * (nx / 2 + 1);
  const float eps = std::numeric_limits<float>::epsilon();
  // transferConstants (RLgpuImpl.cu:74-91)
  unsigned nxyz = nx * ny * nz;
  if (!set_const("const_nx", &nx, 4) || !set_const("const_ny", &ny, 4) ||
      !set_const("const_nz", &nz, 4) || !set_const("const_nxyz", &nxyz, 4) ||
      !set_const("const_nxotf", &nxotf, 4) || !set_const("const_nyotf", &nyotf, 4) ||
      !set_const("const_nzotf", &nzotf, 4) || !set_const("const_kxscale", &kxs, 4) ||
      !set_const("const_kyscale", &kys, 4) || !set_const("const_kzscale", &kzs, 4) ||
      !set_const("const_eps", &eps, 4))
    return 0;
  float2 *d_rawotf = nullptr, *d_otf = nullptr, *d_fft = nullptr;
  float *CC = nullptr, *rawb = nullptr, *Xm1 = nullptr, *Y = nullptr, *G1 = nullptr, *G2 = nullptr;
  double* d_part = nullptr;
  const size_t notf = (size_t)nxotf * nyotf * nzotf;
  const unsigned nbDot = (unsigned)ceil(((float)N) / 1024 / 2);
  bool ok = ok_rt(cudaMalloc(&d_rawotf, notf * sizeof(float2)), "malloc") &&
            ok_rt(cudaMalloc(&d_otf, M * sizeof(float2)), "malloc") &&
            ok_rt(cudaMalloc(&d_fft, M * sizeof(float2)), "malloc") &&
            ok_rt(cudaMalloc(&CC, N * 4), "malloc") && ok_rt(cudaMalloc(&rawb, N * 4), "malloc") &&
            ok_rt(cudaMalloc(&Xm1, N * 4), "malloc") && ok_rt(cudaMalloc(&Y, N * 4), "malloc") &&
            ok_rt(cudaMalloc(&G1, N * 4), "malloc") && ok_rt(cudaMalloc(&G2, N * 4), "malloc") &&
            ok_rt(cudaMalloc(&d_part, 2 * nbDot * sizeof(double)), "malloc");
  cufftHandle pf = 0, pi = 0;
  if (ok) {
    cudaMemcpy(d_rawotf, otf_host, notf * sizeof(float2), cudaMemcpyHostToDevice);
    cudaMemcpy(rawb, raw, N * 4, cudaMemcpyDeviceToDevice);
    // makeOTFarray (RLgpuImpl.cu:368-381)
    void* a_otf[] = {&d_rawotf, &d_otf};
    unsigned bnx = (unsigned)ceil((nx / 2 + 1) / (float)128);
    ok = launch(fn(g_rl, "_Z19makeOTFarray_kernelP6float2S0_"), dim3(bnx, ny, nz), dim3(128), 0,
                a_otf);
    ok = ok && cufftPlan3d(&pf, nz, ny, nx, CUFFT_R2C) == CUFFT_SUCCESS &&
         cufftPlan3d(&pi, nz, ny, nx, CUFFT_C2R) == CUFFT_SUCCESS;
    if (!ok && g_err.empty()) g_err = "cufftPlan3d failed";
  }
  CUfunction f_scale = fn(g_rl, "_Z12scale_kernelPfd");
  CUfunction f_filt = fn(g_rl, "_Z13filter_kernelP6float2S0_i");
  CUfunction f_filtc = fn(g_rl, "_Z17filterConj_kernelP6float2S0_i");
  CUfunction f_lr = fn(g_rl, "_Z13LRcore_kernelPfS_");
  CUfunction f_est = fn(g_rl, "_Z19currEstimate_kernelPfS_S_");
  CUfunction f_diff = fn(g_rl, "_Z19currPrevDiff_kernelPfS_S_");
  CUfunction f_dot = fn(g_rl, "_Z19innerProduct_kernelPfS_Pd");
  CUfunction f_pred = fn(g_rl, "_Z23updatePrediction_kernelPfS_S_f");
  auto filter = [&](bool conj) -> bool {
    // filterGPU (RLgpuImpl.cu:156-225)
    double factor = 1. / (nx * ny * nz);
    void* a1[] = {&CC, &factor};
    if (!launch(f_scale, grid1024(N), dim3(1024), 0, a1)) return false;
    if (cufftExecR2C(pf, CC, (cufftComplex*)d_fft) != CUFFT_SUCCESS) {
      g_err = "cufftExecR2C";
      return false;
    }
    int msz = (int)M;
    void* a2[] = {&d_fft, &d_otf, &msz};
    if (!launch(conj ? f_filtc : f_filt, grid1024(M), dim3(1024), 0, a2)) return false;
    if (cufftExecC2R(pi, (cufftComplex*)d_fft, CC) != CUFFT_SUCCESS) {
      g_err = "cufftExecC2R";
      return false;
    }
    return true;
  };
  std::vector<double> part(2 * nbDot);
  for (int k = 0; ok && k < nIter; ++k) {
    double lambda = 0;
    if (k > 1) {
      // calcAccelFactor (RLgpuImpl.cu:510-569)
      void* a[] = {&G1, &G2, &d_part};
      ok = launch(f_dot, dim3(nbDot), dim3(1024), 1024 * sizeof(double) * 2, a) &&
           ok_rt(cudaMemcpy(part.data(), d_part, part.size() * sizeof(double),
                            cudaMemcpyDeviceToHost),
                 "partials");
      if (!ok) break;
      double num = 0, den = 0;
      for (unsigned i = 0; i < nbDot; ++i) {
        num += part[i];
        den += part[i + nbDot];
      }
      lambda = num / (den + eps);
      lambda = std::max(std::min(lambda, 1.), 0.);
      float lf = (float)lambda;
      void* ap[] = {&Y, &X, &Xm1, &lf};
      ok = launch(f_pred, grid1024(N), dim3(1024), 0, ap);
    } else {
      ok = ok_rt(cudaMemcpy(Y, X, N * 4, cudaMemcpyDeviceToDevice), "copy");
    }
    if (lambdas) lambdas[k] = lambda;
    ok = ok && ok_rt(cudaMemcpy(Xm1, X, N * 4, cudaMemcpyDeviceToDevice), "copy");
    if (ok && k > 0) ok = ok_rt(cudaMemcpy(G2, G1, N * 4, cudaMemcpyDeviceToDevice), "copy");
    ok = ok && ok_rt(cudaMemcpy(CC, Y, N * 4, cudaMemcpyDeviceToDevice), "copy") && filter(false);
    void* alr[] = {&CC, &rawb};
    ok = ok && launch(f_lr, grid1024(N), dim3(1024), 0, alr) && filter(true);
    void* ae[] = {&X, &CC, &Y};
    ok = ok && launch(f_est, grid1024(N), dim3(1024), 0, ae);
    void* ad[] = {&X, &Y, &G1};
    ok = ok && launch(f_diff, grid1024(N), dim3(1024), 0, ad);
  }
  ok = ok && ok_rt(cudaDeviceSynchronize(), "sync");
  if (pf) cufftDestroy(pf);
  if (pi) cufftDestroy(pi);
  cudaFree(d_rawotf);
  cudaFree(d_otf);
  cudaFree(d_fft);
  cudaFree(CC);
  cudaFree(rawb);
  cudaFree(Xm1);
  cudaFree(Y);
  cudaFree(G1);
  cudaFree(G2);
  cudaFree(d_part);
  return ok ? 1 : 0;
}


// ---------------------------------------------------------------- session
// One RL_interface call's device work, for timing the reference's own GPU
// path: buffers and plans are made once (the reference allocates its
// buffers on every call, RL-Biggs-Andrews.cpp:92-96, 211-260, which this
// leaves out in the reference's favour).
namespace {
struct RefSession {
  bool open = false;
  int nx_raw = 0, ny = 0, nz = 0, nx = 0;  // raw grid and deskewed (decon) width
  int nxotf = 0, nyotf = 0, nzotf = 0;
  float kxs = 0.f, kys = 0.f, kzs = 0.f;
  double deskew = 0.0;
  int nx_rot = 0, nz_rot = 0;
  size_t N = 0, M = 0, Nraw = 0;
  float2 *rawotf = nullptr, *otf = nullptr, *fft = nullptr;
  float *X0 = nullptr, *X = nullptr, *CC = nullptr, *rawb = nullptr, *Xm1 = nullptr, *Y = nullptr;
  float *G1 = nullptr, *G2 = nullptr, *rot = nullptr;
  double* part = nullptr;
  double* intres = nullptr;
  unsigned* counter = nullptr;
  unsigned nbDot = 0, nbSum = 0;
  cufftHandle pf = 0, pi = 0;
  std::vector<double> hpart, hsum;
  std::vector<unsigned> hcnt;
};
std::vector<RefSession> g_sessions;

void session_free(RefSession& s) {
  if (s.pf) cufftDestroy(s.pf);
  if (s.pi) cufftDestroy(s.pi);
  void* bufs[] = {s.rawotf, s.otf, s.fft, s.X0,   s.X,      s.CC,      s.rawb,
                  s.Xm1,    s.Y,   s.G1,  s.G2,   s.rot,    s.part,    s.intres,
                  s.counter};
  for (void* b : bufs)
    if (b) cudaFree(b);
  s = RefSession{};
}

RefSession* session(int h) {
  if (h < 0 || h >= (int)g_sessions.size() || !g_sessions[h].open) {
    g_err = "no such session";
    return nullptr;
  }
  return &g_sessions[h];
}
}  // namespace

void ref_session_close(int h) {
  if (h >= 0 && h < (int)g_sessions.size()) session_free(g_sessions[h]);
}

// nx_raw, ny, nz: the cropped raw grid; deskewFactor / nx_desk as
// RL_interface_init computes them (nx_desk = nx_raw when deskewFactor is 0);
// rot4: the rotation matrix, or NULL for no rotation (then nx_rot, nz_rot
// are ignored).  Returns a session handle (>= 0), or -1.  Each session holds
// its own buffers, cuFFT plans and OTF array, as one RL_interface_init
// state of the reference; the constants of the reference kernels are set
// again by every step.
int ref_session_open(int nx_raw, int ny, int nz, double deskewFactor, int nx_desk,
                     const float* otf_host, int nxotf, int nyotf, int nzotf, float kxs, float kys,
                     float kzs, const float* rot4, int nx_rot, int nz_rot) {
  int h = 0;
  while (h < (int)g_sessions.size() && g_sessions[h].open) ++h;
  if (h == (int)g_sessions.size()) g_sessions.emplace_back();
  RefSession& s = g_sessions[h];
  s = RefSession{};
  s.nxotf = nxotf;
  s.nyotf = nyotf;
  s.nzotf = nzotf;
  s.kxs = kxs;
  s.kys = kys;
  s.kzs = kzs;
  s.nx_raw = nx_raw;
  s.ny = ny;
  s.nz = nz;
  s.deskew = deskewFactor;
  s.nx = fabs(deskewFactor) > 0.0 ? nx_desk : nx_raw;
  s.nx_rot = rot4 ? nx_rot : 0;
  s.nz_rot = rot4 ? nz_rot : 0;
  s.N = (size_t)s.nx * ny * nz;
  s.M = (size_t)nz * ny * (s.nx / 2 + 1);
  s.Nraw = (size_t)nx_raw * ny * nz;
  const int nx = s.nx;
  const float eps = std::numeric_limits<float>::epsilon();
  unsigned nxyz = (unsigned)s.N;
  if (!set_const("const_nx", &nx, 4) || !set_const("const_ny", &ny, 4) ||
      !set_const("const_nz", &nz, 4) || !set_const("const_nxyz", &nxyz, 4) ||
      !set_const("const_nxotf", &nxotf, 4) || !set_const("const_nyotf", &nyotf, 4) ||
      !set_const("const_nzotf", &nzotf, 4) || !set_const("const_kxscale", &kxs, 4) ||
      !set_const("const_kyscale", &kys, 4) || !set_const("const_kzscale", &kzs, 4) ||
      !set_const("const_eps", &eps, 4))
    return -1;
  const size_t notf = (size_t)nxotf * nyotf * nzotf;
  s.nbDot = (unsigned)ceil(((float)s.N) / 1024 / 2);
  s.nbSum = (unsigned)ceil(s.Nraw / (float)1024 / 2);
  bool ok = ok_rt(cudaMalloc(&s.rawotf, notf * sizeof(float2)), "malloc") &&
            ok_rt(cudaMalloc(&s.otf, s.M * sizeof(float2)), "malloc") &&
            ok_rt(cudaMalloc(&s.fft, s.M * sizeof(float2)), "malloc") &&
            ok_rt(cudaMalloc(&s.X0, s.Nraw * 4), "malloc") &&
            ok_rt(cudaMalloc(&s.X, s.N * 4), "malloc") && ok_rt(cudaMalloc(&s.CC, s.N * 4), "malloc") &&
            ok_rt(cudaMalloc(&s.rawb, s.N * 4), "malloc") &&
            ok_rt(cudaMalloc(&s.Xm1, s.N * 4), "malloc") && ok_rt(cudaMalloc(&s.Y, s.N * 4), "malloc") &&
            ok_rt(cudaMalloc(&s.G1, s.N * 4), "malloc") && ok_rt(cudaMalloc(&s.G2, s.N * 4), "malloc") &&
            ok_rt(cudaMalloc(&s.part, 2 * s.nbDot * sizeof(double)), "malloc") &&
            ok_rt(cudaMalloc(&s.intres, s.nbSum * sizeof(double)), "malloc") &&
            ok_rt(cudaMalloc(&s.counter, s.nbSum * sizeof(unsigned)), "malloc") &&
            (!rot4 || ok_rt(cudaMalloc(&s.rot, 4 * sizeof(float)), "malloc"));
  if (ok && rot4) ok = ok_rt(cudaMemcpy(s.rot, rot4, 16, cudaMemcpyHostToDevice), "rot");
  if (ok) {
    ok = ok_rt(cudaMemcpy(s.rawotf, otf_host, notf * sizeof(float2), cudaMemcpyHostToDevice),
               "otf");
    void* a_otf[] = {&s.rawotf, &s.otf};
    unsigned bnx = (unsigned)ceil((nx / 2 + 1) / (float)128);
    ok = ok && launch(fn(g_rl, "_Z19makeOTFarray_kernelP6float2S0_"), dim3(bnx, ny, nz),
                      dim3(128), 0, a_otf);
    ok = ok && cufftPlan3d(&s.pf, nz, ny, nx, CUFFT_R2C) == CUFFT_SUCCESS &&
         cufftPlan3d(&s.pi, nz, ny, nx, CUFFT_C2R) == CUFFT_SUCCESS;
    if (!ok && g_err.empty()) g_err = "cufftPlan3d failed";
  }
  ok = ok && ok_rt(cudaDeviceSynchronize(), "sync");
  s.hpart.resize(2 * s.nbDot);
  s.hsum.resize(s.nbSum);
  s.hcnt.resize(s.nbSum);
  if (!ok) {
    session_free(s);
    return -1;
  }
  s.open = true;
  return h;
}

// transferConstants for session s (RLgpuImpl.cu:74-91)
static bool session_constants(const RefSession& s) {
  const int nx = s.nx, ny = s.ny, nz = s.nz;
  const unsigned nxyz = (unsigned)s.N;
  const float eps = std::numeric_limits<float>::epsilon();
  return set_const("const_nx", &nx, 4) && set_const("const_ny", &ny, 4) &&
         set_const("const_nz", &nz, 4) && set_const("const_nxyz", &nxyz, 4) &&
         set_const("const_nxotf", &s.nxotf, 4) && set_const("const_nyotf", &s.nyotf, 4) &&
         set_const("const_nzotf", &s.nzotf, 4) && set_const("const_kxscale", &s.kxs, 4) &&
         set_const("const_kyscale", &s.kys, 4) && set_const("const_kzscale", &s.kzs, 4) &&
         set_const("const_eps", &eps, 4);
}

// One call: raw (device, the cropped (nz, ny, nx_raw) stack as float, which
// the reference converts on the host) -> out (device, the rotated result, or
// the deskewed decon grid without rotation).  Returns after the device work.
int ref_session_step(int h, const float* d_raw, float background, int nIter, float* d_out) {
  RefSession* sp = session(h);
  if (!sp) return 0;
  RefSession& s = *sp;
  if (!session_constants(s)) return 0;
  const size_t N = s.N, M = s.M;
  const float eps = std::numeric_limits<float>::epsilon();
  // X_k <- raw (the reference's H2D), backgroundSubtraction_GPU (RLgpuImpl.cu:134-154)
  bool ok = ok_rt(cudaMemcpyAsync(s.X0, d_raw, s.Nraw * 4, cudaMemcpyDeviceToDevice), "copy");
  {
    size_t n = s.Nraw;
    void* a[] = {&s.X0, &n, &background};
    ok = ok && launch(fn(g_rl, "_Z14bgsubtr_kernelPfmf"), grid1024(s.Nraw), dim3(1024), 0, a);
  }
  // meanAboveBackground_GPU (RLgpuImpl.cu:668-718): computed on every call
  if (ok) {
    int n = (int)s.Nraw;
    void* a1[] = {&s.X0, &s.intres, &n};
    ok = launch(fn(g_rl, "_Z16summation_kernelPfPdi"), dim3(s.nbSum), dim3(1024),
                1024 * sizeof(double), a1) &&
         ok_rt(cudaMemcpy(s.hsum.data(), s.intres, s.nbSum * sizeof(double),
                          cudaMemcpyDeviceToHost),
               "sum");
    double sum = 0;
    for (double v : s.hsum) sum += v;
    float mean = (float)(sum / (double)s.Nraw);
    void* a2[] = {&s.X0, &s.intres, &s.counter, &mean, &n};
    ok = ok &&
         launch(fn(g_rl, "_Z21sumAboveThresh_kernelPfPdPjfi"), dim3(s.nbSum), dim3(1024),
                1024 * (sizeof(double) + sizeof(unsigned)), a2) &&
         ok_rt(cudaMemcpy(s.hcnt.data(), s.counter, s.nbSum * sizeof(unsigned),
                          cudaMemcpyDeviceToHost),
               "count") &&
         ok_rt(cudaMemcpy(s.hsum.data(), s.intres, s.nbSum * sizeof(double),
                          cudaMemcpyDeviceToHost),
               "sum");
  }
  // deskew_GPU (geometryTransform.cu:33-48) into the decon grid
  if (ok && fabs(s.deskew) > 0.0) {
    int nxr = s.nx_raw, ny = s.ny, nz = s.nz, nxo = s.nx, shift = 0;
    double f = s.deskew;
    float pad = 0.f;
    void* a[] = {&s.X0, &nxr, &ny, &nz, &s.X, &nxo, &shift, &f, &pad};
    unsigned nxb = (unsigned)ceil(nxo / (float)128);
    ok = launch(fn(g_geo, "_Z13deskew_kernelPfiiiS_iidf"), dim3(nxb, ny, nz), dim3(128), 0, a);
  } else if (ok) {
    ok = ok_rt(cudaMemcpyAsync(s.X, s.X0, N * 4, cudaMemcpyDeviceToDevice), "copy");
  }
  ok = ok && ok_rt(cudaMemcpyAsync(s.rawb, s.X, N * 4, cudaMemcpyDeviceToDevice), "copy");
  CUfunction f_scale = fn(g_rl, "_Z12scale_kernelPfd");
  CUfunction f_filt = fn(g_rl, "_Z13filter_kernelP6float2S0_i");
  CUfunction f_filtc = fn(g_rl, "_Z17filterConj_kernelP6float2S0_i");
  CUfunction f_lr = fn(g_rl, "_Z13LRcore_kernelPfS_");
  CUfunction f_est = fn(g_rl, "_Z19currEstimate_kernelPfS_S_");
  CUfunction f_diff = fn(g_rl, "_Z19currPrevDiff_kernelPfS_S_");
  CUfunction f_dot = fn(g_rl, "_Z19innerProduct_kernelPfS_Pd");
  CUfunction f_pred = fn(g_rl, "_Z23updatePrediction_kernelPfS_S_f");
  auto filter = [&](bool conj) -> bool {
    double factor = 1. / (double)N;
    void* a1[] = {&s.CC, &factor};
    if (!launch(f_scale, grid1024(N), dim3(1024), 0, a1)) return false;
    if (cufftExecR2C(s.pf, s.CC, (cufftComplex*)s.fft) != CUFFT_SUCCESS) {
      g_err = "cufftExecR2C";
      return false;
    }
    int msz = (int)M;
    void* a2[] = {&s.fft, &s.otf, &msz};
    if (!launch(conj ? f_filtc : f_filt, grid1024(M), dim3(1024), 0, a2)) return false;
    if (cufftExecC2R(s.pi, (cufftComplex*)s.fft, s.CC) != CUFFT_SUCCESS) {
      g_err = "cufftExecC2R";
      return false;
    }
    return true;
  };
  for (int k = 0; ok && k < nIter; ++k) {
    if (k > 1) {
      void* a[] = {&s.G1, &s.G2, &s.part};
      ok = launch(f_dot, dim3(s.nbDot), dim3(1024), 1024 * sizeof(double) * 2, a) &&
           ok_rt(cudaMemcpy(s.hpart.data(), s.part, s.hpart.size() * sizeof(double),
                            cudaMemcpyDeviceToHost),
                 "partials");
      if (!ok) break;
      double num = 0, den = 0;
      for (unsigned i = 0; i < s.nbDot; ++i) {
        num += s.hpart[i];
        den += s.hpart[i + s.nbDot];
      }
      double lambda = num / (den + eps);
      lambda = std::max(std::min(lambda, 1.), 0.);
      float lf = (float)lambda;
      void* ap[] = {&s.Y, &s.X, &s.Xm1, &lf};
      ok = launch(f_pred, grid1024(N), dim3(1024), 0, ap);
    } else {
      ok = ok_rt(cudaMemcpyAsync(s.Y, s.X, N * 4, cudaMemcpyDeviceToDevice), "copy");
    }
    ok = ok && ok_rt(cudaMemcpyAsync(s.Xm1, s.X, N * 4, cudaMemcpyDeviceToDevice), "copy");
    if (ok && k > 0) ok = ok_rt(cudaMemcpyAsync(s.G2, s.G1, N * 4, cudaMemcpyDeviceToDevice), "copy");
    ok = ok && ok_rt(cudaMemcpyAsync(s.CC, s.Y, N * 4, cudaMemcpyDeviceToDevice), "copy") &&
         filter(false);
    void* alr[] = {&s.CC, &s.rawb};
    ok = ok && launch(f_lr, grid1024(N), dim3(1024), 0, alr) && filter(true);
    void* ae[] = {&s.X, &s.CC, &s.Y};
    ok = ok && launch(f_est, grid1024(N), dim3(1024), 0, ae);
    void* ad[] = {&s.X, &s.Y, &s.G1};
    ok = ok && launch(f_diff, grid1024(N), dim3(1024), 0, ad);
  }
  // rotate_GPU (geometryTransform.cu:90-106)
  if (ok && s.rot) {
    int nx = s.nx, ny = s.ny, nz = s.nz, nxo = s.nx_rot, nzo = s.nz_rot;
    void* a[] = {&s.X, &nx, &ny, &nz, &d_out, &nxo, &nzo, &s.rot};
    unsigned nxb = (unsigned)ceil(nxo / (float)128);
    ok = launch(fn(g_geo, "_Z13rotate_kernelPfiiiS_iiS_"), dim3(nxb, ny, nzo), dim3(128), 0, a);
  } else if (ok) {
    ok = ok_rt(cudaMemcpyAsync(d_out, s.X, N * 4, cudaMemcpyDeviceToDevice), "copy");
  }
  return ok && ok_rt(cudaDeviceSynchronize(), "sync") ? 1 : 0;
}

}  // extern "C"
