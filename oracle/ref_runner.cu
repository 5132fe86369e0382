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

}  // extern "C"
