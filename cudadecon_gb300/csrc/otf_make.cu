// OTF generation on the GPU: makeOTF of the reference's libradialft
// (src/radialft_interface.cpp:95-197).  A PSF stack (a bead) becomes the
// radially averaged complex OTF table that RL_interface_init reads (width
// 2*nz floats, height nx/2+1), or the 3D OTF.
//
// The O(N) steps run on the device: the peak search and the background sum
// of determine_center_and_background (199-262), the background subtraction,
// the 3D R2C transform (this library's FFT passes), the phase shift of
// shift_center (286-319) and the ring sums of radialft (321-381).  Each ring
// bin (kr, kz) is summed by one thread in the reference's loop order (ky,
// then kx), so the sums do not depend on scheduling.  The small table steps
// (division by the counts, Hermitian symmetrisation, cleanup, fixorigin,
// rescale) run on the host in the reference's float / double arithmetic.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <string>
#include <vector>

#include "../../include/cudadecon.h"
#include "decon_common.cuh"
#include "otf_io.h"

namespace cdx {

namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 304;  // 2 per SM on a 152-SM GPU

// Peak search: per block the largest value above 0 and its first index.
__global__ void k_argmax(const float* __restrict__ v, long long n, float* bmax, long long* bidx) {
  __shared__ float sv[kRedThreads];
  __shared__ long long si[kRedThreads];
  float best = 0.f;
  long long bi = -1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float x = v[i];
    if (x > best) {  // strictly larger: the first index keeps ties
      best = x;
      bi = i;
    }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const float o = sv[threadIdx.x + s];
      const long long oi = si[threadIdx.x + s];
      if (oi >= 0 && (si[threadIdx.x] < 0 || o > sv[threadIdx.x] ||
                      (o == sv[threadIdx.x] && oi < si[threadIdx.x]))) {
        sv[threadIdx.x] = o;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    bmax[blockIdx.x] = sv[0];
    bidx[blockIdx.x] = si[0];
  }
}

// Double sum of the first nrows rows (nx floats each) of slice zs.
__global__ void k_rows_sum(const float* __restrict__ v, int nx, int ny, int zs, int nrows,
                           double* part) {
  __shared__ double sd[kRedThreads];
  const long long n = (long long)nrows * nx;
  const float* base = v + (long long)zs * ny * nx;
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += (double)base[i];
  sd[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) sd[threadIdx.x] += sd[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sd[0];
}

__global__ void k_sub(float* v, long long n, float bg) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = __fsub_rn(v[i], bg);
}

// shift_center on the half spectrum in [z][y][kx] order: multiply by
// exp(i phi), phi = dphiz kz + dphiy ky + dphix kx evaluated in float.
__global__ void k_shift_center(float2* b, int nx, int ny, int nz, float dphix, float dphiy,
                               float dphiz) {
  const int nxh = nx / 2 + 1;
  const long long n = (long long)nxh * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % nxh);
    const long long r = i / nxh;
    const int iy = (int)(r % ny);
    const int iz = (int)(r / ny);
    const int ky = iy > ny / 2 ? iy - ny : iy;
    const int kz = iz > nz / 2 ? iz - nz : iz;
    const float phi1 = __fmul_rn(dphiz, (float)kz);
    const float phi2 = __fmul_rn(dphiy, (float)ky);
    const float phi = __fadd_rn(__fadd_rn(phi1, phi2), __fmul_rn(dphix, (float)kx));
    float s, c;
    sincosf(phi, &s, &c);
    const float2 x = b[i];
    b[i] = make_float2(__fsub_rn(__fmul_rn(x.x, c), __fmul_rn(x.y, s)),
                       __fadd_rn(__fmul_rn(x.x, s), __fmul_rn(x.y, c)));
  }
}

// Ring sums: thread (r, kz) adds the half-spectrum values listed for ring r
// (offsets ky*nxh + kx within a z slice, in the reference's loop order).
__global__ void k_ring_sums(const float2* __restrict__ b, int nxh, int ny, int nz,
                            const int* __restrict__ start, const int* __restrict__ offs,
                            float2* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nxh * nz) return;
  const int r = i / nz;
  const int kz = i - r * nz;
  const float2* slice = b + (long long)kz * ny * nxh;
  float2 s = make_float2(0.f, 0.f);
  for (int k = start[r]; k < start[r + 1]; ++k) {
    const float2 v = slice[offs[k]];
    s.x = __fadd_rn(s.x, v.x);
    s.y = __fadd_rn(s.y, v.y);
  }
  out[i] = s;
}

int grid1(long long n) {
  long long b = (n + 255) / 256;
  if (b > 4096) b = 4096;
  if (b < 1) b = 1;
  return (int)b;
}

float fitparabola(float a1, float a2, float a3) {
  // radialft_interface.cpp:270-284
  const float slope = 0.5 * (a3 - a1);
  const float curve = (a3 + a1) - 2 * a2;
  if (curve == 0) return 0.0f;
  const float peak = -slope / curve;
  if (peak > 1.5 || peak < -1.5) return 0.0f;
  return peak;
}

}  // namespace

// Parameters of makeOTF (radialft_interface.cpp:52-58).
struct OtfMakeParams {
  int lambdanm;
  float dz;
  int interpkr;
  bool bUserBackground;
  float background;
  float NA, NIMM, dr;
  int krmax;
  bool bDoCleanup, b3Dout;
};

// The OTF of a PSF stack d_psf ((nz, ny, nx) float32 on the device; it is
// overwritten by the background-subtracted stack).  Fills `out` like the
// reference's output image: radial (w = 2 nz, h = nx/2+1, d = 1) or 3D
// (w = 2 (nx/2+1), h = ny, d = nz).
static int make_otf_device(float* d_psf, int nx, int ny, int nz, const OtfMakeParams& p,
                           HostImage& out, cudaStream_t st) {
  if (nx < 3 || ny < 3 || nz < 3) {
    set_error("makeOTF", "PSF sizes must be at least 3");
    return cudaErrorInvalidValue;
  }
  if (!fft_len_supported(nx) || !fft_len_supported(ny) || !fft_len_supported(nz)) {
    set_error("makeOTF", "PSF sizes must be products of 2, 3, 5 and 7");
    return cudaErrorInvalidValue;
  }
  const long long n = (long long)nx * ny * nz;
  const int nxh = nx / 2 + 1;
  float* d_bmax = nullptr;
  long long* d_bidx = nullptr;
  double* d_part = nullptr;
  float2 *d_S = nullptr, *d_std = nullptr, *d_ring = nullptr;
  int *d_start = nullptr, *d_offs = nullptr;
  FftLen fx, fy, fz;
  const Geom g = make_geom(nx, ny, nz);
  auto cleanup_all = [&]() {
    cudaFree(d_bmax);
    cudaFree(d_bidx);
    cudaFree(d_part);
    cudaFree(d_S);
    cudaFree(d_std);
    cudaFree(d_ring);
    cudaFree(d_start);
    cudaFree(d_offs);
    fft_len_free(fx);
    fft_len_free(fy);
    fft_len_free(fz);
  };
#define OTF_CHECK(x)                    \
  do {                                  \
    cudaError_t e_ = (x);               \
    if (e_ != cudaSuccess) {            \
      set_cuda_error("makeOTF", e_);    \
      cleanup_all();                    \
      return e_;                        \
    }                                   \
  } while (0)
  OTF_CHECK(cudaMalloc(&d_bmax, kRedBlocks * sizeof(float)));
  OTF_CHECK(cudaMalloc(&d_bidx, kRedBlocks * sizeof(long long)));
  OTF_CHECK(cudaMalloc(&d_part, kRedBlocks * sizeof(double)));
  // ---- determine_center_and_background (radialft_interface.cpp:199-262)
  k_argmax<<<kRedBlocks, kRedThreads, 0, st>>>(d_psf, n, d_bmax, d_bidx);
  OTF_CHECK(cudaGetLastError());
  std::vector<float> hmax(kRedBlocks);
  std::vector<long long> hidx(kRedBlocks);
  OTF_CHECK(cudaMemcpyAsync(hmax.data(), d_bmax, kRedBlocks * sizeof(float),
                            cudaMemcpyDeviceToHost, st));
  OTF_CHECK(cudaMemcpyAsync(hidx.data(), d_bidx, kRedBlocks * sizeof(long long),
                            cudaMemcpyDeviceToHost, st));
  OTF_CHECK(cudaStreamSynchronize(st));
  float maxval = 0.f;
  long long mi = -1;
  for (int b = 0; b < kRedBlocks; ++b)
    if (hidx[b] >= 0 && (mi < 0 || hmax[b] > maxval || (hmax[b] == maxval && hidx[b] < mi))) {
      maxval = hmax[b];
      mi = hidx[b];
    }
  int maxi = 0, maxj = 0, maxk = 0;
  if (mi >= 0) {
    maxk = (int)(mi / ((long long)nx * ny));
    const long long rem = mi - (long long)maxk * nx * ny;
    maxi = (int)(rem / nx);
    maxj = (int)(rem - (long long)maxi * nx);
  }
  const int iminus = (maxi - 1 + ny) % ny, iplus = (maxi + 1) % ny;
  const int jminus = (maxj - 1 + nx) % nx, jplus = (maxj + 1) % nx;
  const int kminus = (maxk - 1 + nz) % nz, kplus = (maxk + 1) % nz;
  auto at = [&](int k, int i, int j, float* v) {
    return cudaMemcpyAsync(v, d_psf + ((long long)k * ny + i) * nx + j, sizeof(float),
                           cudaMemcpyDeviceToHost, st);
  };
  float nb[6];
  OTF_CHECK(at(kminus, maxi, maxj, &nb[0]));
  OTF_CHECK(at(kplus, maxi, maxj, &nb[1]));
  OTF_CHECK(at(maxk, iminus, maxj, &nb[2]));
  OTF_CHECK(at(maxk, iplus, maxj, &nb[3]));
  OTF_CHECK(at(maxk, maxi, jminus, &nb[4]));
  OTF_CHECK(at(maxk, maxi, jplus, &nb[5]));
  OTF_CHECK(cudaStreamSynchronize(st));
  float zc = maxk + fitparabola(nb[0], maxval, nb[1]);
  zc += 0.6;
  const float yc = maxi + fitparabola(nb[2], maxval, nb[3]);
  const float xc = maxj + fitparabola(nb[4], maxval, nb[5]);
  float background = p.background;
  if (!p.bUserBackground) {
    // mean over rows y < yc - 20 of slice floor(zc), divided as the
    // reference divides: by (yc - 20) * nx
    int nrows = 0;
    while (nrows < ny && nrows < yc - 20) ++nrows;
    const int zs = (int)floor(zc);
    double sum = 0;
    if (nrows > 0 && zs >= 0 && zs < nz) {
      k_rows_sum<<<kRedBlocks, kRedThreads, 0, st>>>(d_psf, nx, ny, zs, nrows, d_part);
      OTF_CHECK(cudaGetLastError());
      std::vector<double> hp(kRedBlocks);
      OTF_CHECK(cudaMemcpyAsync(hp.data(), d_part, kRedBlocks * sizeof(double),
                                cudaMemcpyDeviceToHost, st));
      OTF_CHECK(cudaStreamSynchronize(st));
      for (double v : hp) sum += v;
    }
    background = sum / ((yc - 20) * nx);
  }
  k_sub<<<grid1(n), 256, 0, st>>>(d_psf, n, background);
  OTF_CHECK(cudaGetLastError());
  // ---- unnormalised 3D R2C (the reference's fftwf_plan_dft_r2c_3d, 135-142)
  if (fft_len_init(fx, nx) || fft_len_init(fy, ny) || fft_len_init(fz, nz)) {
    cleanup_all();
    return cudaErrorInvalidValue;
  }
  const OtfDev none{};
  OTF_CHECK(cudaMalloc(&d_S, sizeof(float2) * (size_t)g.spec_elems()));
  OTF_CHECK(cudaMalloc(&d_std, sizeof(float2) * (size_t)nxh * ny * nz));
  if (launch_x_fwd(g, fx, d_psf, nullptr, nullptr, 0, d_S, st) ||
      launch_y_pass(g, fy, d_S, false, st) || launch_z_pass(g, fz, d_S, none, false, st, true) ||
      launch_spec_to_std(g, d_S, d_std, st)) {
    cleanup_all();
    return cudaErrorLaunchFailure;
  }
  // ---- shift_center (286-319)
  const float dphiz = 2 * M_PI * zc / nz;
  const float dphiy = 2 * M_PI * yc / ny;
  const float dphix = 2 * M_PI * xc / nx;
  k_shift_center<<<grid1((long long)nxh * ny * nz), 256, 0, st>>>(d_std, nx, ny, nz, dphix, dphiy,
                                                                 dphiz);
  OTF_CHECK(cudaGetLastError());
  if (p.b3Dout) {
    // 3D OTF in the reference's in-place R2C layout (150-154)
    out.w = 2 * nxh;
    out.h = ny;
    out.d = nz;
    out.data.assign((size_t)2 * nxh * ny * nz, 0.f);
    OTF_CHECK(cudaMemcpyAsync(out.data.data(), d_std, sizeof(float) * out.data.size(),
                              cudaMemcpyDeviceToHost, st));
    OTF_CHECK(cudaStreamSynchronize(st));
    cleanup_all();
    std::complex<float>* c = reinterpret_cast<std::complex<float>*>(out.data.data());
    if (p.interpkr > 1) {
      // fixorigin on the +/-45 degree lines (445-486)
      std::vector<std::complex<float>> proj(nxh, 0.f);
      for (int z = 0; z < nz; ++z)
        for (int x = 1; x < nxh && x < ny; ++x) {
          proj[x] += c[((size_t)z * ny + x) * nxh + x];
          proj[x] += c[((size_t)z * ny + (ny - x)) * nxh + x];
        }
      const int kx2 = p.interpkr;
      std::complex<double> mean_val = 0, num = 0, den = 0;
      for (int x = 1; x <= kx2 && x < nxh; ++x) mean_val += std::complex<double>(proj[x]);
      mean_val /= kx2;
      const double mean_kx = (kx2 + 1) / 2.;
      for (int x = 1; x <= kx2 && x < nxh; ++x) {
        const std::complex<double> v = proj[x];
        num += (x - mean_kx) * (v - mean_val);
        den += (x - mean_kx) * (x - mean_kx);
      }
      const std::complex<double> origin = mean_val - (num / den) * mean_kx;
      c[0] = std::complex<float>((float)origin.real(), (float)origin.imag());
    }
    // rescale (506-517)
    float valmax = 0.f;
    for (size_t i = 0; i < out.data.size() / 2; ++i) valmax = std::max(valmax, std::abs(c[i]));
    for (float& v : out.data) v /= valmax;
    return 0;
  }
  // ---- radialft (321-381): ring lists in the reference's loop order
  std::vector<int> bin((size_t)ny * nxh, -1), start(nxh + 1, 0), offs;
  for (int iin = 0; iin < ny; ++iin) {
    const int ky = iin > ny / 2 ? iin - ny : iin;
    for (int kx = 0; kx < nxh; ++kx) {
      const float rdist = sqrt((double)(kx * kx + ky * ky));
      if (rdist < nx / 2 + 1) {
        const int r = (int)rint(rdist);
        if (r < nxh) {
          bin[(size_t)iin * nxh + kx] = r;
          ++start[r + 1];
        }
      }
    }
  }
  for (int r = 0; r < nxh; ++r) start[r + 1] += start[r];
  offs.assign(start[nxh], 0);
  {
    std::vector<int> fillp(start.begin(), start.end() - 1);
    for (int iin = 0; iin < ny; ++iin)
      for (int kx = 0; kx < nxh; ++kx) {
        const int r = bin[(size_t)iin * nxh + kx];
        if (r >= 0) offs[fillp[r]++] = iin * nxh + kx;
      }
  }
  const int nbins = nxh * nz;
  OTF_CHECK(cudaMalloc(&d_start, sizeof(int) * (nxh + 1)));
  OTF_CHECK(cudaMalloc(&d_offs, sizeof(int) * std::max<size_t>(offs.size(), 1)));
  OTF_CHECK(cudaMalloc(&d_ring, sizeof(float2) * nbins));
  OTF_CHECK(cudaMemcpyAsync(d_start, start.data(), sizeof(int) * (nxh + 1),
                            cudaMemcpyHostToDevice, st));
  if (!offs.empty())
    OTF_CHECK(cudaMemcpyAsync(d_offs, offs.data(), sizeof(int) * offs.size(),
                              cudaMemcpyHostToDevice, st));
  k_ring_sums<<<(nbins + 127) / 128, 128, 0, st>>>(d_std, nxh, ny, nz, d_start, d_offs, d_ring);
  OTF_CHECK(cudaGetLastError());
  std::vector<std::complex<float>> avg(nbins);
  OTF_CHECK(cudaMemcpyAsync(avg.data(), d_ring, sizeof(float2) * nbins, cudaMemcpyDeviceToHost,
                            st));
  OTF_CHECK(cudaStreamSynchronize(st));
  cleanup_all();
#undef OTF_CHECK
  for (int r = 0; r < nxh; ++r) {
    const int cnt = start[r + 1] - start[r];
    if (cnt > 0)
      for (int kz = 0; kz < nz; ++kz) avg[(size_t)r * nz + kz] /= cnt;
  }
  for (int kx = 0; kx < nxh; ++kx) {
    avg[(size_t)kx * nz] = std::complex<float>(avg[(size_t)kx * nz].real(), 0);
    for (int kz = 1; kz <= nz / 2; ++kz) {
      const size_t i = (size_t)kx * nz + kz, ic = (size_t)kx * nz + (nz - kz);
      avg[i] = (avg[i] + std::conj(avg[ic])) / 2.f;
      avg[ic] = std::conj(avg[i]);
    }
  }
  if (p.bDoCleanup) {
    // cleanup (383-417)
    const float dkr = 1 / (ny * p.dr), dkz = 1 / (nz * p.dz);
    const float lamda = p.lambdanm * 0.001;
    const float sinalpha = p.NA / p.NIMM;
    const float cosalpha = cos(asin(sinalpha));
    float krmax = 2 * p.NA / lamda;
    if (p.krmax * dkr < krmax && p.krmax != 0) krmax = p.krmax * dkr;
    for (int ix = 0; ix < nxh; ++ix) {
      const float kr = ix * dkr;
      if (kr <= krmax) {
        const float beta = asin((p.NA - kr * lamda) / p.NIMM);
        const float kzedge = (p.NIMM / lamda) * (cos(beta) - cosalpha);
        const int kzstart = (int)rint((kzedge / dkz) + 1);
        const int kzend = nz - kzstart;
        for (int iz = std::max(kzstart, 0); iz <= kzend && iz < nz; ++iz) avg[(size_t)ix * nz + iz] = 0;
      } else {
        for (int iz = 0; iz < nz; ++iz) avg[(size_t)ix * nz + iz] = 0;
      }
    }
  }
  int kx2 = p.interpkr;
  if (kx2 > 0) {
    // fixorigin (419-443), retried with fewer points as the reference does
    for (;;) {
      if (kx2 >= nxh) kx2 = nxh - 1;
      bool ok = true;
      const double mean_kx = (kx2 + 1) / 2.;
      for (int z = 0; z < nz && ok; ++z) {
        std::complex<double> mean_val = 0, num = 0, den = 0;
        for (int x = 1; x <= kx2; ++x) mean_val += std::complex<double>(avg[(size_t)x * nz + z]);
        mean_val /= kx2;
        for (int x = 1; x <= kx2; ++x) {
          const std::complex<double> v = avg[(size_t)x * nz + z];
          num += (x - mean_kx) * (v - mean_val);
          den += (x - mean_kx) * (x - mean_kx);
        }
        const std::complex<double> o = mean_val - (num / den) * mean_kx;
        avg[z] = std::complex<float>((float)o.real(), (float)o.imag());
        if (z == 0 && std::abs(avg[z]) <= std::abs(avg[nz + z])) ok = false;
      }
      if (ok) break;
      --kx2;
      if (kx2 < 4) {
        set_error("makeOTF", "#pixels < 4 used in kr=0 extrapolation");
        return cudaErrorInvalidValue;
      }
    }
  }
  // rescale (488-504)
  float valmax = 0;
  for (const auto& v : avg) valmax = std::max(valmax, std::abs(v));
  const float scalefactor = 1 / valmax;
  for (auto& v : avg) v *= scalefactor;
  out.w = 2 * nz;
  out.h = nxh;
  out.d = 1;
  out.data.resize((size_t)2 * nbins);
  memcpy(out.data.data(), avg.data(), sizeof(float) * out.data.size());
  return 0;
}

}  // namespace cdx

using namespace cdx;

extern "C" {

int makeOTF(const char* const ifiles, const char* const ofiles, int lambdanm, float dz,
            int interpkr, bool bUserBackground, float background, float NA, float NIMM, float dr,
            int krmax, bool bDoCleanup, bool b3Dout) {
  HostImage psf;
  std::string err;
  if (!ifiles || !ofiles || !load_image_file(ifiles, psf, err)) {
    set_error("makeOTF: PSF", ifiles ? err.c_str() : "null file name");
    return 1;
  }
  const OtfMakeParams p{lambdanm, dz, interpkr, bUserBackground, background, NA, NIMM,
                        dr,       krmax, bDoCleanup, b3Dout};
  float* d = nullptr;
  cudaStream_t st = nullptr;
  const size_t n = psf.data.size();
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&d, n * sizeof(float)) != cudaSuccess ||
      cudaMemcpy(d, psf.data.data(), n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
    set_cuda_error("makeOTF", cudaGetLastError());
    cudaFree(d);
    if (st) cudaStreamDestroy(st);
    return 1;
  }
  HostImage out;
  const int rc = make_otf_device(d, psf.w, psf.h, psf.d, p, out, st);
  cudaFree(d);
  cudaStreamDestroy(st);
  if (rc) return 1;
  if (!save_float_tiff(ofiles, out, err)) {
    set_error("makeOTF: output", err.c_str());
    return 1;
  }
  return 0;
}

int cdx_make_otf(const float* psf, int nx, int ny, int nz, int lambdanm, float dz, int interpkr,
                 int bUserBackground, float background, float NA, float NIMM, float dr, int krmax,
                 int bDoCleanup, int b3Dout, float* out, size_t capacity, int* out_w, int* out_h,
                 int* out_d) {
  if (!psf || nx < 1 || ny < 1 || nz < 1) {
    set_error("cdx_make_otf", "null PSF or empty sizes");
    return 0;
  }
  const OtfMakeParams p{lambdanm, dz, interpkr, bUserBackground != 0, background, NA, NIMM,
                        dr,       krmax, bDoCleanup != 0, b3Dout != 0};
  const size_t n = (size_t)nx * ny * nz;
  float* d = nullptr;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&d, n * sizeof(float)) != cudaSuccess ||
      cudaMemcpy(d, psf, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
    set_cuda_error("cdx_make_otf", cudaGetLastError());
    cudaFree(d);
    if (st) cudaStreamDestroy(st);
    return 0;
  }
  HostImage img;
  const int rc = make_otf_device(d, nx, ny, nz, p, img, st);
  cudaFree(d);
  cudaStreamDestroy(st);
  if (rc) return 0;
  if (out_w) *out_w = img.w;
  if (out_h) *out_h = img.h;
  if (out_d) *out_d = img.d;
  if (out) {
    if (capacity < img.data.size()) {
      set_error("cdx_make_otf", "output capacity too small");
      return 0;
    }
    memcpy(out, img.data.data(), img.data.size() * sizeof(float));
  }
  return 1;
}

int cdx_save_image(const char* path, int width, int height, int depth, const float* data) {
  if (!path || !data || width < 1 || height < 1 || depth < 1) {
    set_error("cdx_save_image", "null path or data, or empty sizes");
    return 0;
  }
  HostImage img;
  img.w = width;
  img.h = height;
  img.d = depth;
  img.data.assign(data, data + (size_t)width * height * depth);
  std::string err;
  if (!save_float_tiff(path, img, err)) {
    set_error("cdx_save_image", err.c_str());
    return 0;
  }
  return 1;
}

}  // extern "C"
