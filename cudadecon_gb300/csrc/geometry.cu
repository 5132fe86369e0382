// Geometry and conditioning kernels around the RL loop: u16 load with crop
// and background subtraction, apodization, z blend, stack duplication,
// bleach statistics, deskew, rotate, sCMOS camera correction and the
// texture-filtered affine transform.
//
// Where a result must match the reference bit for bit, the arithmetic
// follows the reference kernel's evaluation exactly: deskew and rotate spell
// out the roundings and fused multiply-adds with intrinsics (pinned against
// the reference's compiled kernels), camcor keeps the reference's operand
// types and expression shape.
#include "kernels.h"

#include <math.h>

namespace cdx {

static inline dim3 grid1d(long long n, int T) {
  long long b = (n + T - 1) / T;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

// ---------------------------------------------------------------- load
// Reference: CImg<float>(raw) + crop at the origin (RL-Biggs-Andrews.cpp:674-677)
// then bgsubtr_kernel (RLgpuImpl.cu:124-132).
__global__ void k_u16_to_f32_crop(const unsigned short* __restrict__ in, int nx_in, int ny_in,
                                  int nx, int ny, int nz, float* __restrict__ out, float bg,
                                  int sub) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const long long r = i / nx;
    const int y = (int)(r % ny);
    const int z = (int)(r / ny);
    float v = (float)in[((long long)z * ny_in + y) * nx_in + x];
    if (sub) {
      v -= bg;
      v = v > 0 ? v : 0;
    }
    out[i] = v;
  }
}

int launch_u16_to_f32_crop(const unsigned short* in, int nx_in, int ny_in, int nx, int ny, int nz,
                           float* out, float background, int subtract_bg, cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  k_u16_to_f32_crop<<<grid1d(n, 256), 256, 0, st>>>(in, nx_in, ny_in, nx, ny, nz, out, background,
                                                    subtract_bg);
  CDX_LAUNCH_CHECK("k_u16_to_f32_crop");
  return 0;
}

__global__ void k_bgsub(float* img, long long n, float bg) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float v = img[i] - bg;
    img[i] = v > 0 ? v : 0;
  }
}

int launch_bgsub(float* img, long long n, float background, cudaStream_t st) {
  k_bgsub<<<grid1d(n, 256), 256, 0, st>>>(img, n, background);
  CDX_LAUNCH_CHECK("k_bgsub");
  return 0;
}

// Reference scale_kernel (RLgpuImpl.cu:383-388) as used by rescale_GPU:
// the product is formed in double and rounded to float.
__global__ void k_scale(float* img, long long n, double factor) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    img[i] *= factor;
}

int launch_scale(float* img, long long n, double factor, cudaStream_t st) {
  k_scale<<<grid1d(n, 256), 256, 0, st>>>(img, n, factor);
  CDX_LAUNCH_CHECK("k_scale");
  return 0;
}

// ---------------------------------------------------------------- apodize
// Cosine taper of napodize edge rows, then columns, towards the opposite
// edge (reference apodize_x_kernel / apodize_y_kernel, RLgpuImpl.cu:864-894).
__global__ void k_apodize_x(int napodize, int nx, int ny, float* image) {
  const int k = blockDim.x * blockIdx.x + threadIdx.x;
  if (k >= nx) return;
  const long long off = (long long)blockIdx.y * nx * ny;
  const float diff = (image[off + (long long)(ny - 1) * nx + k] - image[off + k]) / 2.0;
  for (int l = 0; l < napodize; ++l) {
    const float fact = diff * (1.0 - sin((((float)l + 0.5) / (float)napodize) * M_PI * 0.5));
    image[off + (long long)l * nx + k] += fact;
    image[off + (long long)(ny - 1 - l) * nx + k] -= fact;
  }
}

__global__ void k_apodize_y(int napodize, int nx, int ny, float* image) {
  const int l = blockDim.x * blockIdx.x + threadIdx.x;
  if (l >= ny) return;
  const long long off = (long long)blockIdx.y * nx * ny + (long long)l * nx;
  const float diff = (image[off + nx - 1] - image[off]) / 2.0;
  for (int k = 0; k < napodize; ++k) {
    const float fact = diff * (1.0 - sin(((k + 0.5) / (float)napodize) * M_PI * 0.5));
    image[off + k] += fact;
    image[off + nx - 1 - k] -= fact;
  }
}

int launch_apodize(float* img, int nx, int ny, int nz, int napodize, cudaStream_t st) {
  if (napodize <= 0) return 0;
  // The reference writes outside the slice when napodize exceeds the image;
  // the taper is limited to the image here.
  if (napodize > nx) napodize = nx;
  if (napodize > ny) napodize = ny;
  k_apodize_x<<<dim3(ceil_div(nx, 64), nz), 64, 0, st>>>(napodize, nx, ny, img);
  CDX_LAUNCH_CHECK("k_apodize_x");
  k_apodize_y<<<dim3(ceil_div(ny, 64), nz), 64, 0, st>>>(napodize, nx, ny, img);
  CDX_LAUNCH_CHECK("k_apodize_y");
  return 0;
}

// ---------------------------------------------------------------- z blend
// The reference zBlend_kernel (RLgpuImpl.cu:908-925) indexes the slice with
// blockDim.z (always 1) instead of its block index, so its nZblend blocks
// all update slices 1 and nz-2 with the weight of index 1.  This kernel
// reproduces that result with the nZblend updates applied one after the
// other (the reference's updates race with each other).
__global__ void k_zblend(int nx, int ny, int nz, int nZblend, float* image) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= nx) return;
  const long long nxy = (long long)nx * ny;
  const long long ro = (long long)y * nx + x;
  const unsigned zidx = 1;
  for (int rep = 0; rep < nZblend; ++rep) {
    const float diff = image[(nz - 1) * nxy + ro] - image[ro];
    const float fact = diff * (1.0 - sin(((zidx + 0.5) / (float)nZblend) * M_PI * 0.5));
    image[zidx * nxy + ro] += fact;
    image[(nz - zidx - 1) * nxy + ro] -= fact;
  }
}

int launch_zblend(float* img, int nx, int ny, int nz, int nZblend, cudaStream_t st) {
  if (nZblend <= 0 || nz < 3) return 0;
  k_zblend<<<dim3(ceil_div(nx, 128), ny), 128, 0, st>>>(nx, ny, nz, nZblend, img);
  CDX_LAUNCH_CHECK("k_zblend");
  return 0;
}

// Mirror the stack into a buffer of 2*nz slices (dupRevStack_kernel,
// geometryTransform.cu:152-164).
__global__ void k_dup_rev(float* img, int nx, int ny, int nz) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y, z = blockIdx.z;
  if (x >= nx) return;
  const long long nxy = (long long)nx * ny;
  img[(long long)(2 * nz - z - 1) * nxy + (long long)y * nx + x] =
      img[(long long)z * nxy + (long long)y * nx + x];
}

int launch_dup_rev(float* img, int nx, int ny, int nz, cudaStream_t st) {
  k_dup_rev<<<dim3(ceil_div(nx, 128), ny, nz), 128, 0, st>>>(img, nx, ny, nz);
  CDX_LAUNCH_CHECK("k_dup_rev");
  return 0;
}

// ---------------------------------------------------------------- bleach statistics
// Mean of the voxels above the mean (meanAboveBackground_GPU,
// RLgpuImpl.cu:668-718): sum in double, mean rounded to float, then sum and
// count of voxels strictly above it; returns sum/count.
constexpr int kStatBlocks = 1216;

__global__ void k_sum_above(const float* __restrict__ img, long long n, const double* mean_src,
                            int above, double* partial, unsigned* cnt) {
  __shared__ double sh[32];
  __shared__ unsigned shc[32];
  float thresh = 0.f;
  if (above) thresh = (float)(mean_src[0] / (double)n);
  double s = 0.0;
  unsigned c = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = img[i];
    if (!above) {
      s += v;
    } else if (v > thresh) {
      s += v;
      ++c;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[w] = s;
    shc[w] = c;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    s = l < nw ? sh[l] : 0.0;
    c = l < nw ? shc[l] : 0u;
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (l == 0) {
      partial[blockIdx.x] = s;
      cnt[blockIdx.x] = c;
    }
  }
}

__global__ void k_reduce_partials(const double* partial, const unsigned* cnt, int nb, double* out,
                                  unsigned long long* out_cnt) {
  __shared__ double sh[32];
  __shared__ unsigned long long shc[32];
  double s = 0.0;
  unsigned long long c = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    s += partial[i];
    c += cnt[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[w] = s;
    shc[w] = c;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    s = l < nw ? sh[l] : 0.0;
    c = l < nw ? shc[l] : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (l == 0) {
      out[0] = s;
      if (out_cnt) out_cnt[0] = c;
    }
  }
}

int mean_above_background(const float* img, long long n, double* d_tmp, unsigned* d_cnt,
                          double* result, cudaStream_t st) {
  // d_tmp: kStatBlocks + 2 doubles; d_cnt: kStatBlocks + 2 unsigned (the
  // last two slots of d_cnt hold a 64-bit count)
  double* sums = d_tmp + kStatBlocks;
  unsigned long long* total = reinterpret_cast<unsigned long long*>(d_cnt + kStatBlocks);
  k_sum_above<<<kStatBlocks, 256, 0, st>>>(img, n, nullptr, 0, d_tmp, d_cnt);
  CDX_LAUNCH_CHECK("k_sum_above");
  k_reduce_partials<<<1, 1024, 0, st>>>(d_tmp, d_cnt, kStatBlocks, sums, nullptr);
  CDX_LAUNCH_CHECK("k_reduce_partials");
  k_sum_above<<<kStatBlocks, 256, 0, st>>>(img, n, sums, 1, d_tmp, d_cnt);
  CDX_LAUNCH_CHECK("k_sum_above");
  k_reduce_partials<<<1, 1024, 0, st>>>(d_tmp, d_cnt, kStatBlocks, sums + 1, total);
  CDX_LAUNCH_CHECK("k_reduce_partials");
  double h_sum = 0.0;
  unsigned long long h_cnt = 0;
  CDX_CHECK(cudaMemcpyAsync(&h_sum, sums + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
  CDX_CHECK(cudaMemcpyAsync(&h_cnt, total, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  CDX_CHECK(cudaStreamSynchronize(st));
  *result = h_sum / (double)(unsigned)h_cnt;
  return 0;
}

// ---------------------------------------------------------------- deskew
// Shear along x by deskewFactor*(z - nz/2) with linear interpolation inside
// each x row; padVal outside (reference deskew_kernel, geometryTransform.cu:4-31).
// The arithmetic is written out with intrinsics in the order the reference's
// nvcc build evaluates it (pinned against the reference kernel on the GPU):
// the source coordinate in double with one fused multiply-add, rounded once
// to float; the blend (1-offset)*a + offset*b with the first product fused.
// The source coordinate depends on (xout, zout) only, so each thread
// evaluates it once (in double, as the reference does per voxel) and then
// walks kGeomRows rows of y; GB300's FP64 rate is a small fraction of its
// FP32 rate.
constexpr int kGeomRows = 16;

__global__ void k_deskew(const float* __restrict__ in, int nx, int ny, int nz,
                         float* __restrict__ out, int nxOut, int extraShift, double deskewFactor,
                         float padVal) {
  const unsigned xout = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned zout = blockIdx.y;
  const unsigned y0 = blockIdx.z * kGeomRows;
  if (xout >= (unsigned)nxOut) return;
  const double a = __dadd_rn(__dsub_rn((double)xout, nxOut / 2.), (double)extraShift);
  const double b = __dsub_rn((double)zout, nz / 2.);
  const float xin = __double2float_rn(__dadd_rn(__fma_rn(-deskewFactor, b, a), nx / 2.));
  const unsigned y1 = min(y0 + kGeomRows, (unsigned)ny);
  if (xin >= 0 && xin < nx - 1) {
    const float fl = floorf(xin);
    const float offset = __fsub_rn(xin, fl);
    const float w0 = __fsub_rn(1.f, offset);
    for (unsigned y = y0; y < y1; ++y) {
      const size_t indin = ((size_t)zout * ny + y) * nx + (unsigned int)fl;
      out[((size_t)zout * ny + y) * nxOut + xout] =
          __fmaf_rn(w0, __ldg(in + indin), __fmul_rn(offset, __ldg(in + indin + 1)));
    }
  } else {
    for (unsigned y = y0; y < y1; ++y) out[((size_t)zout * ny + y) * nxOut + xout] = padVal;
  }
}

int launch_deskew(const float* in, int nx, int ny, int nz, double deskewFactor, float* out,
                  int nxOut, int extraShift, float padVal, cudaStream_t st) {
  dim3 grid(ceil_div(nxOut, 128), nz, ceil_div(ny, kGeomRows));
  k_deskew<<<grid, 128, 0, st>>>(in, nx, ny, nz, out, nxOut, extraShift, deskewFactor, padVal);
  CDX_LAUNCH_CHECK("k_deskew");
  return 0;
}

// ---------------------------------------------------------------- rotate
// Rotation about y with bilinear interpolation in (x, z) and the output z
// flipped (reference rotate_kernel, geometryTransform.cu:50-88).  The matrix
// is passed by value.
struct Rot4 {
  float p[4];
};

// Arithmetic written out as the reference's nvcc build evaluates it (pinned
// against the reference kernel on the GPU): each coordinate is
// fmaf(r0, zc, r1*xc) in float, then the half size is added in double and
// the sum rounded to float; each of the three blends fuses its first product.
__global__ void k_rotate(const float* __restrict__ in, int nx_in, int ny, int nz_in,
                         float* __restrict__ out, int nx_out, int nz_out, Rot4 rot) {
  const unsigned xout = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned zout = blockIdx.y;
  const unsigned y0 = blockIdx.z * kGeomRows;
  if (xout >= (unsigned)nx_out) return;
  const float xc = __double2float_rn(__dsub_rn((double)xout, nx_out / 2.));
  const float zc = __double2float_rn(__dsub_rn((double)zout, nz_out / 2.));
  const float zin = __double2float_rn(
      __dadd_rn((double)__fmaf_rn(rot.p[0], zc, __fmul_rn(rot.p[1], xc)), nz_in / 2.));
  const float xin = __double2float_rn(
      __dadd_rn((double)__fmaf_rn(rot.p[2], zc, __fmul_rn(rot.p[3], xc)), nx_in / 2.));
  const size_t nxy_in = (size_t)nx_in * ny;
  const size_t nxy_out = (size_t)nx_out * ny;
  const size_t obase = (size_t)(nz_out - 1 - zout) * nxy_out + xout;
  const unsigned y1 = min(y0 + kGeomRows, (unsigned)ny);
  if (xin >= 0 && xin < nx_in - 1 && zin >= 0 && zin < nz_in - 1) {
    const float fz = floorf(zin), fx = floorf(xin);
    const size_t ibase = (size_t)(unsigned)fz * nxy_in + (unsigned)fx;
    const float xo = __fsub_rn(xin, fx), zo = __fsub_rn(zin, fz);
    const float wx = __fsub_rn(1.f, xo), wz = __fsub_rn(1.f, zo);
    for (unsigned y = y0; y < y1; ++y) {
      const size_t i00 = ibase + (size_t)y * nx_in;
      const size_t i10 = i00 + nxy_in;
      const float a = __fmaf_rn(wx, __ldg(in + i00), __fmul_rn(xo, __ldg(in + i00 + 1)));
      const float b = __fmaf_rn(wx, __ldg(in + i10), __fmul_rn(xo, __ldg(in + i10 + 1)));
      out[obase + (size_t)y * nx_out] = __fmaf_rn(wz, a, __fmul_rn(zo, b));
    }
  } else {
    for (unsigned y = y0; y < y1; ++y) out[obase + (size_t)y * nx_out] = 0.f;
  }
}

int launch_rotate(const float* in, int nx_in, int ny, int nz_in, const float* rot_host, float* out,
                  int nx_out, int nz_out, cudaStream_t st) {
  Rot4 r;
  for (int i = 0; i < 4; ++i) r.p[i] = rot_host[i];
  dim3 grid(ceil_div(nx_out, 128), nz_out, ceil_div(ny, kGeomRows));
  k_rotate<<<grid, 128, 0, st>>>(in, nx_in, ny, nz_in, out, nx_out, nz_out, r);
  CDX_LAUNCH_CHECK("k_rotate");
  return 0;
}

// ---------------------------------------------------------------- camcor
// sCMOS residual-charge correction (reference camcor_kernel, camcor.cu:80-108):
//   out = (u16)(v - offset - 0.9*a*(1 - exp(-b*(v_prev - offset))))
// with a, b, offset the planes 0, 1, 2 of camparam and v_prev the previous z
// slice; slice 0 takes slice nz-1 (the wrap-mode texture fetch of the
// reference).  Plain coalesced loads replace the point-sampled textures.
__global__ void k_camcor(const unsigned short* __restrict__ raw, int nx, int ny, int nz,
                         const float* __restrict__ camparam, unsigned short* __restrict__ output) {
  const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned y = blockIdx.y;
  const unsigned z = blockIdx.z;
  if (x >= (unsigned)nx) return;
  const size_t nxy = (size_t)nx * ny;
  const size_t pix = (size_t)y * nx + x;
  const float a = camparam[pix];
  const float b = camparam[nxy + pix];
  const float offset = camparam[2 * nxy + pix];
  const unsigned voxel = raw[(size_t)z * nxy + pix];
  const unsigned zp = z == 0 ? (unsigned)nz - 1 : z - 1;
  const unsigned previousvoxel = raw[(size_t)zp * nxy + pix];
  const size_t i = (size_t)z * nxy + pix;
  output[i] = (unsigned short)voxel - offset - 0.9f * a * (1 - expf(-b * (previousvoxel - offset)));
}

int launch_camcor(const unsigned short* raw, int nx, int ny, int nz, const float* camparam,
                  unsigned short* out, cudaStream_t st) {
  dim3 grid(ceil_div(nx, 128), ny, nz);
  k_camcor<<<grid, 128, 0, st>>>(raw, nx, ny, nz, camparam, out);
  CDX_LAUNCH_CHECK("k_camcor");
  return 0;
}

__global__ void k_f32_to_u16(const float* __restrict__ in, unsigned short* __restrict__ out,
                             long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (unsigned short)in[i];
}

int launch_f32_to_u16(const float* in, unsigned short* out, long long n, cudaStream_t st) {
  k_f32_to_u16<<<grid1d(n, 256), 256, 0, st>>>(in, out, n);
  CDX_LAUNCH_CHECK("k_f32_to_u16");
  return 0;
}

}  // namespace cdx
