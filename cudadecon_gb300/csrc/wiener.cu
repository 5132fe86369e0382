// One-step Wiener filter, the reference's alternative to RL (linearDecon.cpp:
// 116-168 wienerfilter with otfinterpolate 78-114, applied at 1116-1127).
// Filtering the spectrum by conj(OTF) (1 - kr/kcut) / (|OTF|^2 + w^2) inside
// the lateral cutoff (0 outside) is a convolution, so it runs as the RL
// convolution passes with this per-frequency factor, built here once per
// call in the spectrum layout with the 1/N of the inverse transform folded in.
#include "kernels.h"

namespace cdx {

__global__ void k_wiener_h(Geom g, const float2* __restrict__ otf, int nr, int nzotf, float dkx,
                           float dky, float kxscale, float kyscale, float kzscale, float rcutoff,
                           float w, float invN, float2* __restrict__ H) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y;
  const int j = blockIdx.z;  // kx
  if (y >= g.ny) return;
  const float kz = (float)(z > g.nz / 2 ? z - g.nz : z);
  const float ky = (float)(y > g.ny / 2 ? y - g.ny : y);
  const float kx = (float)j;
  // kr = sqrt(kx*kx*dkx*dkx + ky*ky*dky*dky), evaluated left to right in float
  const float kr = sqrtf(__fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(kx, kx), dkx), dkx),
                                   __fmul_rn(__fmul_rn(__fmul_rn(ky, ky), dky), dky)));
  float2 h = make_float2(0.f, 0.f);
  if (kr <= rcutoff) {
    // otfinterpolate: bilinear in (kr, kz) over the radial table, kz wrapping
    const float fx = __fmul_rn(kx, kxscale), fy = __fmul_rn(ky, kyscale);
    const float fz = __fmul_rn(kz, kzscale);
    const float krindex = sqrtf(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)));
    const float kzindex = fz < 0.f ? __fadd_rn(fz, (float)nzotf) : fz;
    float2 o = make_float2(0.f, 0.f);
    if (krindex < (float)(nr - 1) && kzindex < (float)nzotf) {
      const int ir = (int)floorf(krindex);
      const int iz = (int)floorf(kzindex);
      const float ar = __fsub_rn(krindex, (float)ir), az = __fsub_rn(kzindex, (float)iz);
      const int iz1 = iz == nzotf - 1 ? 0 : iz + 1;
      const float2 o00 = otf[ir * nzotf + iz], o01 = otf[ir * nzotf + iz1];
      const float2 o10 = otf[(ir + 1) * nzotf + iz], o11 = otf[(ir + 1) * nzotf + iz1];
      const float bz = __fsub_rn(1.f, az), br = __fsub_rn(1.f, ar);
      const float2 a = make_float2(__fadd_rn(__fmul_rn(o00.x, bz), __fmul_rn(o01.x, az)),
                                   __fadd_rn(__fmul_rn(o00.y, bz), __fmul_rn(o01.y, az)));
      const float2 b = make_float2(__fadd_rn(__fmul_rn(o10.x, bz), __fmul_rn(o11.x, az)),
                                   __fadd_rn(__fmul_rn(o10.y, bz), __fmul_rn(o11.y, az)));
      o = make_float2(__fadd_rn(__fmul_rn(br, a.x), __fmul_rn(ar, b.x)),
                      __fadd_rn(__fmul_rn(br, a.y), __fmul_rn(ar, b.y)));
    }
    const float amp2 = __fadd_rn(__fmul_rn(o.x, o.x), __fmul_rn(o.y, o.y));
    const float rho = __fdiv_rn(kr, rcutoff);
    const float s = __fmul_rn(__fdiv_rn(__fsub_rn(1.f, rho), __fadd_rn(amp2, w)), invN);
    h = make_float2(__fmul_rn(o.x, s), __fmul_rn(-o.y, s));  // conj(OTF) * s
  }
  H[(long long)j * g.plane + (long long)z * g.nyp + y] = h;
}

int launch_wiener_h(const Geom& g, const float2* otf, int nr, int nzotf, float dkx, float dky,
                    float kxscale, float kyscale, float kzscale, float rcutoff, float w,
                    float2* H, cudaStream_t st) {
  const float invN = (float)(1.0 / ((double)g.nx * g.ny * g.nz));
  dim3 grid(ceil_div(g.ny, 128), g.nz, g.nxh);
  k_wiener_h<<<grid, 128, 0, st>>>(g, otf, nr, nzotf, dkx, dky, kxscale, kyscale, kzscale,
                                   rcutoff, w, invN, H);
  CDX_LAUNCH_CHECK("k_wiener_h");
  return 0;
}

__global__ void k_minus(const float* __restrict__ in, float* __restrict__ out, long long n,
                        float bg) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = __fsub_rn(in[i], bg);
}

int launch_minus(const float* in, float* out, long long n, float bg, cudaStream_t st) {
  long long b = (n + 255) / 256;
  if (b > 8192) b = 8192;
  k_minus<<<(int)(b < 1 ? 1 : b), 256, 0, st>>>(in, out, n, bg);
  CDX_LAUNCH_CHECK("k_minus");
  return 0;
}

}  // namespace cdx
