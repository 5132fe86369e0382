// The Richardson-Lucy / Biggs-Andrews hot loop as fused FFT passes.
//
// One iteration of the reference (src/RL-Biggs-Andrews.cpp:282-367) is
//   Y   = k>1 ? max(X + lambda*(X - X_{k-1}), 0) : X        (RLgpuImpl.cu:658-666)
//   CC  = C2R(R2C(Y/N) * OTF)                                (RLgpuImpl.cu:156-225, 331-339)
//   CC  = clamp(raw / (|CC|>0 ? CC : eps) + eps, -10, 10)    (RLgpuImpl.cu:416-434)
//   CC  = C2R(R2C(CC/N) * conj(OTF))                         (RLgpuImpl.cu:341-350)
//   X   = max(CC*Y, 0); G = X - Y                            (RLgpuImpl.cu:462-470, 501-508)
//   lambda_next = (G.G_old)/(G_old.G_old + eps), in [0,1]    (RLgpuImpl.cu:510-633)
// Here it runs as nine kernels: x_fwd (with the prediction prologue), y, z
// (fwd * OTF * inv), y, x_inv+ratio+x_fwd, y, z (conj), y, x_inv+update (with
// the FP64 dot products and an on-device lambda).  The 1/N normalisation is
// folded into the OTF table.  No intermediate real volume is written between
// the two convolutions.
#include "decon_common.cuh"

#include <math.h>
#include <vector>

namespace cdx {

Geom make_geom(int nx, int ny, int nz) {
  Geom g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.nxh = nx / 2 + 1;
  g.nyp = ny + (ny & 1);
  g.plane = (long long)nz * g.nyp;
  return g;
}

// ---------------------------------------------------------------- FFT plans
static bool factorize(int L, std::vector<int>& rad) {
  rad.clear();
  int n = L;
  int p2 = 0;
  while (n % 2 == 0) { n /= 2; ++p2; }
  while (p2 >= 4) { rad.push_back(16); p2 -= 4; }
  if (p2 == 3) rad.push_back(8);
  else if (p2 == 2) rad.push_back(4);
  else if (p2 == 1) rad.push_back(2);
  while (n % 9 == 0) { rad.push_back(9); n /= 9; }
  while (n % 3 == 0) { rad.push_back(3); n /= 3; }
  while (n % 7 == 0) { rad.push_back(7); n /= 7; }
  while (n % 5 == 0) { rad.push_back(5); n /= 5; }
  if (n != 1) return false;
  if ((int)rad.size() > kMaxStages) return false;
  if (rad.empty()) rad.push_back(1);  // L == 1: identity
  return true;
}

bool fft_len_supported(int L) {
  std::vector<int> r;
  return L >= 1 && L <= kMaxFftLen && factorize(L, r);
}

// Fill a device plan for the radix sequence rad and upload its twiddles:
// stage s (radix R, span Ns) holds exp(-2*pi*i*r*k/(Ns*R)) at
// [Ns-1 + (r-1)*Ns + k], computed in double and rounded once to float.
static int build_fft_dev(int L, const std::vector<int>& rad, FftDev& d, float2** d_tw) {
  d.L = L;
  d.nst = (rad.size() == 1 && rad[0] == 1) ? 0 : (int)rad.size();
  std::vector<float2> tw(L, make_float2(1.f, 0.f));
  const double two_pi = 6.283185307179586476925286766559;
  int Ns = 1;
  for (int i = 0; i < kMaxStages; ++i) {
    StageDev& sd = d.st[i];
    if (i < d.nst) {
      const int R = rad[i];
      sd.R = R;
      sd.LR = L / R;
      sd.Ns = Ns;
      sd.toff = Ns - 1;
      sd.invLR = 1.0f / (float)sd.LR;
      sd.invNs = 1.0f / (float)Ns;
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < Ns; ++k) {
          const double a = -two_pi * (double)r * (double)k / ((double)Ns * R);
          tw[sd.toff + (r - 1) * Ns + k] = make_float2((float)cos(a), (float)sin(a));
        }
      Ns *= R;
    } else {
      sd = StageDev{1, L, Ns, 0, 1.0f / (float)L, 1.0f / (float)Ns};
    }
  }
  CDX_CHECK(cudaMalloc(d_tw, sizeof(float2) * L));
  CDX_CHECK(cudaMemcpy(*d_tw, tw.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
  d.tw = *d_tw;
  return 0;
}

int fft_len_init(FftLen& f, int L) {
  std::vector<int> rad;
  if (L < 1 || L > kMaxFftLen || !factorize(L, rad)) {
    set_error("fft_len_init", "length is not a product of 2, 3, 5 and 7");
    return cudaErrorInvalidValue;
  }
  if (int rc = build_fft_dev(L, rad, f.dev, &f.d_tw)) return rc;
  f.has_static = static_radices(L, rad);
  if (f.has_static) {
    if (int rc = build_fft_dev(L, rad, f.sdev, &f.d_tws)) return rc;
  }
  int pairs = 0;
  f.has_xr = xr_radices(L, rad, pairs);
  if (f.has_xr) {
    if (int rc = build_fft_dev(L, rad, f.xrdev, &f.d_twxr)) return rc;
  }
  f.has_gx = gx_radices(L, rad);
  if (f.has_gx) {
    if (int rc = build_fft_dev(L, rad, f.gxdev, &f.d_twgx)) return rc;
  }
  f.has_gz = gz_radices(L, rad);
  if (f.has_gz) {
    if (int rc = build_fft_dev(L, rad, f.gzdev, &f.d_twgz)) return rc;
  }
  int q0 = 0, q1 = 0;
  f.has_tc = tc_plan_radices(L, q0, q1);
  if (f.has_tc) {
    if (int rc = tc_tables_init(f.tc, L)) return rc;
    CDX_CHECK(cudaMalloc(&f.tc.d_err, sizeof(int)));
    CDX_CHECK(cudaMemset(f.tc.d_err, 0, sizeof(int)));
  }
  return 0;
}

int tc_check(const FftLen& f) {
  if (!f.has_tc || !f.tc.d_err) return 0;
  int e = 0;
  CDX_CHECK(cudaMemcpy(&e, f.tc.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    set_error("tensor-core x pass", "a wait on the tensor core ran out (result invalid)");
    return cudaErrorLaunchTimeout;
  }
  return 0;
}

static int g_dft_form = 0;
int dft_form() { return g_dft_form; }
void set_dft_form(int form) { g_dft_form = form; }

void fft_len_free(FftLen& f) {
  if (f.d_tw) cudaFree(f.d_tw);
  if (f.d_tws) cudaFree(f.d_tws);
  if (f.d_twxr) cudaFree(f.d_twxr);
  if (f.d_twgx) cudaFree(f.d_twgx);
  f.d_twgx = nullptr;
  f.gxdev.tw = nullptr;
  f.has_gx = false;
  if (f.d_twgz) cudaFree(f.d_twgz);
  f.d_twgz = nullptr;
  f.gzdev.tw = nullptr;
  f.has_gz = false;
  f.d_tw = nullptr;
  f.d_tws = nullptr;
  f.d_twxr = nullptr;
  f.dev.tw = nullptr;
  f.sdev.tw = nullptr;
  f.xrdev.tw = nullptr;
  f.has_static = false;
  f.has_xr = false;
  if (f.has_tc) tc_tables_free(f.tc);
  f.has_tc = false;
}

// Row pairs per block of the x passes: the registered tile of a compile-time
// plan, else the generic tile.
static int x_tile_pairs(int nx) {
  switch (nx) {
#define CDX_PAIRS_CASE(L, PP) \
  case L:                     \
    return PP;
    CDX_X_PLANS(CDX_PAIRS_CASE)
#undef CDX_PAIRS_CASE
    default:
      return x_pairs(nx);
  }
}

// Blocks of the x pass with the most (the smallest tile): the dot-product
// partials are sized by it.
int x_pass_blocks(const Geom& g) {
  int p = x_tile_pairs(g.nx);
  std::vector<int> rad;
  int pxr = 0;
  if (xr_radices(g.nx, rad, pxr) && pxr < p) p = pxr;
  int pgx = 0;
  if (gx_pairs(g.nx, pgx) && pgx < p) p = pgx;
  return ceil_div(g.ny, 2 * p) * g.nz;
}

__global__ void k_spec_to_std(Geom g, const float2* __restrict__ S, float2* __restrict__ out) {
  const long long n = (long long)g.nz * g.ny * g.nxh;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % g.nxh);
    const long long r = i / g.nxh;
    const int y = (int)(r % g.ny);
    const int z = (int)(r / g.ny);
    out[i] = S[(long long)kx * g.plane + (long long)z * g.nyp + y];
  }
}

int launch_spec_to_std(const Geom& g, const float2* S, float2* out, cudaStream_t st) {
  k_spec_to_std<<<1216, 256, 0, st>>>(g, S, out);
  CDX_LAUNCH_CHECK("k_spec_to_std");
  return 0;
}

// ---------------------------------------------------------------- OTF tables
// Radially averaged OTF resampled along kz for every z frequency of the
// volume: t[z][ir] = otf[ir][iz]*(1-az) + otf[ir][iz+1 (wrapping)]*az, zero
// where kzindex falls outside [0, nz_otf), times scale (= 1/N).  Stored as
// pairs tz[z][ir] = (t[z][ir], t[z][ir+1]) so that the radial interpolation
// of the z pass takes one 16-byte load; the radius runs fastest, so the
// columns of a z tile (neighbouring ky, hence neighbouring radii) gather from
// one or two cache lines per kz.
// Follows dev_otfinterpolate's RA branch (RLgpuImpl.cu:233-273) with the kz
// coordinate of makeOTFarray_kernel (RLgpuImpl.cu:357).
__device__ __forceinline__ float2 otf_tz_value(int ir, int nzotf, float kzindex,
                                               const float2* __restrict__ otf, float scale) {
  float2 v = make_float2(0.f, 0.f);
  if (kzindex < (float)nzotf && kzindex >= 0.f) {
    const int iz = (int)floorf(kzindex);
    const float az = kzindex - (float)iz;
    const int izp = (iz == nzotf - 1) ? 0 : iz + 1;
    const float2 a = otf[(long long)ir * nzotf + iz];
    const float2 b = otf[(long long)ir * nzotf + izp];
    v = make_float2(a.x * (1.f - az) + b.x * az, a.y * (1.f - az) + b.y * az);
  }
  return make_float2(v.x * scale, v.y * scale);
}

__global__ void k_otf_tz(int nz, int nr, int nzotf, float kzscale, const float2* __restrict__ otf,
                         float4* __restrict__ tz, float scale) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int ir = blockIdx.y;
  if (z >= nz) return;
  const int kz = z > (nz >> 1) ? z - nz : z;
  const float fz = (float)kz * kzscale;
  const float kzindex = fz < 0.f ? fz + (float)nzotf : fz;
  const float2 a = otf_tz_value(ir, nzotf, kzindex, otf, scale);
  const float2 b = ir + 1 < nr ? otf_tz_value(ir + 1, nzotf, kzindex, otf, scale)
                               : make_float2(0.f, 0.f);
  tz[(long long)z * nr + ir] = make_float4(a.x, a.y, b.x, b.y);
}

int launch_otf_tz(const Geom& g, const float2* raw_otf, const RawOtfDims& od, float4* tz,
                  float scale, cudaStream_t st) {
  dim3 grid(ceil_div(g.nz, 128), od.nx_otf);
  k_otf_tz<<<grid, 128, 0, st>>>(g.nz, od.nx_otf, od.nz_otf, od.kzscale, raw_otf, tz, scale);
  CDX_LAUNCH_CHECK("k_otf_tz");
  return 0;
}

// Full 3D (non radially averaged) OTF: trilinear with y/z wrap, as the
// non-RA branch of dev_otfinterpolate (RLgpuImpl.cu:274-319), laid out in the
// spectrum order and scaled.
__global__ void k_otf_full(Geom g, int nxotf, int nyotf, int nzotf, float kxs, float kys, float kzs,
                           const float2* __restrict__ otf, float2* __restrict__ full, float scale) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y;
  const int kx = blockIdx.z;
  if (y >= g.ny) return;
  const int ky = y > (g.ny >> 1) ? y - g.ny : y;
  const int kz = z > (g.nz >> 1) ? z - g.nz : z;
  const float kxindex = (float)kx * kxs;
  const float fy = (float)ky * kys;
  const float fz = (float)kz * kzs;
  const float kyindex = fy < 0.f ? fy + (float)nyotf : fy;
  const float kzindex = fz < 0.f ? fz + (float)nzotf : fz;
  float2 v = make_float2(0.f, 0.f);
  if (kxindex < (float)(nxotf - 1) && kyindex < (float)nyotf && kzindex < (float)nzotf &&
      kyindex >= 0.f && kzindex >= 0.f) {
    const int ix = (int)floorf(kxindex), iy = (int)floorf(kyindex), iz = (int)floorf(kzindex);
    const int iy1 = (iy + 1) % nyotf, iz1 = (iz + 1) % nzotf;
    const float ax = kxindex - ix, ay = kyindex - iy, az = kzindex - iz;
    const long long nxy = (long long)nxotf * nyotf;
    const float2 o000 = otf[iz * nxy + (long long)iy * nxotf + ix];
    const float2 o001 = otf[iz * nxy + (long long)iy * nxotf + ix + 1];
    const float2 o010 = otf[iz * nxy + (long long)iy1 * nxotf + ix];
    const float2 o011 = otf[iz * nxy + (long long)iy1 * nxotf + ix + 1];
    const float2 o100 = otf[iz1 * nxy + (long long)iy * nxotf + ix];
    const float2 o101 = otf[iz1 * nxy + (long long)iy * nxotf + ix + 1];
    const float2 o110 = otf[iz1 * nxy + (long long)iy1 * nxotf + ix];
    const float2 o111 = otf[iz1 * nxy + (long long)iy1 * nxotf + ix + 1];
    v.x = (1 - az) * (o000.x * (1 - ay) * (1 - ax) + o001.x * (1 - ay) * ax + o010.x * ay * (1 - ax) +
                      o011.x * ay * ax) +
          az * (o100.x * (1 - ay) * (1 - ax) + o101.x * (1 - ay) * ax + o110.x * ay * (1 - ax) +
                o111.x * ay * ax);
    v.y = (1 - az) * (o000.y * (1 - ay) * (1 - ax) + o001.y * (1 - ay) * ax + o010.y * ay * (1 - ax) +
                      o011.y * ay * ax) +
          az * (o100.y * (1 - ay) * (1 - ax) + o101.y * (1 - ay) * ax + o110.y * ay * (1 - ax) +
                o111.y * ay * ax);
  }
  full[(long long)kx * g.plane + (long long)z * g.nyp + y] = make_float2(v.x * scale, v.y * scale);
}

int launch_otf_full(const Geom& g, const float2* raw_otf, const RawOtfDims& od, float2* full,
                    float scale, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 128), g.nz, g.nxh);
  k_otf_full<<<grid, 128, 0, st>>>(g, od.nx_otf, od.ny_otf, od.nz_otf, od.kxscale, od.kyscale,
                                   od.kzscale, raw_otf, full, scale);
  CDX_LAUNCH_CHECK("k_otf_full");
  return 0;
}

}  // namespace cdx
