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
#include "kernels.h"

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

int fft_len_init(FftLen& f, int L) {
  std::vector<int> rad;
  if (L < 1 || L > kMaxFftLen || !factorize(L, rad)) {
    set_error("fft_len_init", "length is not a product of 2, 3, 5 and 7");
    return cudaErrorInvalidValue;
  }
  f.dev.L = L;
  f.dev.nst = (rad.size() == 1 && rad[0] == 1) ? 0 : (int)rad.size();
  std::vector<float2> tw(L, make_float2(1.f, 0.f));
  const double two_pi = 6.283185307179586476925286766559;
  int Ns = 1;
  for (int i = 0; i < kMaxStages; ++i) {
    StageDev& sd = f.dev.st[i];
    if (i < f.dev.nst) {
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
  CDX_CHECK(cudaMalloc(&f.d_tw, sizeof(float2) * L));
  CDX_CHECK(cudaMemcpy(f.d_tw, tw.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
  f.dev.tw = f.d_tw;
  return 0;
}

void fft_len_free(FftLen& f) {
  if (f.d_tw) cudaFree(f.d_tw);
  f.d_tw = nullptr;
  f.dev.tw = nullptr;
}

// ---------------------------------------------------------------- helpers
// Prediction of the reference's updatePrediction_kernel (RLgpuImpl.cu:658-666):
// Y = X + lambda*(X - X_{k-1}) with lambda as float, then clamped at 0.
__device__ __forceinline__ float predict_y(float x, float xm1, float lam) {
  float y = __fmaf_rn(lam, __fsub_rn(x, xm1), x);
  return y > 0.f ? y : 0.f;
}

// Split the FFT Z of packed rows (a + i b) into the half spectra of a and b.
__device__ __forceinline__ float4 split_pair(float2 zk, float2 zm) {
  // A = (Z[k] + conj(Z[n-k]))/2, B = (Z[k] - conj(Z[n-k]))/(2i)
  return make_float4(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y), 0.5f * (zk.y + zm.y),
                     0.5f * (zm.x - zk.x));
}

// Row pairs per x tile: up to 8 (16 rows -> 128-byte spectrum runs), fewer
// for long rows so that the tile fits kMaxThreads * kEpt elements.
static int x_pairs(int nx) {
  int p = (kMaxThreads * kEpt) / nx;
  if (p > 8) p = 8;
  if (nx >= 512 && p > 4) p = 4;  // long rows: smaller tiles, more resident blocks
  if (p < 1) p = 1;
  return p;
}

int x_pass_blocks(const Geom& g) { return ceil_div(g.ny, 2 * x_pairs(g.nx)) * g.nz; }

static int threads_for(long long elems) {
  long long t = (elems + kEpt - 1) / kEpt;
  t = ((t + 31) / 32) * 32;
  if (t < 64) t = 64;
  if (t > kMaxThreads) t = kMaxThreads;
  return (int)t;
}

// Bytes of dynamic shared memory: twiddles + padded tile (+ extra float2s).
static size_t fft_smem(int L, long long tile, long long extra = 0) {
  return sizeof(float2) * ((size_t)L + spad_size((int)tile) + (size_t)extra);
}

// Allow a kernel the dynamic shared memory it is launched with (the default
// limit is 48 KB; long rows need more).
template <class K>
static int smem_optin(K kernel, size_t bytes) {
  // prefer the largest shared-memory carveout so that several tiles fit an SM
  CDX_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  if (bytes <= 48 * 1024) return 0;
  CDX_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return 0;
}

// Store the packed-row FFT held in the tile (P vectors of length nx) into S.
__device__ __forceinline__ void store_half_spectra(const Geom& g, const SmemIO& io, int P, int z,
                                                   int y0, float2* S) {
  const int nx = g.nx;
  for (int idx = threadIdx.x; idx < g.nxh * P; idx += blockDim.x) {
    const int p = idx % P;
    const int k = idx / P;
    const int ya = y0 + 2 * p;
    if (ya >= g.ny) continue;
    const float2 zk = io.ld(p, k);
    const float2 zm = io.ld(p, k == 0 ? 0 : nx - k);
    *reinterpret_cast<float4*>(S + (long long)k * g.plane + (long long)z * g.nyp + ya) =
        split_pair(zk, zm);
  }
}

// Load the two half spectra of rows (ya, ya+1) and rebuild the packed
// full-length spectrum Z = A + iB in the tile.  The imaginary parts of the
// DC and (even nx) Nyquist bins are dropped, as a C2R transform does.
__device__ __forceinline__ void load_packed_spectra(const Geom& g, const float2* S, const SmemIO& io,
                                                    int P, int z, int y0) {
  const int nx = g.nx;
  const int n = g.nxh * P;
  const int T = blockDim.x;
  constexpr int B = 8;  // loads issued before the first shared store
  for (int base = threadIdx.x; base < n; base += B * T) {
    float4 v[B];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int idx = base + b * T;
      const int p = idx % P;
      const int k = idx / P;
      const int ya = y0 + 2 * p;
      v[b] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (idx < n && ya < g.ny)
        v[b] = __ldg(reinterpret_cast<const float4*>(S + (long long)k * g.plane +
                                                     (long long)z * g.nyp + ya));
    }
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int idx = base + b * T;
      if (idx >= n) break;
      const int p = idx % P;
      const int k = idx / P;
      float4 w = v[b];
      if (k == 0 || 2 * k == nx) {
        w.y = 0.f;
        w.w = 0.f;
      }
      // Z[k] = A + iB; Z[nx-k] = conj(A) + i conj(B)
      io.st(p, k, make_float2(w.x - w.w, w.y + w.z));
      if (k > 0 && 2 * k != nx) io.st(p, nx - k, make_float2(w.x + w.w, w.z - w.y));
    }
  }
}

// ---------------------------------------------------------------- async row copies
// Rows y0 .. y0+nr-1 of one z slice are contiguous (nr*nx floats); they are
// copied into shared memory with cp.async at the start of an x kernel, so
// the copy overlaps the transform without occupying registers, and the
// fused epilogue later reads them from shared memory.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Copy count floats from src (global) to dst (shared); 16-byte copies when
// both addresses allow them, 4-byte copies otherwise.
__device__ __forceinline__ void prefetch_floats(float* dst, const float* src, int count) {
  if (((reinterpret_cast<unsigned long long>(src) | reinterpret_cast<unsigned long long>(dst)) &
       15) == 0) {
    const int n4 = count >> 2;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) cp_async16(dst + 4 * i, src + 4 * i);
    for (int i = 4 * n4 + threadIdx.x; i < count; i += blockDim.x) cp_async4(dst + i, src + i);
  } else {
    for (int i = threadIdx.x; i < count; i += blockDim.x) cp_async4(dst + i, src + i);
  }
}

// Shared float2 offset after the twiddles and the padded tile of an x kernel,
// rounded up to 16 bytes; each prefetched array holds 2P rows of nx floats.
__host__ __device__ __forceinline__ int x_rows_offset(int nx, int P) {
  const int o = nx + spad_size(P * nx);
  return o + (o & 1);
}

// ---------------------------------------------------------------- stage I/O
// Outputs per load batch of the fused epilogues (bounds their registers).
constexpr int kStoreBatch = 4;

// First-stage loader of the forward x pass: row pair v of the tile (rows
// y0+2v and y0+2v+1 of slice z) packed as a + i b, with the prediction
// Y = max(X + lambda (X - X_{k-1}), 0) applied on the fly when predict != 0.
struct RowPairLoad {
  static constexpr bool kSmem = false;
  static constexpr bool kGroup = false;
  const float* X;
  const float* Xm1;
  float lam;
  int predict;
  long long zoff;
  int y0, ny, nx;
  __device__ __forceinline__ float2 ld(int v, int e) const {
    const int ya = y0 + 2 * v;
    float a = 0.f, b = 0.f;
    if (ya < ny) {
      const long long o = zoff + (long long)ya * nx + e;
      a = __ldg(X + o);
      if (predict) a = predict_y(a, __ldg(Xm1 + o), lam);
      if (ya + 1 < ny) {
        b = __ldg(X + o + nx);
        if (predict) b = predict_y(b, __ldg(Xm1 + o + nx), lam);
      }
    }
    return make_float2(a, b);
  }
};

// Rows r0 + v of the spectrum (one (kx, z) row of length ny each).
struct SpecRowIO {
  static constexpr bool kSmem = false;
  static constexpr bool kGroup = false;
  float2* S;
  long long r0, nrows;
  int nyp;
  __device__ __forceinline__ float2 ld(int v, int e) const {
    const long long r = r0 + v;
    return r < nrows ? S[r * nyp + e] : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void st(int v, int e, float2 x) const {
    const long long r = r0 + v;
    if (r < nrows) S[r * nyp + e] = x;
  }
};

// Columns y0 + v of one kx plane of the spectrum, element e = z.
struct SpecColIO {
  static constexpr bool kSmem = false;
  static constexpr bool kGroup = false;
  float2* base;
  int y0, ny, nyp;
  __device__ __forceinline__ float2 ld(int v, int e) const {
    const int y = y0 + v;
    return y < ny ? base[(long long)e * nyp + y] : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void st(int v, int e, float2 x) const {
    const int y = y0 + v;
    if (y < ny) base[(long long)e * nyp + y] = x;
  }
};

// Last forward z stage: multiply by the OTF tile and store to shared memory.
struct OtfMulStore {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  SmemIO io;
  const float2* otf;  // [e * W + v]
  int W, conj;
  __device__ __forceinline__ void st(int v, int e, float2 x) const {
    const float2 o = otf[e * W + v];
    io.st(v, e, conj ? cmulconj(x, o) : cmul(x, o));
  }
};

// Last inverse x stage of the first convolution: the RL ratio of the
// reference's LRcore_kernel (RLgpuImpl.cu:416-434) for both rows of pair v,
// written to the tile for the forward transform that follows.
__device__ __forceinline__ float rl_ratio(float c, float raw, float eps) {
  float v = fabsf(c) > 0.f ? c : eps;
  v = __fadd_rn(__fdiv_rn(raw, v), eps);
  v = v > 10.f ? 10.f : v;
  v = v < -10.f ? -10.f : v;
  return v;
}

struct RatioStore {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  SmemIO io;
  const float* raw;  // shared: rows y0 .. y0+2P-1 of the slice
  int y0, ny, nx;
  float eps;
  __device__ __forceinline__ void st(int v, int e, float2 c) const {
    const int ya = y0 + 2 * v;
    float2 r = make_float2(0.f, 0.f);
    if (ya < ny) r.x = rl_ratio(c.x, raw[(2 * v) * nx + e], eps);
    if (ya + 1 < ny) r.y = rl_ratio(c.y, raw[(2 * v + 1) * nx + e], eps);
    io.st(v, e, r);
  }
};

// Last inverse x stage of the second convolution: estimate update
// (currEstimate_kernel + currPrevDiff_kernel, RLgpuImpl.cu:462-470, 501-508)
// with the Biggs-Andrews dot products of innerProduct_kernel
// (RLgpuImpl.cu:571-633: float products, double sums).
struct UpdateStore {
  static constexpr bool kSmem = false;
  static constexpr bool kGroup = false;
  const float* Xs;   // shared copies of rows y0 .. y0+2P-1 of X, X_{k-1} and G
  const float* Xm1s;
  const float* Gs;
  float* Xout;       // global
  float* G;          // global
  float lam;
  int predict, dots;
  long long zoff;
  int y0, ny, nx;
  double* s1;
  double* s2;
  __device__ __forceinline__ void one(int rloc, int e, float cc) const {
    const int l = rloc * nx + e;
    const float x = Xs[l];
    const float yv = predict ? predict_y(x, Xm1s[l], lam) : x;
    float xn = __fmul_rn(cc, yv);
    xn = xn > 0.f ? xn : 0.f;
    const float gn = __fsub_rn(xn, yv);
    if (dots) {
      const float go = Gs[l];
      *s1 += (double)__fmul_rn(gn, go);
      *s2 += (double)__fmul_rn(go, go);
    }
    const long long o = zoff + (long long)(y0 + rloc) * nx + e;
    Xout[o] = xn;
    G[o] = gn;
  }
  __device__ __forceinline__ void st(int v, int e, float2 c) const {
    const int ya = y0 + 2 * v;
    if (ya < ny) one(2 * v, e, c.x);
    if (ya + 1 < ny) one(2 * v + 1, e, c.y);
  }
};

struct PlainRowStore {
  static constexpr bool kSmem = false;
  static constexpr bool kGroup = false;
  float* out;
  long long zoff;
  int y0, ny, nx;
  __device__ __forceinline__ void st(int v, int e, float2 c) const {
    const int ya = y0 + 2 * v;
    if (ya < ny) {
      const long long o = zoff + (long long)ya * nx + e;
      out[o] = c.x;
      if (ya + 1 < ny) out[o + nx] = c.y;
    }
  }
};

// ---------------------------------------------------------------- x forward
__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_fwd(Geom g, FftDev fx, const float* __restrict__ X, const float* __restrict__ Xm1,
        const float* __restrict__ lamp, int predict, float2* __restrict__ S, int P) {
  extern __shared__ float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  load_twiddles(fx, stw);
  __syncthreads();
  const RowPairLoad ld{X, Xm1, predict ? __ldg(lamp) : 0.f, predict, (long long)z * g.ny * nx,
                       y0, g.ny, nx};
  fft_run<false>(fx, P, 1.f, false, stw, io, ld, io);
  store_half_spectra(g, io, P, z, y0, S);
}

int launch_x_fwd(const Geom& g, const FftLen& fx, const float* X, const float* Xm1,
                 const float* lam, int predict, float2* S, cudaStream_t st) {
  const int P = x_pairs(g.nx);
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  int T = threads_for((long long)P * g.nx);
  size_t smem = fft_smem(g.nx, (long long)P * g.nx);
  if (int rc = smem_optin(k_x_fwd, smem)) return rc;
  k_x_fwd<<<grid, T, smem, st>>>(g, fx.dev, X, Xm1, lam, predict, S, P);
  CDX_LAUNCH_CHECK("k_x_fwd");
  return 0;
}

// ---------------------------------------------------------------- y pass
template <bool INV>
__global__ void __launch_bounds__(kMaxThreads, 1)
k_y_pass(Geom g, FftDev fy, float2* __restrict__ S, int V) {
  extern __shared__ float2 smem[];
  const int ny = g.ny;
  float2* stw = smem;
  const SmemIO io{smem + ny, 1, ny};
  load_twiddles(fy, stw);
  __syncthreads();
  const SpecRowIO gio{S, (long long)blockIdx.x * V, (long long)g.nxh * g.nz, g.nyp};
  fft_run<INV>(fy, V, 1.f, false, stw, io, gio, gio);
}

int launch_y_pass(const Geom& g, const FftLen& fy, float2* S, bool inverse, cudaStream_t st) {
  int V = 2048 / g.ny;
  if (V < 1) V = 1;
  const long long nrows = (long long)g.nxh * g.nz;
  int T = threads_for((long long)V * g.ny);
  size_t smem = fft_smem(g.ny, (long long)V * g.ny);
  dim3 grid((unsigned)((nrows + V - 1) / V));
  if (int rc = smem_optin(inverse ? k_y_pass<true> : k_y_pass<false>, smem)) return rc;
  if (inverse)
    k_y_pass<true><<<grid, T, smem, st>>>(g, fy.dev, S, V);
  else
    k_y_pass<false><<<grid, T, smem, st>>>(g, fy.dev, S, V);
  CDX_LAUNCH_CHECK("k_y_pass");
  return 0;
}

// ---------------------------------------------------------------- z pass
// Columns (consecutive y) per z tile: 16 (128-byte runs) while the tile fits
// kMaxThreads * kEpt elements, fewer for long z.
static int z_cols(int nz) {
  int w = (kMaxThreads * kEpt) / nz;
  if (w > 16) w = 16;
  if (w < 1) w = 1;
  return w;
}

__global__ void __launch_bounds__(kMaxThreads, 1)
k_z_pass(Geom g, FftDev fz, float2* __restrict__ S, OtfDev otf, int conj, int fwd_only, int W) {
  extern __shared__ float2 smem[];
  const int nz = g.nz;
  const int kx = blockIdx.y;
  const int y0 = blockIdx.x * W;
  float2* stw = smem;
  const SmemIO io{smem + nz, W, 1};
  float2* otf_tile = smem + nz + spad_size(W * nz);
  load_twiddles(fz, stw);
  const float invW = 1.f / (float)W;
  const SpecColIO gio{S + (long long)kx * g.plane, y0, g.ny, g.nyp};
  if (fwd_only) {
    __syncthreads();
    fft_run<false>(fz, W, invW, true, stw, io, gio, gio);
    return;
  }
  // OTF of every (y, z) of the tile, interpolated on the fly from the
  // kz-resampled radial table (dev_otfinterpolate RA branch,
  // RLgpuImpl.cu:238-273: kr = sqrt(kx^2 + ky^2), zero at kr >= nr-1) or
  // read from the precomputed 3D array
  for (int idx = threadIdx.x; idx < W * nz; idx += blockDim.x) {
    const int w = idx % W;
    const int z = idx / W;
    const int y = y0 + w;
    float2 o = make_float2(0.f, 0.f);
    if (y < g.ny) {
      if (otf.mode == 1) {
        o = __ldg(otf.full + (long long)kx * g.plane + (long long)z * g.nyp + y);
      } else {
        const int ky = y > (g.ny >> 1) ? y - g.ny : y;
        const float fx = (float)kx * otf.kxscale;
        const float fy = (float)ky * otf.kyscale;
        const float kr = sqrtf(fx * fx + fy * fy);
        if (kr < (float)(otf.nr - 1)) {
          const int ir = (int)floorf(kr);
          const float ar = kr - (float)ir;
          const float2 t0 = __ldg(otf.tz + (long long)ir * nz + z);
          const float2 t1 = __ldg(otf.tz + (long long)(ir + 1) * nz + z);
          o = make_float2((1.f - ar) * t0.x + ar * t1.x, (1.f - ar) * t0.y + ar * t1.y);
        }
      }
    }
    otf_tile[idx] = o;
  }
  __syncthreads();
  const OtfMulStore ost{io, otf_tile, W, conj};
  fft_run<false>(fz, W, invW, true, stw, io, gio, ost);
  fft_run<true>(fz, W, invW, true, stw, io, io, gio);
}

int launch_z_pass(const Geom& g, const FftLen& fz, float2* S, const OtfDev& otf, bool conj,
                  cudaStream_t st, bool fwd_only) {
  const int W = z_cols(g.nz);
  dim3 grid(ceil_div(g.ny, W), g.nxh);
  int T = threads_for((long long)W * g.nz);
  size_t smem = fft_smem(g.nz, (long long)W * g.nz, (long long)W * g.nz);
  if (int rc = smem_optin(k_z_pass, smem)) return rc;
  k_z_pass<<<grid, T, smem, st>>>(g, fz.dev, S, otf, conj ? 1 : 0, fwd_only ? 1 : 0, W);
  CDX_LAUNCH_CHECK("k_z_pass");
  return 0;
}

// ---------------------------------------------------------------- x inverse
__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_inv_ratio_fwd(Geom g, FftDev fx, float2* __restrict__ S, const float* __restrict__ raw,
                  float eps, int P) {
  extern __shared__ float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  float* raws = reinterpret_cast<float*>(smem + x_rows_offset(nx, P));
  const int nr = min(2 * P, g.ny - y0);
  prefetch_floats(raws, raw + ((long long)z * g.ny + y0) * nx, nr * nx);
  cp_async_commit();
  load_twiddles(fx, stw);
  load_packed_spectra(g, S, io, P, z, y0);
  cp_async_wait_all();
  __syncthreads();
  const RatioStore rs{io, raws, y0, g.ny, nx, eps};
  fft_run<true>(fx, P, 1.f, false, stw, io, io, rs);
  fft_run<false>(fx, P, 1.f, false, stw, io, io, io);
  store_half_spectra(g, io, P, z, y0, S);
}

int launch_x_inv_ratio_fwd(const Geom& g, const FftLen& fx, float2* S, const float* raw,
                           float eps, cudaStream_t st) {
  const int P = x_pairs(g.nx);
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  int T = threads_for((long long)P * g.nx);
  size_t smem = sizeof(float2) * ((size_t)x_rows_offset(g.nx, P) + (size_t)P * g.nx);
  if (int rc = smem_optin(k_x_inv_ratio_fwd, smem)) return rc;
  k_x_inv_ratio_fwd<<<grid, T, smem, st>>>(g, fx.dev, S, raw, eps, P);
  CDX_LAUNCH_CHECK("k_x_inv_ratio_fwd");
  return 0;
}

// Block-wide sum of two doubles; result valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < nw ? red[lane] : 0.0;
    b = lane < nw ? red[32 + lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
  }
}

__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_inv_update(Geom g, FftDev fx, const float2* __restrict__ S, const float* __restrict__ X,
               const float* Xm1, const float* __restrict__ lamp, int predict, float* Xout,
               float* __restrict__ G, int dots, double* partials, unsigned* counter,
               float* lam_next, float eps, int P) {
  extern __shared__ float2 smem[];
  __shared__ double red[64];
  __shared__ bool last;
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  // prefetch rows of X, X_{k-1} (when predicting) and G (when the dots are
  // needed) into shared memory; they are read by the epilogue
  float* Xs = reinterpret_cast<float*>(smem + x_rows_offset(nx, P));
  float* Xm1s = Xs + 2 * P * nx;
  float* Gs = Xm1s + 2 * P * nx;
  const int nr = min(2 * P, g.ny - y0);
  const long long roff = ((long long)z * g.ny + y0) * nx;
  prefetch_floats(Xs, X + roff, nr * nx);
  if (predict) prefetch_floats(Xm1s, Xm1 + roff, nr * nx);
  if (dots) prefetch_floats(Gs, G + roff, nr * nx);
  cp_async_commit();
  load_twiddles(fx, stw);
  load_packed_spectra(g, S, io, P, z, y0);
  cp_async_wait_all();
  __syncthreads();
  double s1 = 0.0, s2 = 0.0;
  const UpdateStore us{Xs, Xm1s, Gs, Xout, G, predict ? __ldg(lamp) : 0.f, predict, dots,
                       (long long)z * g.ny * nx, y0, g.ny, nx, &s1, &s2};
  fft_run<true>(fx, P, 1.f, false, stw, io, io, us);
  if (!dots) return;
  block_sum2(s1, s2, red);
  const int nblk = gridDim.x * gridDim.y;
  const int bid = blockIdx.y * gridDim.x + blockIdx.x;
  if (threadIdx.x == 0) {
    partials[bid] = s1;
    partials[nblk + bid] = s2;
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == (unsigned)nblk - 1);
  }
  __syncthreads();
  if (!last) return;
  // Last block: reduce all partials in a fixed order (deterministic).
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += __ldcg(partials + i);
    b += __ldcg(partials + nblk + i);
  }
  block_sum2(a, b, red);
  if (threadIdx.x == 0) {
    // calcAccelFactor (RLgpuImpl.cu:565) then the clamp of RL-Biggs-Andrews.cpp:298
    double l = a / (b + (double)eps);
    l = (1.0 < l) ? 1.0 : l;
    l = (l < 0.0) ? 0.0 : l;
    *lam_next = (float)l;
    *counter = 0u;
  }
}

int launch_x_inv_update(const Geom& g, const FftLen& fx, const float2* S, const float* X,
                        const float* Xm1, const float* lam, int predict, float* Xout, float* G,
                        int dots, RLWork& w, float* lam_next, float eps, cudaStream_t st) {
  const int P = x_pairs(g.nx);
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  const int nblk = grid.x * grid.y;
  if (dots && nblk > w.max_blocks) {
    set_error("launch_x_inv_update", "partials buffer too small");
    return cudaErrorInvalidValue;
  }
  int T = threads_for((long long)P * g.nx);
  size_t smem = sizeof(float2) * ((size_t)x_rows_offset(g.nx, P) + 3 * (size_t)P * g.nx);
  if (int rc = smem_optin(k_x_inv_update, smem)) return rc;
  k_x_inv_update<<<grid, T, smem, st>>>(g, fx.dev, S, X, Xm1, lam, predict, Xout, G, dots,
                                        w.partials, w.counter, lam_next, eps, P);
  CDX_LAUNCH_CHECK("k_x_inv_update");
  return 0;
}

__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_inv_plain(Geom g, FftDev fx, const float2* __restrict__ S, float* __restrict__ out, int P) {
  extern __shared__ float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  load_twiddles(fx, stw);
  load_packed_spectra(g, S, io, P, z, y0);
  __syncthreads();
  const PlainRowStore ps{out, (long long)z * g.ny * nx, y0, g.ny, nx};
  fft_run<true>(fx, P, 1.f, false, stw, io, io, ps);
}

int launch_x_inv_plain(const Geom& g, const FftLen& fx, const float2* S, float* out,
                       cudaStream_t st) {
  const int P = x_pairs(g.nx);
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  int T = threads_for((long long)P * g.nx);
  size_t smem = fft_smem(g.nx, (long long)P * g.nx);
  if (int rc = smem_optin(k_x_inv_plain, smem)) return rc;
  k_x_inv_plain<<<grid, T, smem, st>>>(g, fx.dev, S, out, P);
  CDX_LAUNCH_CHECK("k_x_inv_plain");
  return 0;
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
// volume: tz[ir][z] = otf[ir][iz]*(1-az) + otf[ir][iz+1 (wrapping)]*az, zero
// where kzindex falls outside [0, nz_otf), times scale (= 1/N).
// Follows dev_otfinterpolate's RA branch (RLgpuImpl.cu:233-273) with the kz
// coordinate of makeOTFarray_kernel (RLgpuImpl.cu:357).
__global__ void k_otf_tz(int nz, int nr, int nzotf, float kzscale, const float2* __restrict__ otf,
                         float2* __restrict__ tz, float scale) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int ir = blockIdx.y;
  if (z >= nz) return;
  const int kz = z > (nz >> 1) ? z - nz : z;
  const float fz = (float)kz * kzscale;
  const float kzindex = fz < 0.f ? fz + (float)nzotf : fz;
  float2 v = make_float2(0.f, 0.f);
  if (kzindex < (float)nzotf && kzindex >= 0.f) {
    const int iz = (int)floorf(kzindex);
    const float az = kzindex - (float)iz;
    const int izp = (iz == nzotf - 1) ? 0 : iz + 1;
    const float2 a = otf[(long long)ir * nzotf + iz];
    const float2 b = otf[(long long)ir * nzotf + izp];
    v = make_float2(a.x * (1.f - az) + b.x * az, a.y * (1.f - az) + b.y * az);
  }
  tz[(long long)ir * nz + z] = make_float2(v.x * scale, v.y * scale);
}

int launch_otf_tz(const Geom& g, const float2* raw_otf, const RawOtfDims& od, float2* tz,
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
