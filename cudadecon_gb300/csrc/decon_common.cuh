// Device helpers and tile I/O shared by the pass kernels (decon_x_fwd.cu,
// decon_x_inv.cu, decon_yz.cu): packed-row spectrum split/merge, async row
// copies into shared memory, and the first-stage loaders / last-stage
// storers that fuse the RL prologue and epilogues into the transforms.
#pragma once

#include "kernels.h"
#include "static_plans.cuh"

namespace cdx {

// ---------------------------------------------------------------- helpers
// Float-float accumulation (Knuth's TwoSum): hi + lo carries the running sum
// with about 48 significant bits, so a thread's partial sums of float
// products match double accumulation (the reference sums in double,
// RLgpuImpl.cu:582-592) at FP32 cost; GB300's FP64 throughput is low.
__device__ __forceinline__ void acc_add(float& hi, float& lo, float p) {
  const float s = __fadd_rn(hi, p);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

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
static inline int x_pairs(int nx) {
  int p = (kMaxThreads * kEpt) / nx;
  if (p > 8) p = 8;
  if (nx >= 512 && p > 4) p = 4;  // long rows: smaller tiles, more resident blocks
  if (p < 1) p = 1;
  return p;
}



static inline int threads_for(long long elems) {
  long long t = (elems + kEpt - 1) / kEpt;
  t = ((t + 31) / 32) * 32;
  if (t < 64) t = 64;
  if (t > kMaxThreads) t = kMaxThreads;
  return (int)t;
}

// Bytes of dynamic shared memory: twiddles + padded tile (+ extra float2s).
static inline size_t fft_smem(int L, long long tile, long long extra = 0) {
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
  float* acc;  // float-float accumulators: s1 (hi, lo), s2 (hi, lo)
  __device__ __forceinline__ void one(int rloc, int e, float cc) const {
    const int l = rloc * nx + e;
    const float x = Xs[l];
    const float yv = predict ? predict_y(x, Xm1s[l], lam) : x;
    float xn = __fmul_rn(cc, yv);
    xn = xn > 0.f ? xn : 0.f;
    const float gn = __fsub_rn(xn, yv);
    if (dots) {
      const float go = Gs[l];
      acc_add(acc[0], acc[1], __fmul_rn(gn, go));
      acc_add(acc[2], acc[3], __fmul_rn(go, go));
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

}  // namespace cdx
