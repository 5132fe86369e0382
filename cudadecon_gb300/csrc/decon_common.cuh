// Device helpers and tile I/O shared by the pass kernels (decon_x_*.cu,
// decon_y.cu, decon_z.cu): packed-row spectrum split/merge, async copies
// into shared memory, and the first-stage loaders / last-stage storers that
// fuse the RL prologue and epilogues into the transforms.
#pragma once

#include "kernels.h"
#include "static_plans.cuh"

namespace cdx {

// ---------------------------------------------------------------- launch order
// The pass kernels of an RL iteration are launched with programmatic stream
// serialization: a pass's blocks may start (and stage their twiddles) while
// the previous pass of the stream drains its last wave.  Before touching
// global data that the previous pass reads or writes, each pass waits here
// until that pass has completed and its writes are visible.  Launched
// without the attribute, or after a non-kernel operation, the wait returns
// at once.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Let the next pass of the stream be scheduled once every block of this one
// has started (its blocks then take SMs as this pass's last wave retires;
// they still wait for this pass to complete before touching its data).
__device__ __forceinline__ void grid_dep_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class... KArgs, class... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

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

// Float-float accumulation of a second float-float value (hi, lo).
__device__ __forceinline__ void ff_add(float4& s, float4 r) {
  acc_add(s.x, s.y, r.x);
  s.y = __fadd_rn(s.y, r.y);
  acc_add(s.z, s.w, r.z);
  s.w = __fadd_rn(s.w, r.w);
}

// Warp-wide float-float sum (tree over the lanes); result in lane 0.
__device__ __forceinline__ float4 warp_sum2_ff(float4 s) {
  for (int o = 16; o > 0; o >>= 1) {
    float4 r;
    r.x = __shfl_down_sync(0xffffffffu, s.x, o);
    r.y = __shfl_down_sync(0xffffffffu, s.y, o);
    r.z = __shfl_down_sync(0xffffffffu, s.z, o);
    r.w = __shfl_down_sync(0xffffffffu, s.w, o);
    ff_add(s, r);
  }
  return s;
}

// Block-wide sum of two float-float values (ah + al, bh + bl): a shuffle tree
// in each warp, then one over the warps' sums, all with TwoSum in FP32
// (GB300's FP64 rate is a small fraction of its FP32 rate).  Returns (sum a
// hi, lo, sum b hi, lo), valid in thread 0.  The order of the additions is
// fixed, so the result is the same on every run.
__device__ __forceinline__ float4 block_sum2_ff(float ah, float al, float bh, float bl,
                                               float4* red) {
  float4 s = warp_sum2_ff(make_float4(ah, al, bh, bl));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (warp == 0) s = warp_sum2_ff(lane < nw ? red[lane] : make_float4(0.f, 0.f, 0.f, 0.f));
  return s;
}

// Prediction of the reference's updatePrediction_kernel (RLgpuImpl.cu:658-666):
// Y = X + lambda*(X - X_{k-1}) with lambda as float, then clamped at 0.
__device__ __forceinline__ float predict_y(float x, float xm1, float lam) {
  float y = __fmaf_rn(lam, __fsub_rn(x, xm1), x);
  return y > 0.f ? y : 0.f;
}

// Radial OTF interpolation (dev_otfinterpolate RA branch, RLgpuImpl.cu:238-273):
// the column (kx, ky = y folded) lies at radius kr = |(kx kxscale, ky kyscale)|
// of the table; zero at kr >= nr - 1.  Returns whether the column is inside,
// with the table column ir and the fraction ar.
__device__ __forceinline__ bool otf_radius(const OtfDev& otf, int kx, int y, int ny, int& ir,
                                           float& ar) {
  const int ky = y > (ny >> 1) ? y - ny : y;
  const float fx = __fmul_rn((float)kx, otf.kxscale);
  const float fy = __fmul_rn((float)ky, otf.kyscale);
  const float kr = __fsqrt_rn(__fmaf_rn(fx, fx, __fmul_rn(fy, fy)));
  if (!(kr < (float)(otf.nr - 1))) return false;
  ir = (int)floorf(kr);
  ar = kr - (float)ir;
  return true;
}

// OTF value between the table pair t = (value at ir, value at ir + 1) at
// fraction ar, with its roundings written out, so that every pass computes
// the same value.
__device__ __forceinline__ float2 otf_lerp(float4 t, float ar) {
  const float a0 = __fsub_rn(1.f, ar);
  return make_float2(__fmaf_rn(ar, t.z, __fmul_rn(a0, t.x)), __fmaf_rn(ar, t.w, __fmul_rn(a0, t.y)));
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

// Allow a kernel the dynamic shared memory it is launched with.  The default
// limit is 48 KB for static and dynamic shared memory together, so the
// attribute is raised for every launch, not only past 48 KB of dynamic
// memory (a kernel with static shared memory crosses the limit earlier).
template <class K>
static int smem_optin(K kernel, size_t bytes) {
  // prefer the largest shared-memory carveout so that several tiles fit an SM
  CDX_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  CDX_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return 0;
}

// Store the packed-row FFT held in the tile (P vectors of length nx) into S
// (PC: P as a compile-time constant, 0 when it is only known at run time).
template <int PC, class IO>
__device__ __forceinline__ void store_half_spectra(const Geom& g, const IO& io, int P, int z,
                                                   int y0, float2* S) {
  const int nx = g.nx;
  const float invP = 1.f / (float)P;
  for (int idx = threadIdx.x; idx < g.nxh * P; idx += blockDim.x) {
    int p, k;
    divmod_small<PC>(idx, P, invP, k, p);
    const int ya = y0 + 2 * p;
    if (ya >= g.ny) continue;
    const float2 zk = io.ld(p, k);
    const float2 zm = io.ld(p, k == 0 ? 0 : nx - k);
    *reinterpret_cast<float4*>(S + (long long)k * g.plane + (long long)z * g.nyp + ya) =
        split_pair(zk, zm);
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
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// L2 policy that marks lines evict-first.  The x passes copy the real arrays
// they read once per iteration (X, X_{k-1}, the raw stack, Y, G_{k-1}) with
// it, so those lines leave the L2 before the spectrum the kernel writes,
// which the next y pass reads.
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void cp_async16_ef(void* dst, const void* src, unsigned long long pol) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src),
               "l"(pol)
               : "memory");
}

// Copy count floats from src (global) to dst (shared); 16-byte copies when
// both addresses allow them, 4-byte copies otherwise.  With ef, the 16-byte
// copies leave their lines evict-first in L2.
__device__ __forceinline__ void prefetch_floats(float* dst, const float* src, int count,
                                                bool ef = false) {
  if (ef && ((reinterpret_cast<unsigned long long>(src) | reinterpret_cast<unsigned long long>(dst)) &
             15) == 0) {
    const unsigned long long pol = l2_evict_first_policy();
    const int n4 = count >> 2;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) cp_async16_ef(dst + 4 * i, src + 4 * i, pol);
    for (int i = 4 * n4 + threadIdx.x; i < count; i += blockDim.x) cp_async4(dst + i, src + i);
    return;
  }
  if (((reinterpret_cast<unsigned long long>(src) | reinterpret_cast<unsigned long long>(dst)) &
       15) == 0) {
    const int n4 = count >> 2;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) cp_async16(dst + 4 * i, src + 4 * i);
    for (int i = 4 * n4 + threadIdx.x; i < count; i += blockDim.x) cp_async4(dst + i, src + i);
  } else {
    for (int i = threadIdx.x; i < count; i += blockDim.x) cp_async4(dst + i, src + i);
  }
}

// Shared-memory layout of an x kernel, in float2 units: the twiddles (nx),
// then the tile region (16-byte aligned), then the prefetched row arrays
// (2P rows of nx floats each).  The tile region holds the padded transform
// tile and, before the first stage, the staged half spectra (P vectors of
// nx/2+1 float4) that the first stage reads: the two alias.
__host__ __device__ __forceinline__ int x_tile_offset(int nx) { return nx + (nx & 1); }
__host__ __device__ __forceinline__ int x_tile_size(int nx, int P) {
  const int a = spad_size(P * nx);
  const int b = 2 * (nx / 2 + 1) * P;
  const int m = a > b ? a : b;
  return m + (m & 1);
}
__host__ __device__ __forceinline__ int x_rows_offset(int nx, int P) {
  return x_tile_offset(nx) + x_tile_size(nx, P);
}

// Issue cp.async copies of the half spectra of rows (y0+2p, y0+2p+1),
// p < P, of slice z into the staging array stg[p * nxh + k] (float4 =
// A[k], B[k]); pairs beyond ny are not copied.  Consecutive threads copy
// the P pairs of one kx (a contiguous run of 16P bytes in S).
template <int PC>
__device__ __forceinline__ void prefetch_packed_spectra(const Geom& g, const float2* S, float4* stg,
                                                        int P, int z, int y0, bool ef = false) {
  const int nxh = g.nxh;
  const int n = nxh * P;
  const float invP = 1.f / (float)P;
  const long long zo = (long long)z * g.nyp + y0;
  const unsigned long long pol = ef ? l2_evict_first_policy() : 0ull;
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    int p, k;
    divmod_small<PC>(idx, P, invP, k, p);
    if (y0 + 2 * p < g.ny) {
      if (ef)
        cp_async16_ef(stg + p * nxh + k, S + (long long)k * g.plane + zo + 2 * p, pol);
      else
        cp_async16(stg + p * nxh + k, S + (long long)k * g.plane + zo + 2 * p);
    }
  }
}

// ---------------------------------------------------------------- stage I/O
// First-stage loader of the forward x pass from rows prefetched into shared
// memory (Xs, Xm1s: 2P rows of nx floats, nr of them valid).  With predict,
// each element is the prediction Y = max(X + lambda (X - X_{k-1}), 0), which
// is also stored to the block's rows Yg in global memory (the first stage
// reads every element exactly once).  Y is read again only by the update
// pass at the end of the iteration, so it is stored evict-first (__stcs),
// leaving the L2 to the spectrum the y pass reads next.
struct RowPairSmemLoad {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  const float* Xs;
  const float* Xm1s;
  float* Yg;
  float lam;
  int predict, nr, nx;
  __device__ __forceinline__ float2 ld(int v, int e) const {
    const int ra = 2 * v;
    float a = 0.f, b = 0.f;
    if (ra < nr) {
      const int o = ra * nx + e;
      a = Xs[o];
      if (predict) {
        a = predict_y(a, Xm1s[o], lam);
        __stcs(Yg + o, a);
      }
      if (ra + 1 < nr) {
        b = Xs[o + nx];
        if (predict) {
          b = predict_y(b, Xm1s[o + nx], lam);
          __stcs(Yg + o + nx, b);
        }
      }
    }
    return make_float2(a, b);
  }
};

// First-stage loader of the inverse x passes: element e of the packed
// full-length spectrum Z = A + iB of pair v, rebuilt from the staged half
// spectra (prefetch_packed_spectra).  The imaginary parts of the DC and
// (even nx) Nyquist bins are dropped, as a C2R transform does.
struct PackedSpecLoad {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  const float4* stg;
  int nxh, nx, npairs;  // npairs: pairs with rows inside the volume
  __device__ __forceinline__ float2 ld(int v, int e) const {
    if (v >= npairs) return make_float2(0.f, 0.f);
    const bool lo = e < nxh;
    const int k = lo ? e : nx - e;
    float4 w = stg[v * nxh + k];
    if (k == 0 || 2 * k == nx) {
      w.y = 0.f;
      w.w = 0.f;
    }
    // Z[k] = A + iB; Z[nx-k] = conj(A) + i conj(B)
    return lo ? make_float2(w.x - w.w, w.y + w.z) : make_float2(w.x + w.w, w.z - w.y);
  }
};

// PackedSpecLoad for a compile-time row length NX (the x kernels of the
// compile-time plans).  The first stage of those plans reads element
// e = R*LR + j of vector v with R and LR compile-time and 0 <= j < LR
// (ld_at): whether e lies in the lower half (k = e) or the upper (k = NX -
// e), and whether it can be the DC or Nyquist bin, is then known at compile
// time for every R but the one whose range straddles NX/2 + 1.  Same values
// as PackedSpecLoad, without its per-element selects.
template <int NX>
struct PackedSpecLoadS {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  static constexpr bool kLdAt = true;
  static constexpr int NXH = NX / 2 + 1;
  const float4* stg;
  int npairs;  // pairs with rows inside the volume
  __device__ __forceinline__ static float2 lo_val(float4 w) {
    return make_float2(w.x - w.w, w.y + w.z);
  }
  __device__ __forceinline__ static float2 hi_val(float4 w) {
    return make_float2(w.x + w.w, w.z - w.y);
  }
  __device__ __forceinline__ float2 ld(int v, int e) const {
    if (v >= npairs) return make_float2(0.f, 0.f);
    const bool lo = e < NXH;
    const int k = lo ? e : NX - e;
    float4 w = stg[v * NXH + k];
    if (k == 0 || 2 * k == NX) {
      w.y = 0.f;
      w.w = 0.f;
    }
    return lo ? lo_val(w) : hi_val(w);
  }
  template <int R, int LR>
  __device__ __forceinline__ float2 ld_at(int v, int j) const {
    constexpr int e0 = R * LR;  // e = e0 + j, 0 <= j < LR
    if constexpr (e0 + LR <= NXH) {
      if (v >= npairs) return make_float2(0.f, 0.f);
      const int k = e0 + j;
      float4 w = stg[v * NXH + k];
      // the DC bin (e = 0) and, for even NX, the Nyquist bin (e = NX/2)
      constexpr bool has_dc = e0 == 0;
      constexpr bool has_nyq = NX % 2 == 0 && e0 <= NX / 2 && NX / 2 < e0 + LR;
      if constexpr (has_dc || has_nyq) {
        if ((has_dc && j == 0) || (has_nyq && k == NX / 2)) {
          w.y = 0.f;
          w.w = 0.f;
        }
      }
      return lo_val(w);
    } else if constexpr (e0 >= NXH) {
      // upper half: k = NX - e in [1, NX/2), neither DC nor Nyquist
      if (v >= npairs) return make_float2(0.f, 0.f);
      return hi_val(stg[v * NXH + (NX - e0 - j)]);
    } else {
      return ld(v, e0 + j);
    }
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
  // 0 / v is a signed zero and the sum with eps is eps either way; zero
  // numerators (common after background subtraction) skip the division,
  // whose general path is far slower for them.
  const float q = __fdiv_rn(raw == 0.f ? 1.f : raw, v);
  v = __fadd_rn(raw == 0.f ? 0.f : q, eps);
  v = v > 10.f ? 10.f : v;
  v = v < -10.f ? -10.f : v;
  return v;
}

template <class IO>
struct RatioStore {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  IO io;
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
