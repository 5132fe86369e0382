// CTA-level mixed-radix FFT engine (radices 2,3,4,5,7,8,9,16) operating in
// place on a tile of complex vectors held in shared memory.
//
// Algorithm: Stockham autosort, decimation in time, as formulated for GPUs by
// Govindaraju et al., "High Performance Discrete Fourier Transforms on
// Graphics Processors" (SC'08): stage s with radix R and span Ns takes the R
// inputs of butterfly j at stride L/R, multiplies input r by
// exp(-2*pi*i * r*(j mod Ns) / (Ns*R)), applies an R-point DFT and writes
// output q to (j div Ns)*Ns*R + (j mod Ns) + q*Ns.
//
// A stage reads the R inputs of each butterfly it owns into registers and
// writes the R outputs; the first stage may read straight from global memory
// and the last one may write straight to global memory (or apply a fused
// epilogue), so a transform of s stages makes s-1 round trips through the
// shared tile.  In-place stages synchronise between their reads and writes.
// A thread owns at most kEpt elements per stage, so a tile of V vectors of
// length L must satisfy V*L <= blockDim.x * kEpt.
//
// Twiddles come from per-stage tables computed in double precision on the
// host, rounded once to float and staged in shared memory by each block.
//
// This replaces the cuFFT R2C/C2R calls of the reference
// (src/RLgpuImpl.cu:183 and :218); it is used for the x, y and z passes of the
// 3D transforms in decon_kernels.cu.
#pragma once

#include "common.cuh"

namespace cdx {

constexpr int kMaxStages = 14;
constexpr int kEpt = 8;         // maximum complex elements held per thread per stage
constexpr int kMaxThreads = 1024; // FFT kernels launch at most this many threads
// Longest transform: one vector must fit a tile of kMaxThreads * kEpt elements.
constexpr int kMaxFftLen = kMaxThreads * kEpt;


// ------------------------------------------------------------- constants
// cos(2*pi*m/R) and sin(2*pi*m/R) for the odd radices, m = 0..R-1.
template <int R>
__host__ __device__ __forceinline__ float odd_cos(int m);
template <int R>
__host__ __device__ __forceinline__ float odd_sin(int m);

template <>
__host__ __device__ __forceinline__ float odd_cos<3>(int m) { return m == 0 ? 1.f : -0.5f; }
template <>
__host__ __device__ __forceinline__ float odd_sin<3>(int m) {
  return m == 0 ? 0.f : (m == 1 ? 8.660254038e-01f : -8.660254038e-01f);
}
template <>
__host__ __device__ __forceinline__ float odd_cos<5>(int m) {
  switch (m) {
    case 0: return 1.f;
    case 1: case 4: return 3.090169944e-01f;
    default: return -8.090169944e-01f;
  }
}
template <>
__host__ __device__ __forceinline__ float odd_sin<5>(int m) {
  switch (m) {
    case 0: return 0.f;
    case 1: return 9.510565163e-01f;
    case 2: return 5.877852523e-01f;
    case 3: return -5.877852523e-01f;
    default: return -9.510565163e-01f;
  }
}
template <>
__host__ __device__ __forceinline__ float odd_cos<7>(int m) {
  switch (m) {
    case 0: return 1.f;
    case 1: case 6: return 6.234898019e-01f;
    case 2: case 5: return -2.225209340e-01f;
    default: return -9.009688679e-01f;
  }
}
template <>
__host__ __device__ __forceinline__ float odd_sin<7>(int m) {
  switch (m) {
    case 0: return 0.f;
    case 1: return 7.818314825e-01f;
    case 2: return 9.749279122e-01f;
    case 3: return 4.338837391e-01f;
    case 4: return -4.338837391e-01f;
    case 5: return -9.749279122e-01f;
    default: return -7.818314825e-01f;
  }
}
template <>
__host__ __device__ __forceinline__ float odd_cos<9>(int m) {
  switch (m) {
    case 0: return 1.f;
    case 1: case 8: return 7.660444431e-01f;
    case 2: case 7: return 1.736481777e-01f;
    case 3: case 6: return -0.5f;
    default: return -9.396926208e-01f;
  }
}
template <>
__host__ __device__ __forceinline__ float odd_sin<9>(int m) {
  switch (m) {
    case 0: return 0.f;
    case 1: return 6.427876097e-01f;
    case 2: return 9.848077530e-01f;
    case 3: return 8.660254038e-01f;
    case 4: return 3.420201433e-01f;
    case 5: return -3.420201433e-01f;
    case 6: return -8.660254038e-01f;
    case 7: return -9.848077530e-01f;
    default: return -6.427876097e-01f;
  }
}

// ------------------------------------------------------------- R-point DFTs
// Forward: y_q = sum_r x_r exp(-2*pi*i*r*q/R); inverse uses exp(+...).
// Inverse transforms are unnormalised, like cuFFT's and FFTW's.

template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
  __host__ __device__ __forceinline__ static void run(float2* x) {
    float2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  }
};

// multiply by -i (forward) or +i (inverse)
template <bool INV>
__host__ __device__ __forceinline__ float2 rot_q(float2 a) { return INV ? mul_pi(a) : mul_mi(a); }

template <bool INV>
struct Dft<4, INV> {
  __host__ __device__ __forceinline__ static void run(float2* x) {
    float2 a = cadd(x[0], x[2]), b = csub(x[0], x[2]);
    float2 c = cadd(x[1], x[3]), d = rot_q<INV>(csub(x[1], x[3]));
    x[0] = cadd(a, c);
    x[2] = csub(a, c);
    x[1] = cadd(b, d);
    x[3] = csub(b, d);
  }
};

template <bool INV>
struct Dft<8, INV> {
  // one radix-2 decimation-in-frequency step followed by two radix-4 DFTs
  __host__ __device__ __forceinline__ static void run(float2* x) {
    const float h = 7.071067812e-01f;
    float2 u[4], v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      u[r] = cadd(x[r], x[r + 4]);
      v[r] = csub(x[r], x[r + 4]);
    }
    // v[r] *= w8^r, w8 = exp(-+2*pi*i/8)
    v[1] = INV ? make_float2(h * (v[1].x - v[1].y), h * (v[1].x + v[1].y))
               : make_float2(h * (v[1].x + v[1].y), h * (v[1].y - v[1].x));
    v[2] = rot_q<INV>(v[2]);
    v[3] = INV ? make_float2(-h * (v[3].x + v[3].y), h * (v[3].x - v[3].y))
               : make_float2(h * (v[3].y - v[3].x), -h * (v[3].x + v[3].y));
    Dft<4, INV>::run(u);
    Dft<4, INV>::run(v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      x[2 * q] = u[q];
      x[2 * q + 1] = v[q];
    }
  }
};

template <bool INV>
struct Dft<16, INV> {
  // 4 x 4 decomposition: n = n1 + 4*n2, k = 4*k1 + k2.
  __host__ __device__ __forceinline__ static void run(float2* x) {
    const float c1 = 9.238795325e-01f, s1 = 3.826834324e-01f, h = 7.071067812e-01f;
    float2 t[4][4];
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
      float2 a[4] = {x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]};
      Dft<4, INV>::run(a);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) t[n1][k2] = a[k2];
    }
    // twiddle t[n1][k2] *= w16^(n1*k2)
    const float sg = INV ? 1.f : -1.f;  // sign of the imaginary part of w16
    // exponents n1*k2 in {0..9}: w16^m = cos(2*pi*m/16) + sg*i*sin(2*pi*m/16)
#pragma unroll
    for (int n1 = 1; n1 < 4; ++n1) {
#pragma unroll
      for (int k2 = 1; k2 < 4; ++k2) {
        const int m = n1 * k2;
        float cr, ci;
        switch (m) {
          case 1: cr = c1; ci = s1; break;
          case 2: cr = h; ci = h; break;
          case 3: cr = s1; ci = c1; break;
          case 4: cr = 0.f; ci = 1.f; break;
          case 6: cr = -h; ci = h; break;
          default: cr = -c1; ci = -s1; break;  // m == 9: cos = -c1, sin = -s1
        }
        t[n1][k2] = cmul(t[n1][k2], make_float2(cr, sg * ci));
      }
    }
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      float2 a[4] = {t[0][k2], t[1][k2], t[2][k2], t[3][k2]};
      Dft<4, INV>::run(a);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) x[4 * k1 + k2] = a[k1];
    }
  }
};

// Odd radix by the symmetric/antisymmetric pairing of inputs p and R-p.
template <int R, bool INV>
struct DftOdd {
  __host__ __device__ __forceinline__ static void run(float2* x) {
    constexpr int H = (R - 1) / 2;
    float2 s[H + 1], d[H + 1];
#pragma unroll
    for (int p = 1; p <= H; ++p) {
      s[p] = cadd(x[p], x[R - p]);
      d[p] = csub(x[p], x[R - p]);
    }
    float2 y0 = x[0];
#pragma unroll
    for (int p = 1; p <= H; ++p) y0 = cadd(y0, s[p]);
    float2 out[R];
    out[0] = y0;
#pragma unroll
    for (int q = 1; q <= H; ++q) {
      float2 a = x[0];
      float2 b = make_float2(0.f, 0.f);
#pragma unroll
      for (int p = 1; p <= H; ++p) {
        const float c = odd_cos<R>((p * q) % R), sn = odd_sin<R>((p * q) % R);
        a.x = fmaf(c, s[p].x, a.x);
        a.y = fmaf(c, s[p].y, a.y);
        b.x = fmaf(sn, d[p].x, b.x);
        b.y = fmaf(sn, d[p].y, b.y);
      }
      // forward: y_q = a - i b, y_{R-q} = a + i b
      float2 ib = mul_pi(b);
      out[q] = INV ? cadd(a, ib) : csub(a, ib);
      out[R - q] = INV ? csub(a, ib) : cadd(a, ib);
    }
#pragma unroll
    for (int q = 0; q < R; ++q) x[q] = out[q];
  }
};
template <bool INV> struct Dft<3, INV> : DftOdd<3, INV> {};
template <bool INV> struct Dft<5, INV> : DftOdd<5, INV> {};
template <bool INV> struct Dft<7, INV> : DftOdd<7, INV> {};
template <bool INV> struct Dft<9, INV> : DftOdd<9, INV> {};

// ------------------------------------------------------------- tile I/O
// Shared-memory tiles are padded with one element per 16 so that the strided
// Stockham accesses (stride R or Ns elements) spread over the banks.
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int spad_size(int n) { return n + (n >> 4) + 1; }

// Exact floor(a / d) for 0 <= a < 2^22 from a float reciprocal of d: the
// quotient of (a + 1/2) is at least 1/(2d) away from an integer, far more
// than the rounding error of one multiply.
__device__ __forceinline__ int fdiv(int a, float inv_d) {
  return __float2int_rz(__fmul_rn((float)a + 0.5f, inv_d));
}

// Element e of vector v of a padded shared-memory tile.
struct SmemIO {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  float2* sm;
  int es, vs;
  __device__ __forceinline__ float2 ld(int v, int e) const { return sm[spad(v * vs + e * es)]; }
  __device__ __forceinline__ void st(int v, int e, float2 x) const { sm[spad(v * vs + e * es)] = x; }
};

// Store the R outputs of one butterfly (elements base + q*stride of vector
// v).  Storers that set kGroup receive them together so that their own
// global loads (fused epilogues) are all issued before any store.
template <int R, class St>
__device__ __forceinline__ void store_group(const St& st, int v, int base, int stride,
                                            const float2* x) {
  if constexpr (St::kGroup) {
    st.template st_group<R>(v, base, stride, x);
  } else {
#pragma unroll
    for (int q = 0; q < R; ++q) st.st(v, base + q * stride, x[q]);
  }
}

// ------------------------------------------------------------- one stage
// Stage geometry, precomputed on the host: LR = L/R butterflies per vector,
// span Ns, the offset of the stage's twiddles, and float reciprocals for fdiv.
struct StageDev {
  int R, LR, Ns, toff;  // toff: offset of this stage's twiddles in the table
  float invLR, invNs;
};

struct FftDev {
  int L;
  int nst;
  StageDev st[kMaxStages];
  // Per-stage twiddles in global memory: stage s with radix R and span Ns
  // holds w[toff + (r-1)*Ns + k] = exp(-2*pi*i*r*k/(Ns*R)), r = 1..R-1,
  // k = 0..Ns-1, so threads with consecutive k read consecutive words.  The
  // stages together hold L-1 entries (sum of (R-1)*Ns telescopes).
  const float2* tw;
};

// One Stockham stage over V vectors.  The R inputs of every butterfly are
// read with ld.ld(v, e), outputs written with st.st(v, e, x).  vfast puts
// consecutive threads on consecutive vectors (interleaved tiles), otherwise
// on consecutive butterflies of a vector.  SYNC_MID separates the reads from
// the writes (needed when both touch the same shared tile); SYNC_END makes
// the writes visible to the next stage.  stw is the twiddle table in smem.
template <int R, bool INV, bool SYNC_MID, bool SYNC_END, class Ld, class St>
__device__ __forceinline__ void stage_io(const StageDev& sd, int V, float invV, bool vfast,
                                         const float2* stw, const Ld& ld, const St& st) {
  constexpr int NB = (kEpt + R - 1) / R;
  // Opaque copies: the butterfly indices below do not depend on the stage
  // and would otherwise be hoisted and kept live across stages.
  int tid = threadIdx.x, T = blockDim.x;
  asm volatile("" : "+r"(tid), "+r"(T));
  const int LR = sd.LR, Ns = sd.Ns;
  const int nbf = V * LR;
  float2 x[NB][R];
  int jj[NB], vv[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int b = tid + i * T;
    jj[i] = -1;
    vv[i] = 0;
    if (b < nbf) {
      int j, v;
      if (vfast) {
        j = fdiv(b, invV);
        v = b - j * V;
      } else {
        v = fdiv(b, sd.invLR);
        j = b - v * LR;
      }
      jj[i] = j;
      vv[i] = v;
#pragma unroll
      for (int r = 0; r < R; ++r) x[i][r] = ld.ld(v, j + r * LR);
    }
  }
  if (SYNC_MID) __syncthreads();
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = jj[i];
    if (j >= 0) {
      const int k = j - fdiv(j, sd.invNs) * Ns;
      if (Ns > 1) {
        const float2* tw = stw + sd.toff + k;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float2 w = tw[(r - 1) * Ns];
          x[i][r] = INV ? cmulconj(x[i][r], w) : cmul(x[i][r], w);
        }
      }
      Dft<R, INV>::run(x[i]);
      store_group<R>(st, vv[i], (j - k) * R + k, Ns, x[i]);
    }
  }
  if (SYNC_END) __syncthreads();
}

template <bool INV, bool SYNC_MID, bool SYNC_END, class Ld, class St>
__device__ __forceinline__ void stage_any(const StageDev& sd, int V, float invV, bool vfast,
                                          const float2* stw, const Ld& ld, const St& st) {
  switch (sd.R) {
    case 2: stage_io<2, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    case 3: stage_io<3, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    case 4: stage_io<4, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    case 5: stage_io<5, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    case 7: stage_io<7, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    case 8: stage_io<8, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    case 9: stage_io<9, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
    default: stage_io<16, INV, SYNC_MID, SYNC_END>(sd, V, invV, vfast, stw, ld, st); break;
  }
}

// Middle stages (shared tile in place) as one homogeneous loop per radix: the
// plan lists radices in the fixed order 16..., {8|4|2}, 9..., 3..., 7..., 5...
// (a single loop with a switch on the radix makes the compiler keep every
// case's registers live).
template <int R, bool INV>
__device__ __forceinline__ void run_middle(const FftDev& f, int& s, int last, int V, float invV,
                                           bool vfast, const float2* stw, const SmemIO& io) {
  while (s < last && f.st[s].R == R) {
    stage_io<R, INV, true, true>(f.st[s], V, invV, vfast, stw, io, io);
    ++s;
  }
}

// Full transform of V vectors of length f.L.  The first stage reads with
// ld0, the last stage writes with stL, and the stages in between work in
// place on the shared tile io.  When stL writes shared memory the function
// ends with a barrier; otherwise the caller decides.  Every thread of the
// block must call it.
template <bool INV, class Ld0, class StL>
__device__ __forceinline__ void fft_run(const FftDev& f, int V, float invV, bool vfast,
                                        const float2* stw, const SmemIO& io, const Ld0& ld0,
                                        const StL& stL) {
  const int ns = f.nst;
  if (ns == 1) {
    // a single stage may read and write the same rows (in place in global
    // memory too), so its reads and writes are always separated
    stage_any<INV, true, StL::kSmem>(f.st[0], V, invV, vfast, stw, ld0, stL);
    return;
  }
  stage_any<INV, Ld0::kSmem, true>(f.st[0], V, invV, vfast, stw, ld0, io);
  int s = 1;
  const int last = ns - 1;
  run_middle<16, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<8, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<4, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<2, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<9, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<3, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<7, INV>(f, s, last, V, invV, vfast, stw, io);
  run_middle<5, INV>(f, s, last, V, invV, vfast, stw, io);
  stage_any<INV, true, StL::kSmem>(f.st[last], V, invV, vfast, stw, io, stL);
}

// Copy the twiddle table of f into shared memory (caller synchronises).
__device__ __forceinline__ void load_twiddles(const FftDev& f, float2* stw) {
  for (int i = threadIdx.x; i < f.L; i += blockDim.x) stw[i] = __ldg(f.tw + i);
}

}  // namespace cdx
