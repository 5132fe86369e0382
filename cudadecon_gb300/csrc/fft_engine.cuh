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
// The tile is transformed in place: in each stage every thread first pulls all
// butterfly inputs it owns into registers, the block synchronises, and then the
// outputs are written back.  A thread owns at most kEpt elements per stage, so
// a tile of V vectors of length L must satisfy V*L <= blockDim.x * kEpt.
//
// Twiddles come from a per-length table tw[m] = exp(-2*pi*i*m/L) computed in
// double precision on the host and rounded once to float.
//
// This replaces the cuFFT R2C/C2R calls of the reference
// (src/RLgpuImpl.cu:183 and :218); it is used for the x, y and z passes of the
// 3D transforms in decon_kernels.cu.
#pragma once

#include "common.cuh"

namespace cdx {

constexpr int kMaxStages = 14;
constexpr int kEpt = 16;        // maximum complex elements held per thread per stage
constexpr int kMaxThreads = 512; // FFT kernels launch at most this many threads
// Longest transform: one vector must fit a tile of kMaxThreads * kEpt elements.
constexpr int kMaxFftLen = kMaxThreads * kEpt;

struct FftDev {
  int L;
  int nst;
  int radix[kMaxStages];
  const float2* tw;  // L entries, exp(-2*pi*i*m/L)
};

// ------------------------------------------------------------- constants
// cos(2*pi*m/R) and sin(2*pi*m/R) for the odd radices, m = 0..R-1.
template <int R>
__device__ __forceinline__ float odd_cos(int m);
template <int R>
__device__ __forceinline__ float odd_sin(int m);

template <>
__device__ __forceinline__ float odd_cos<3>(int m) { return m == 0 ? 1.f : -0.5f; }
template <>
__device__ __forceinline__ float odd_sin<3>(int m) {
  return m == 0 ? 0.f : (m == 1 ? 8.660254038e-01f : -8.660254038e-01f);
}
template <>
__device__ __forceinline__ float odd_cos<5>(int m) {
  switch (m) {
    case 0: return 1.f;
    case 1: case 4: return 3.090169944e-01f;
    default: return -8.090169944e-01f;
  }
}
template <>
__device__ __forceinline__ float odd_sin<5>(int m) {
  switch (m) {
    case 0: return 0.f;
    case 1: return 9.510565163e-01f;
    case 2: return 5.877852523e-01f;
    case 3: return -5.877852523e-01f;
    default: return -9.510565163e-01f;
  }
}
template <>
__device__ __forceinline__ float odd_cos<7>(int m) {
  switch (m) {
    case 0: return 1.f;
    case 1: case 6: return 6.234898019e-01f;
    case 2: case 5: return -2.225209340e-01f;
    default: return -9.009688679e-01f;
  }
}
template <>
__device__ __forceinline__ float odd_sin<7>(int m) {
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
__device__ __forceinline__ float odd_cos<9>(int m) {
  switch (m) {
    case 0: return 1.f;
    case 1: case 8: return 7.660444431e-01f;
    case 2: case 7: return 1.736481777e-01f;
    case 3: case 6: return -0.5f;
    default: return -9.396926208e-01f;
  }
}
template <>
__device__ __forceinline__ float odd_sin<9>(int m) {
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
  __device__ __forceinline__ static void run(float2* x) {
    float2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  }
};

// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot_q(float2 a) { return INV ? mul_pi(a) : mul_mi(a); }

template <bool INV>
struct Dft<4, INV> {
  __device__ __forceinline__ static void run(float2* x) {
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
  __device__ __forceinline__ static void run(float2* x) {
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
  __device__ __forceinline__ static void run(float2* x) {
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
  __device__ __forceinline__ static void run(float2* x) {
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

// ------------------------------------------------------------- one stage
// Tile geometry: V vectors, element e of vector v at buf[v*vs + e*es].
// vfast selects the butterfly->thread mapping: true puts consecutive threads
// on consecutive vectors (for interleaved tiles, vs == 1), false on
// consecutive butterflies of one vector (for contiguous vectors, es == 1).
template <int R, bool INV>
__device__ __forceinline__ void stockham_stage(float2* buf, int L, int Ns, int V, int es, int vs,
                                               bool vfast, const float2* __restrict__ tw) {
  constexpr int NB = (kEpt + R - 1) / R;
  // Opaque copies: the butterfly indices below do not depend on the stage
  // counter, and without this the compiler hoists the indices of every radix
  // case out of the stage loop and keeps them all live (heavy spilling).
  int tid = threadIdx.x, T = blockDim.x;
  asm volatile("" : "+r"(tid), "+r"(T), "+r"(L), "+r"(V));
  const int LR = L / R;
  const int nbf = V * LR;
  float2 x[NB][R];
  int jj[NB], vv[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int b = tid + i * T;
    jj[i] = -1;
    if (b < nbf) {
      int j, v;
      if (vfast) {
        v = b % V;
        j = b / V;
      } else {
        j = b % LR;
        v = b / LR;
      }
      jj[i] = j;
      vv[i] = v;
      const float2* src = buf + v * vs + j * es;
#pragma unroll
      for (int r = 0; r < R; ++r) x[i][r] = src[r * LR * es];
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j = jj[i];
    if (j >= 0) {
      const int k = j % Ns;
      if (Ns > 1) {
        const int step = (L / (Ns * R)) * k;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(tw + r * step);
          x[i][r] = INV ? cmulconj(x[i][r], w) : cmul(x[i][r], w);
        }
      }
      Dft<R, INV>::run(x[i]);
      float2* dst = buf + vv[i] * vs + ((j - k) * R + k) * es;
#pragma unroll
      for (int q = 0; q < R; ++q) dst[q * Ns * es] = x[i][q];
    }
  }
  __syncthreads();
}

// Transform V vectors of length f.L in place.  The plan lists its radices in
// the fixed order 16..., {8|4|2}, 9..., 3..., 7..., 5... (see factorize()),
// so the stages run as one homogeneous loop per radix.  (A single loop with a
// switch on the radix makes the compiler keep every case's registers live.)
// Caller must have synchronised after filling the tile; returns after a final
// __syncthreads().
template <int R, bool INV>
__device__ __forceinline__ int run_radix(float2* buf, const FftDev& f, int& s, int Ns, int V,
                                         int es, int vs, bool vfast) {
  while (s < f.nst && f.radix[s] == R) {
    stockham_stage<R, INV>(buf, f.L, Ns, V, es, vs, vfast, f.tw);
    Ns *= R;
    ++s;
  }
  return Ns;
}

template <bool INV>
__device__ void fft_tile(float2* buf, const FftDev& f, int V, int es, int vs, bool vfast) {
  int s = 0, Ns = 1;
  Ns = run_radix<16, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<8, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<4, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<2, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<9, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<3, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<7, INV>(buf, f, s, Ns, V, es, vs, vfast);
  Ns = run_radix<5, INV>(buf, f, s, Ns, V, es, vs, vfast);
}

}  // namespace cdx
