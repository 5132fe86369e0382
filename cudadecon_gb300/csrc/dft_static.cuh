// Compile-time DFTs of any 2,3,5,7-smooth size Q (up to a few dozen points)
// held in registers, for the specialised FFT kernels (fft_static.cuh).
//
// A composite Q = A*B is split Cooley-Tukey style: with n = n1 + A*n2 and
// k = B*k1 + k2,
//   X[B*k1 + k2] = sum_n1 w_A^(n1 k1) * w_Q^(n1 k2) * sum_n2 x[n1 + A n2] w_B^(n2 k2),
// i.e. A DFTs of size B, a twiddle by w_Q^(n1 k2), then B DFTs of size A.
// The twiddles are compile-time constants: cosines and sines evaluated by a
// constexpr Taylor series in double precision and rounded once to float
// (values within 1e-15 of 0 or +-1 are snapped, so that those products fold
// away).  Everything is __host__ __device__ so the code can be checked on the
// CPU against a direct DFT.
#pragma once

#include <type_traits>

#include "fft_engine.cuh"

namespace cdx {

// ---------------------------------------------------------------- constexpr trig
constexpr double kPiD = 3.14159265358979323846264338327950288;

constexpr double ct_sin_series(double x) {
  // x in [-pi, pi]; 24 terms of the Taylor series (error far below 1e-16)
  double term = x, sum = x;
  for (int n = 1; n < 24; ++n) {
    term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
    sum += term;
  }
  return sum;
}

constexpr double ct_cos_series(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n < 24; ++n) {
    term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
    sum += term;
  }
  return sum;
}

// angle 2*pi*m/q reduced to [-pi, pi]
constexpr double ct_angle(int m, int q) {
  const int r = ((m % q) + q) % q;
  double a = 2.0 * kPiD * (double)r / (double)q;
  if (a > kPiD) a -= 2.0 * kPiD;
  return a;
}

constexpr double ct_snap(double v) {
  return (v < 1e-15 && v > -1e-15) ? 0.0
         : (v > 1.0 - 1e-15)       ? 1.0
         : (v < -1.0 + 1e-15)      ? -1.0
                                   : v;
}

// w_q^m = exp(-2*pi*i*m/q) (forward); the inverse uses the conjugate
template <int Q, int M>
struct Tw {
  static constexpr float re = (float)ct_snap(ct_cos_series(ct_angle(M, Q)));
  static constexpr float im = (float)ct_snap(-ct_sin_series(ct_angle(M, Q)));
};

// x * w_q^m (or its conjugate for the inverse), with the trivial cases folded
template <int Q, int M, bool INV>
__host__ __device__ __forceinline__ float2 twmul(float2 x) {
  constexpr float c = Tw<Q, M>::re;
  constexpr float s = INV ? -Tw<Q, M>::im : Tw<Q, M>::im;
  if constexpr (s == 0.f) {
    if constexpr (c == 1.f) return x;
    else if constexpr (c == -1.f) return make_float2(-x.x, -x.y);
    else return make_float2(c * x.x, c * x.y);
  } else if constexpr (c == 0.f) {
    // multiply by i*s
    if constexpr (s == 1.f) return make_float2(-x.y, x.x);
    else if constexpr (s == -1.f) return make_float2(x.y, -x.x);
    else return make_float2(-s * x.y, s * x.x);
  } else {
    return make_float2(c * x.x - s * x.y, c * x.y + s * x.x);
  }
}

// compile-time loop: f(std::integral_constant<int, I>) for I = 0..N-1
template <int N, int I = 0, class F>
__host__ __device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<N, I + 1>(f);
  }
}

// ---------------------------------------------------------------- sizes
constexpr bool ct_is_base(int q) {
  return q == 1 || q == 2 || q == 3 || q == 4 || q == 5 || q == 7 || q == 8 || q == 9 || q == 16;
}

// Split of a composite size: the first factor is the largest hand-written
// size that divides q and leaves a cofactor > 1.
constexpr int ct_split(int q) {
  constexpr int cands[] = {16, 9, 8, 7, 5, 4, 3, 2};
  for (int c : cands)
    if (q % c == 0 && q / c > 1) return c;
  return q;
}

template <int Q, bool INV, class Enable = void>
struct DftS;

// hand-written sizes: reuse the engine's kernels
template <int Q, bool INV>
struct DftS<Q, INV, std::enable_if_t<ct_is_base(Q)>> {
  __host__ __device__ __forceinline__ static void run(float2* x) {
    if constexpr (Q > 1) Dft<Q, INV>::run(x);
  }
};

template <int Q, bool INV>
struct DftS<Q, INV, std::enable_if_t<!ct_is_base(Q)>> {
  static constexpr int A = ct_split(Q);
  static constexpr int B = Q / A;
  __host__ __device__ __forceinline__ static void run(float2* x) {
    float2 t[A][B];
    static_for<A>([&](auto n1c) {
      constexpr int n1 = decltype(n1c)::value;
      float2 a[B];
      static_for<B>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        a[n2] = x[n1 + A * n2];
      });
      DftS<B, INV>::run(a);
      static_for<B>([&](auto k2c) {
        constexpr int k2 = decltype(k2c)::value;
        t[n1][k2] = twmul<Q, n1 * k2, INV>(a[k2]);
      });
    });
    static_for<B>([&](auto k2c) {
      constexpr int k2 = decltype(k2c)::value;
      float2 a[A];
      static_for<A>([&](auto n1c) {
        constexpr int n1 = decltype(n1c)::value;
        a[n1] = t[n1][k2];
      });
      DftS<A, INV>::run(a);
      static_for<A>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        x[B * k1 + k2] = a[k1];
      });
    });
  }
};

}  // namespace cdx
