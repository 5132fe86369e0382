// Compile-time specialised Stockham transforms for a registry of common
// lengths (the generic engine in fft_engine.cuh handles every other length).
//
// A plan SPlan<L, Q0, Q1, ...> fixes the length and the radices (composite
// radices up to 32 points, computed in registers by DftS).  Every index is
// divided by a compile-time constant, the stage sequence is unrolled, and a
// block has one thread per butterfly of the widest stage, so each thread
// holds exactly one butterfly per stage.  The twiddle layout is the same as
// the generic engine's (stage s at offset Ns-1, [r-1][k]), built on the host
// for the plan's radices.  Lengths that split into two radices (756 = 28*27,
// 100 = 10*10, 256 = 16*16, 1024 = 32*32) need one shared-memory round trip.
#pragma once

#include "dft_static.cuh"

namespace cdx {

template <int L, int... Qs>
struct SPlan {
  static constexpr int kL = L;
  static constexpr int kN = sizeof...(Qs);
  static constexpr int kQ[kN] = {Qs...};
  __host__ __device__ static constexpr int q(int s) { return kQ[s]; }
  // span of stage s: product of the radices before it
  __host__ __device__ static constexpr int ns(int s) {
    int n = 1;
    for (int i = 0; i < s; ++i) n *= kQ[i];
    return n;
  }
  __host__ __device__ static constexpr int qmin() {
    int m = kQ[0];
    for (int i = 1; i < kN; ++i) m = kQ[i] < m ? kQ[i] : m;
    return m;
  }
  __host__ __device__ static constexpr int prod() {
    int p = 1;
    for (int i = 0; i < kN; ++i) p *= kQ[i];
    return p;
  }
  static_assert(prod() == L, "radices must multiply to the length");
};

// Threads a block needs for V vectors: one per butterfly of the widest stage.
template <class Plan, int V>
constexpr int splan_threads() {
  const int t = V * (Plan::kL / Plan::qmin());
  return ((t + 31) / 32) * 32;
}

// One stage: radix Q, span NS.  Thread b owns butterfly b (if b < V*L/Q).
template <int L, int Q, int NS, bool INV, int V, bool VFAST, bool SYNC_MID, bool SYNC_END, class Ld,
          class St>
__device__ __forceinline__ void sstage(const float2* stw, const Ld& ld, const St& st) {
  constexpr int LR = L / Q;
  constexpr int nbf = V * LR;
  const int b = threadIdx.x;
  const bool act = b < nbf;
  int j = 0, v = 0;
  if (VFAST) {
    j = b / V;
    v = b - j * V;
  } else {
    v = b / LR;
    j = b - v * LR;
  }
  float2 x[Q];
  if (act) {
#pragma unroll
    for (int r = 0; r < Q; ++r) x[r] = ld.ld(v, j + r * LR);
  }
  if (SYNC_MID) __syncthreads();
  if (act) {
    const int k = j % NS;
    if constexpr (NS > 1) {
      const float2* tw = stw + (NS - 1) + k;
#pragma unroll
      for (int r = 1; r < Q; ++r) {
        const float2 w = tw[(r - 1) * NS];
        x[r] = INV ? cmulconj(x[r], w) : cmul(x[r], w);
      }
    }
    DftS<Q, INV>::run(x);
    store_group<Q>(st, v, (j - k) * Q + k, NS, x);
  }
  if (SYNC_END) __syncthreads();
}

// Full transform; same contract as fft_run (fft_engine.cuh): the first stage
// reads with ld0, the last writes with stL, the stages between work in place
// on io; ends with a barrier when stL writes shared memory.
template <class Plan, bool INV, int V, bool VFAST, class Ld0, class StL>
__device__ __forceinline__ void sfft_run(const float2* stw, const SmemIO& io, const Ld0& ld0,
                                         const StL& stL) {
  constexpr int L = Plan::kL;
  constexpr int N = Plan::kN;
  if constexpr (N == 1) {
    sstage<L, Plan::q(0), 1, INV, V, VFAST, true, StL::kSmem>(stw, ld0, stL);
  } else {
    sstage<L, Plan::q(0), 1, INV, V, VFAST, Ld0::kSmem, true>(stw, ld0, io);
    static_for<N - 2>([&](auto sc) {
      constexpr int s = decltype(sc)::value + 1;
      sstage<L, Plan::q(s), Plan::ns(s), INV, V, VFAST, true, true>(stw, io, io);
    });
    sstage<L, Plan::q(N - 1), Plan::ns(N - 1), INV, V, VFAST, true, StL::kSmem>(stw, io, stL);
  }
}

// Runners: the pass kernels are templates over how they transform their tile.
struct GenericRunner {
  static constexpr bool kStatic = false;
  template <bool INV, class Ld0, class StL>
  __device__ __forceinline__ static void run(const FftDev& f, int V, float invV, bool vfast,
                                             const float2* stw, const SmemIO& io, const Ld0& ld0,
                                             const StL& stL) {
    fft_run<INV>(f, V, invV, vfast, stw, io, ld0, stL);
  }
};

template <class Plan, int V, bool VFAST>
struct StaticRunner {
  static constexpr bool kStatic = true;
  template <bool INV, class Ld0, class StL>
  __device__ __forceinline__ static void run(const FftDev&, int, float, bool, const float2* stw,
                                             const SmemIO& io, const Ld0& ld0, const StL& stL) {
    sfft_run<Plan, INV, V, VFAST>(stw, io, ld0, stL);
  }
};

}  // namespace cdx
