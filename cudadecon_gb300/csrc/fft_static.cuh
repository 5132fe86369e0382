// Compile-time specialised Stockham transforms for a registry of common
// lengths (the generic engine in fft_engine.cuh handles every other length).
//
// A plan SPlan<L, Q0, Q1, ...> fixes the length and the radices (composite
// radices up to 32 points, computed in registers by DftS).  Every index is
// divided by a compile-time constant, the stage sequence is unrolled, and a
// block has one thread per butterfly of the widest stage, so each thread
// holds exactly one butterfly per stage.  The twiddle layout is the same as
// the generic engine's (stage s at offset Ns-1, [r-1][k]), built on the host
// for the plan's radices.  Lengths that split into two radices (100 = 10*10,
// 256 = 16*16, 1024 = 32*32) need one shared-memory round trip; three radices
// (756 = 9*12*7) cost a second round trip but hold fewer registers per thread
// and let a block own fewer rows.
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
  __host__ __device__ static constexpr int qmax() {
    int m = kQ[0];
    for (int i = 1; i < kN; ++i) m = kQ[i] > m ? kQ[i] : m;
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
__host__ __device__ constexpr int splan_threads() {
  const int t = V * (Plan::kL / Plan::qmin());
  return ((t + 31) / 32) * 32;
}

// Loaders that read element R*LR + j (0 <= j < LR) of a vector through
// ld_at<R, LR>(v, j), with R and LR compile-time (kLdAt) -- see sstage.
template <class T, class = void>
struct has_ld_at : std::false_type {};
template <class T>
struct has_ld_at<T, std::void_t<decltype(T::kLdAt)>> : std::bool_constant<T::kLdAt> {};

// Storers that can write two neighbouring elements as one 16-byte store
// (kPair; st2 with its alignment test) -- see sstage.
template <class T, class = void>
struct has_pair : std::false_type {};
template <class T>
struct has_pair<T, std::void_t<decltype(T::kPair)>> : std::bool_constant<T::kPair> {};

// One stage: radix Q, span NS.  Thread b owns butterfly b (if b < V*L/Q).
template <int L, int Q, int NS, bool INV, int V, bool VFAST, bool SYNC_MID, bool SYNC_END, class Ld,
          class St, bool GTW = false>
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
    if constexpr (!VFAST && has_ld_at<Ld>::value) {
      static_for<Q>([&](auto rc) {
        constexpr int r = decltype(rc)::value;
        x[r] = ld.template ld_at<r, LR>(v, j);
      });
    } else {
#pragma unroll
      for (int r = 0; r < Q; ++r) x[r] = ld.ld(v, j + r * LR);
    }
  }
  if (SYNC_MID) __syncthreads();
  if (act) {
    const int k = j % NS;
    if constexpr (NS > 1) {
      const float2* tw = stw + (NS - 1) + k;
#pragma unroll
      for (int r = 1; r < Q; ++r) {
        const float2 w = GTW ? __ldg(tw + (r - 1) * NS) : tw[(r - 1) * NS];
        x[r] = INV ? cmulconj(x[r], w) : cmul(x[r], w);
      }
    }
    DftS<Q, INV>::run(x);
    if constexpr (!VFAST && NS == 1 && Q % 2 == 0 && has_pair<St>::value) {
      // first stage of a row plan: butterfly j's outputs land at j*Q + q,
      // contiguous, and a half-warp's strided float2 stores (stride Q) hit
      // each bank twice or more for even Q; as 16-byte pairs the stride is
      // Q/2 float4s, which for Q = 10, 14 or 6 reaches every bank once, and
      // the stage issues half the stores.  The tile and row pitch are
      // 16-byte aligned in every kernel that uses it (st.pair_ok checks).
      if (st.pair_ok()) {
#pragma unroll
        for (int q = 0; q < Q; q += 2) st.st2(v, j * Q + q, x[q], x[q + 1]);
      } else {
        store_group<Q>(st, v, j * Q, 1, x);
      }
    } else {
      store_group<Q>(st, v, (j - k) * Q + k, NS, x);
    }
  }
  if (SYNC_END) __syncthreads();
}

// Unpadded tile in natural order: element e of vector v at sm[v * vs + e].
// The static transforms read and write natural-order tiles at unit stride
// across threads (element j + r*LR of butterfly j), so they need no padding.
struct NatIO {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  static constexpr bool kPair = true;
  float2* sm;
  int vs;
  __device__ __forceinline__ float2 ld(int v, int e) const { return sm[v * vs + e]; }
  __device__ __forceinline__ void st(int v, int e, float2 x) const { sm[v * vs + e] = x; }
  // pairs (e, e + 1) with e even are 16-byte aligned when the tile and the
  // row pitch are
  __device__ __forceinline__ bool pair_ok() const {
    return ((reinterpret_cast<unsigned long long>(sm) & 15) | (vs & 1)) == 0;
  }
  __device__ __forceinline__ void st2(int v, int e, float2 a, float2 b) const {
    *reinterpret_cast<float4*>(sm + v * vs + e) = make_float4(a.x, a.y, b.x, b.y);
  }
};

// A row tile with one float2 of padding after every B (B = 0: none): the
// layout between two stages of a three-radix row plan.  The stage before it
// writes at stride Q0 (first stage) or in runs of the span, which for even
// radices or short spans puts several threads of a half-warp on the same
// bank; the padding spreads them.  B is chosen per plan and boundary from a
// bank model of both stages' accesses (gen_plans.py), and B >= 16 keeps the
// tile within the padded size spad_size(V*L) the launchers allocate.
template <int B>
struct PadIO {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  static_assert(B == 0 || B >= 16, "padding period below the allocated slack");
  float2* sm;
  int vs;
  __device__ __forceinline__ int ix(int v, int e) const {
    const int t = v * vs + e;
    return B > 0 ? t + t / B : t;
  }
  __device__ __forceinline__ float2 ld(int v, int e) const { return sm[ix(v, e)]; }
  __device__ __forceinline__ void st(int v, int e, float2 x) const { sm[ix(v, e)] = x; }
};

// Float2s of the middle layout of a two-radix plan over V vectors.
template <class Plan, int V>
constexpr int splan_mid_size() {
  return V * Plan::q(1) * (Plan::q(0) + 1);
}

// Two-radix transform L = Q0*Q1 over V vectors laid out one per group of
// threads.  Stage 0 (radix Q0, Q1 butterflies per vector) writes output q of
// butterfly j to element j*Q0 + q; stage 1 (radix Q1, span Q0) reads
// element j + r*Q0.  Both index a [Q1][Q0] array per vector, stored here
// with rows padded to Q0+1: writes then go to distinct banks, and each
// thread's addresses are a base plus compile-time offsets.  tile holds
// splan_mid_size<Plan, V>() float2s and may alias the sources of ld0 and the
// destinations of stL (the stages synchronise between reads and writes).
template <class Plan, bool INV, int V, bool GTW, class Ld0, class StL>
__device__ __forceinline__ void sfft2_rows(const float2* stw, float2* tile, const Ld0& ld0,
                                           const StL& stL) {
  constexpr int Q0 = Plan::q(0), Q1 = Plan::q(1);
  constexpr int RS = Q0 + 1;   // padded row
  constexpr int VS = Q1 * RS;  // vector
  const int b = threadIdx.x;
  {
    const bool act = b < V * Q1;
    const int v = b / Q1;
    const int j = b - v * Q1;
    float2 x[Q0];
    if (act) {
      if constexpr (has_ld_at<Ld0>::value) {
        static_for<Q0>([&](auto rc) {
          constexpr int r = decltype(rc)::value;
          x[r] = ld0.template ld_at<r, Q1>(v, j);
        });
      } else {
#pragma unroll
        for (int r = 0; r < Q0; ++r) x[r] = ld0.ld(v, j + r * Q1);
      }
    }
    if (Ld0::kSmem) __syncthreads();
    if (act) {
      DftS<Q0, INV>::run(x);
      float2* o = tile + v * VS + j * RS;
#pragma unroll
      for (int q = 0; q < Q0; ++q) o[q] = x[q];
    }
    __syncthreads();
  }
  {
    const bool act = b < V * Q0;
    const int v = b / Q0;
    const int j = b - v * Q0;
    float2 x[Q1];
    if (act) {
      const float2* i = tile + v * VS + j;
#pragma unroll
      for (int r = 0; r < Q1; ++r) x[r] = i[r * RS];
    }
    if (StL::kSmem) __syncthreads();
    if (act) {
      const float2* tw = stw + (Q0 - 1) + j;
#pragma unroll
      for (int r = 1; r < Q1; ++r) {
        const float2 w = GTW ? __ldg(tw + (r - 1) * Q0) : tw[(r - 1) * Q0];
        x[r] = INV ? cmulconj(x[r], w) : cmul(x[r], w);
      }
      DftS<Q1, INV>::run(x);
      store_group<Q1>(stL, v, j, Q0, x);
    }
    if (StL::kSmem) __syncthreads();
  }
}

// Interleaved tile of V columns: element e of column v at sm[e * V + v].
// Consecutive threads own consecutive columns, so every access of a stage
// touches V consecutive float2s and the tile needs no padding.
template <int V>
struct ColIO {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  float2* sm;
  __device__ __forceinline__ float2 ld(int v, int e) const { return sm[e * V + v]; }
  __device__ __forceinline__ void st(int v, int e, float2 x) const { sm[e * V + v] = x; }
};

// Two-radix transform over V interleaved columns (thread b owns column
// b % V).  Same stage arithmetic as sfft2_rows; the middle array is stored
// interleaved like the tile ([Q1][Q0] per column, column fastest).
template <class Plan, bool INV, int V, class Ld0, class StL>
__device__ __forceinline__ void sfft2_cols(const float2* stw, float2* tile, const Ld0& ld0,
                                           const StL& stL) {
  constexpr int Q0 = Plan::q(0), Q1 = Plan::q(1);
  const int b = threadIdx.x;
  {
    const bool act = b < V * Q1;
    const int j = b / V;
    const int v = b - j * V;
    float2 x[Q0];
    if (act) {
#pragma unroll
      for (int r = 0; r < Q0; ++r) x[r] = ld0.ld(v, j + r * Q1);
    }
    if (Ld0::kSmem) __syncthreads();
    if (act) {
      DftS<Q0, INV>::run(x);
      float2* o = tile + (j * Q0) * V + v;
#pragma unroll
      for (int q = 0; q < Q0; ++q) o[q * V] = x[q];
    }
    __syncthreads();
  }
  {
    const bool act = b < V * Q0;
    const int j = b / V;
    const int v = b - j * V;
    float2 x[Q1];
    if (act) {
      const float2* i = tile + j * V + v;
#pragma unroll
      for (int r = 0; r < Q1; ++r) x[r] = i[r * Q0 * V];
    }
    if (StL::kSmem) __syncthreads();
    if (act) {
      const float2* tw = stw + (Q0 - 1) + j;
#pragma unroll
      for (int r = 1; r < Q1; ++r) {
        const float2 w = tw[(r - 1) * Q0];
        x[r] = INV ? cmulconj(x[r], w) : cmul(x[r], w);
      }
      DftS<Q1, INV>::run(x);
      store_group<Q1>(stL, v, j, Q0, x);
    }
    if (StL::kSmem) __syncthreads();
  }
}

// Full transform; same contract as fft_run (fft_engine.cuh): the first stage
// reads with ld0, the last writes with stL, the stages between work in place
// on io; ends with a barrier when stL writes shared memory.
template <class Plan, bool INV, int V, bool VFAST, bool GTW, int B0, int B1, class IO, class Ld0,
          class StL>
__device__ __forceinline__ void sfft_run(const float2* stw, const IO& io, const Ld0& ld0,
                                         const StL& stL) {
  constexpr int L = Plan::kL;
  constexpr int N = Plan::kN;
  static_assert(!GTW || !VFAST, "global twiddles: row plans only");
  if constexpr (N == 2 && !VFAST) {
    sfft2_rows<Plan, INV, V, GTW>(stw, io.sm, ld0, stL);
  } else if constexpr (N == 2) {
    sfft2_cols<Plan, INV, V>(stw, io.sm, ld0, stL);
  } else if constexpr (N == 1) {
    sstage<L, Plan::q(0), 1, INV, V, VFAST, true, StL::kSmem, Ld0, StL, GTW>(stw, ld0, stL);
  } else if constexpr (N == 3 && !VFAST && (B0 > 0 || B1 > 0)) {
    // three radices over row tiles with padded layouts between the stages
    const PadIO<B0> m0{io.sm, io.vs};
    const PadIO<B1> m1{io.sm, io.vs};
    sstage<L, Plan::q(0), 1, INV, V, false, Ld0::kSmem, true, Ld0, PadIO<B0>, GTW>(stw, ld0, m0);
    sstage<L, Plan::q(1), Plan::ns(1), INV, V, false, true, true, PadIO<B0>, PadIO<B1>, GTW>(
        stw, m0, m1);
    sstage<L, Plan::q(2), Plan::ns(2), INV, V, false, StL::kSmem, StL::kSmem, PadIO<B1>, StL,
           GTW>(stw, m1, stL);
  } else {
    // three or more radices: the stages between work in place on the
    // natural-order tile (unit-stride reads; the first stage writes at
    // stride Q0, conflict-free for odd Q0)
    sstage<L, Plan::q(0), 1, INV, V, VFAST, Ld0::kSmem, true, Ld0, IO, GTW>(stw, ld0, io);
    static_for<N - 2>([&](auto sc) {
      constexpr int s = decltype(sc)::value + 1;
      sstage<L, Plan::q(s), Plan::ns(s), INV, V, VFAST, true, true, IO, IO, GTW>(stw, io, io);
    });
    // the last stage's reads and writes need a barrier between them only when
    // its storer writes shared memory
    sstage<L, Plan::q(N - 1), Plan::ns(N - 1), INV, V, VFAST, StL::kSmem, StL::kSmem, IO, StL,
           GTW>(stw, io, stL);
  }
}

// Runners: the pass kernels are templates over how they transform their tile.
// Runner::Tile is the natural-order tile type the pass kernels hand to the
// transform (row tiles: element e of vector v; the generic engine pads it).
struct GenericRunner {
  static constexpr bool kStatic = false;
  static constexpr int kV = 0;  // vectors per tile: runtime
  static constexpr int kThreads = kMaxThreads;  // most threads a block is launched with
  template <int TARGET>
  static constexpr int min_blocks() { return 1; }
  static constexpr bool kGlobalTw = false;
  static constexpr int kTileF2 = 0;  // tile size: from the runtime geometry
  using Tile = SmemIO;
  __device__ __forceinline__ static Tile row_tile(float2* sm, int L) { return SmemIO{sm, 1, L}; }
  __device__ __forceinline__ static SmemIO col_tile(float2* sm, int W) { return SmemIO{sm, W, 1}; }
  template <bool INV, class Ld0, class StL>
  __device__ __forceinline__ static void run(const FftDev& f, int V, float invV, bool vfast,
                                             const float2* stw, const SmemIO& io, const Ld0& ld0,
                                             const StL& stL) {
    fft_run<INV>(f, V, invV, vfast, stw, io, ld0, stL);
  }
};

// GTW: the stage twiddles are read from the global table (through the
// read-only cache) instead of a shared-memory copy, which saves the kernel
// L float2s of shared memory.  REGX: registers per thread added to the
// estimate behind the launch bounds (fewer blocks per SM, more registers
// for each thread).  B0, B1: padding periods of the layouts after the first
// and the second stage of a three-radix row plan (PadIO; 0 = natural).
template <class Plan, int V, bool VFAST, bool GTW = false, int REGX = 0, int B0 = 0, int B1 = 0>
struct StaticRunner {
  static constexpr bool kStatic = true;
  static constexpr int kV = V;
  static constexpr int kThreads = splan_threads<Plan, V>();
  // Blocks per SM to ask the compiler to fit (launch bounds): TARGET, lowered
  // so that each thread keeps about 2*qmax + 22 + REGX registers (the
  // radix's values plus addresses and twiddles).
  template <int TARGET>
  static constexpr int min_blocks() {
    const int fit = 65536 / (kThreads * (2 * Plan::qmax() + 22 + REGX));
    const int b = TARGET < fit ? TARGET : fit;
    return b < 1 ? 1 : b;
  }
  using SPlanT = Plan;
  static constexpr bool kGlobalTw = GTW;
  // float2s of a row tile: the middle layout, the natural layout and the
  // staged half spectra (V vectors of L/2+1 float4) share it
  static constexpr int kTileF2 = [] {
    int m = splan_mid_size<Plan, V>();
    if (V * Plan::kL > m) m = V * Plan::kL;
    if ((B0 > 0 || B1 > 0) && spad_size(V * Plan::kL) > m) m = spad_size(V * Plan::kL);
    if (2 * (Plan::kL / 2 + 1) * V > m) m = 2 * (Plan::kL / 2 + 1) * V;
    return m + (m & 1);
  }();
  using Tile = NatIO;
  __device__ __forceinline__ static Tile row_tile(float2* sm, int L) { return NatIO{sm, L}; }
  __device__ __forceinline__ static ColIO<V> col_tile(float2* sm, int) { return ColIO<V>{sm}; }
  template <bool INV, class IO, class Ld0, class StL>
  __device__ __forceinline__ static void run(const FftDev&, int, float, bool, const float2* stw,
                                             const IO& io, const Ld0& ld0, const StL& stL) {
    sfft_run<Plan, INV, V, VFAST, GTW, B0, B1>(stw, io, ld0, stL);
  }
};

// Vectors per tile: the runner's compile-time count, else the runtime one
// (index arithmetic over the tile then divides by a constant).
template <class Run>
__device__ __forceinline__ int tile_vectors(int v) {
  return Run::kV > 0 ? Run::kV : v;
}

// idx / d and idx % d for 0 <= idx < 2^22: by the constant when D > 0, else
// through fdiv with the float reciprocal inv_d of the runtime d.
template <int D>
__device__ __forceinline__ void divmod_small(int idx, int d, float inv_d, int& q, int& r) {
  if constexpr (D > 0) {
    q = idx / D;
    r = idx - q * D;
  } else {
    q = fdiv(idx, inv_d);
    r = idx - q * d;
  }
}

// A static plan's row tile must fit the padded tile the generic sizing gives
// (spad_size(V*L) float2s), which the pass launchers allocate.
template <class Plan, int V>
constexpr bool splan_rows_fit() {
  return splan_mid_size<Plan, V>() <= spad_size(V * Plan::kL);
}

}  // namespace cdx
