// The x passes in the mixed-precision tensor-core form: the DFTs of the
// row transforms run as tcgen05 MMAs (kind::tf32) with each FP32 operand
// split into a tf32 high and low part, so that hi*hi + lo*hi + hi*lo,
// accumulated in FP32 in tensor memory, carries about 22 significant bits.
//
// A row of length L = Q0*Q1 (Q0, Q1 <= 32) is transformed in two stages
// (Cooley-Tukey, n = Q1*n1 + n2, k = k1 + Q0*k2):
//   stage 1: for every n2, a DFT of length Q0 over n1    -> A1[k1][n2]
//   twiddle: A1[k1][n2] * W_L^(n2*k1)
//   stage 2: for every k1, a DFT of length Q1 over n2    -> X[k1 + Q0*k2]
// Each stage is one GEMM D = A * B^T: the rows of A are the stage's vectors
// (two real columns per complex element), B is the real 2Q x 2Q form of the
// DFT matrix of the radix, and D lands in tensor memory with row m in lane
// m.  Thread m of a 128-thread warpgroup owns vector m: it writes row m of
// A, reads row m of D (tcgen05.ld), applies the twiddles and writes its
// values into the next stage's rows.  Inverse transforms use
// IDFT(x) = conj(DFT(conj(x))), so only forward DFT matrices and twiddles
// are stored.
//
// Vectors are numbered m = (index within the row) * P + (row pair), P row
// pairs per tile (P*Q <= 128): neighbouring threads then touch neighbouring
// row pairs of the spectrum (one 16-byte group each, 16P contiguous bytes
// per kx) and rows of the real arrays at the same x, so global accesses
// stay sector-efficient without staging.  An inverse transform with radices
// (Q0, Q1) leaves thread (p, k1) holding elements e = k1 + Q0*k2; a forward
// transform with radices (Q1, Q0) reads exactly those elements as its
// stage-1 vector (p, n2 = k1), so the ratio pass goes from one to the other
// in registers.
//
// Kernels are persistent (one or two warpgroups per CTA, each on its own
// tiles, sharing the DFT matrices and twiddles in shared memory) and follow
// the plain kernels' arithmetic for the prediction, the RL ratio, the
// estimate update and the float-float dot products.  Every wait on an MMA
// is bounded (about a second of SM clocks); a wait that runs out sets the
// error word, and the CTA frees its tensor memory and returns.
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "decon_common.cuh"
#include "tc_common.cuh"

namespace cdx {

__host__ __device__ constexpr int tc_pad8(int v) { return (v + 7) / 8 * 8; }
__host__ __device__ constexpr int tc_pad16(int v) { return (v + 15) / 16 * 16; }
__host__ __device__ constexpr unsigned tc_align(unsigned v, unsigned a) { return (v + a - 1) / a * a; }

// Compile-time description of a tensor-core row plan: radices, tile, and
// the shared-memory layout of a CTA with WG warpgroups.
template <int Q0_, int Q1_, int WG_>
struct TcPlan {
  static constexpr int Q0 = Q0_, Q1 = Q1_, L = Q0 * Q1, WG = WG_;
  static constexpr int QM = Q0 > Q1 ? Q0 : Q1;
  static constexpr int P = 128 / QM;  // row pairs per tile
  static constexpr int KP0 = tc_pad8(2 * Q0), NP0 = tc_pad16(2 * Q0);
  static constexpr int KP1 = tc_pad8(2 * Q1), NP1 = tc_pad16(2 * Q1);
  static constexpr int KA = KP0 > KP1 ? KP0 : KP1;  // A row length (floats)
  static constexpr int NPM = NP0 > NP1 ? NP0 : NP1;
  static constexpr int TMEM_COLS = 64 * WG;
  // shared-memory byte offsets
  static constexpr unsigned B0 = 0;                              // DFT_Q0: hi, then lo
  static constexpr unsigned B0SZ = (unsigned)NP0 * KP0 * 4;
  static constexpr unsigned B1 = Q0 == Q1 ? B0 : 2 * B0SZ;       // DFT_Q1
  static constexpr unsigned B1SZ = (unsigned)NP1 * KP1 * 4;
  static constexpr unsigned BEND = Q0 == Q1 ? 2 * B0SZ : 2 * B0SZ + 2 * B1SZ;
  static constexpr unsigned ASZ = 128u * KA * 4;                 // one of hi, lo
  static constexpr unsigned A = tc_align(BEND, 1024);            // per warpgroup: hi, lo
  static constexpr int TWS = Q0 + 1;                             // twiddle row stride
  static constexpr unsigned TW = A + WG * 2 * ASZ;               // [Q1][Q0+1] float2
  static constexpr unsigned MB = tc_align(TW + (unsigned)Q1 * TWS * 8, 16);
  static constexpr unsigned BYTES = MB + 64;  // mbarriers, TMEM slot, flags
  // CTAs per SM the launch bounds ask for (shared memory allows this many)
  static constexpr int MINB_ = (int)((228u * 1024u) / (BYTES + 1024u));
  static constexpr int MINB = MINB_ < 1 ? 1 : (MINB_ > 2 ? 2 : MINB_);
  // exchange tile (natural order, P rows of LX float2) aliases this
  // warpgroup's A
  static constexpr int LX = L + 8;
  static_assert(Q0 <= 32 && Q1 <= 32, "radices up to 32");
  static_assert((unsigned)P * LX * 8 <= 2 * ASZ, "exchange tile must fit the A operand");
  static_assert(BYTES <= 227 * 1024, "shared memory");
};

// Per-warpgroup state.
struct TcWg {
  float* Ahi;
  float* Alo;
  float2* X;  // exchange tile (aliases A)
  uint64_t* mbar;
  unsigned phase;
  unsigned tmem;  // this warpgroup's TMEM columns (lane 0)
  unsigned lane_base;  // (32 * (warp % 4)) << 16
  int t;               // thread within the warpgroup
  int wg;
  bool fail;
};

constexpr long long kTcWaitCycles = 2000000000LL;  // about a second at 2 GHz

__device__ __forceinline__ void wg_bar(int wg) {
  asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory");
}
// Barrier of the warpgroup that also ORs a flag over its threads.
__device__ __forceinline__ bool wg_bar_or(int wg, bool v) {
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "barrier.red.or.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((unsigned)v), "r"(1 + wg)
      : "memory");
  return r != 0;
}

// Write complex element j of A row `row`, split into tf32 hi and lo parts.
template <class TP>
__device__ __forceinline__ void a_put(const TcWg& w, int row, int j, float2 v) {
  float hx, lx, hy, ly;
  tc::tf32_split(v.x, hx, lx);
  tc::tf32_split(v.y, hy, ly);
  const unsigned o = tc::op_offset(row, 2 * j, TP::KA) >> 2;
  *reinterpret_cast<float2*>(w.Ahi + o) = make_float2(hx, hy);
  *reinterpret_cast<float2*>(w.Alo + o) = make_float2(lx, ly);
}

// One stage: the warpgroup's A rows times the radix-Q DFT matrix (at byte
// offset boff of shared memory) into TMEM, then each thread loads its D row
// (NP columns) into d.  All 128 threads call it.
template <class TP, int KP, int NP>
__device__ __forceinline__ void tc_stage(TcWg& w, unsigned char* sm, unsigned boff, float* d) {
  tc::fence_proxy_async();
  tc::fence_before_sync();
  wg_bar(w.wg);
  if (w.t == 0) {
    tc::fence_after_sync();
    const unsigned a_hi = tc::smem_addr(w.Ahi), a_lo = tc::smem_addr(w.Alo);
    const unsigned b_hi = tc::smem_addr(sm + boff);
    const unsigned b_lo = b_hi + (unsigned)NP * KP * 4;
    constexpr uint32_t id = tc::idesc_tf32(128, NP);
    constexpr unsigned a_sbo = TP::KA * 32, b_sbo = KP * 32;
#pragma unroll
    for (int term = 0; term < 3; ++term) {
      const unsigned a = term == 1 ? a_lo : a_hi;
      const unsigned b = term == 2 ? b_lo : b_hi;
#pragma unroll
      for (int kb = 0; kb < KP / 8; ++kb)
        tc::mma_tf32(w.tmem, tc::make_desc(a + kb * 256, 128, a_sbo),
                     tc::make_desc(b + kb * 256, 128, b_sbo), id, (term | kb) != 0);
    }
    tc::mma_commit(w.mbar);
  }
  const bool ok = tc::mbar_wait(w.mbar, w.phase, kTcWaitCycles);
  w.phase ^= 1u;
  w.fail |= !ok;
  tc::fence_after_sync();
#pragma unroll
  for (int c = 0; c < NP; c += 16) {
    float v[16];
    tc::tmem_ld16(w.tmem + w.lane_base + c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) d[c + i] = v[i];
  }
  tc::tmem_wait_ld();
}

// Common set-up of a TC kernel: tables into shared memory, TMEM, mbarriers,
// zeroed A operands.  Returns this thread's warpgroup state.
template <class TP>
__device__ __forceinline__ TcWg tc_setup(unsigned char* sm, const float4* btab, const float4* twtab) {
  const int tid = threadIdx.x;
  for (unsigned i = tid; i < TP::BEND / 16; i += blockDim.x)
    reinterpret_cast<float4*>(sm + TP::B0)[i] = __ldg(btab + i);
  for (unsigned i = tid; i < (unsigned)TP::Q1 * TP::TWS * 8 / 16; i += blockDim.x)
    reinterpret_cast<float4*>(sm + TP::TW)[i] = __ldg(twtab + i);
  for (unsigned i = tid; i < TP::WG * 2 * TP::ASZ / 16; i += blockDim.x)
    reinterpret_cast<float4*>(sm + TP::A)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + TP::MB);
  unsigned* slot = reinterpret_cast<unsigned*>(sm + TP::MB + 32);
  if (tid < 32) tc::tmem_alloc(slot, TP::TMEM_COLS);
  if (tid == 0) {
    for (int i = 0; i < TP::WG; ++i) tc::mbar_init(mbar + i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  TcWg w;
  w.wg = tid >> 7;
  w.t = tid & 127;
  w.Ahi = reinterpret_cast<float*>(sm + TP::A + w.wg * 2 * TP::ASZ);
  w.Alo = reinterpret_cast<float*>(sm + TP::A + w.wg * 2 * TP::ASZ + TP::ASZ);
  w.X = reinterpret_cast<float2*>(w.Ahi);
  w.mbar = mbar + w.wg;
  w.phase = 0;
  w.tmem = *slot + (unsigned)(w.wg * 64);
  w.lane_base = (unsigned)((32 * ((tid >> 5) & 3)) << 16);
  w.fail = false;
  return w;
}

template <class TP>
__device__ __forceinline__ void tc_teardown(unsigned char* sm, bool failed, int* err) {
  if (failed && (threadIdx.x & 127) == 0) atomicExch(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_free(*reinterpret_cast<unsigned*>(sm + TP::MB + 32), TP::TMEM_COLS);
  }
}

__device__ __forceinline__ float2 conj2(float2 a) { return make_float2(a.x, -a.y); }

// Element e of the packed full-length spectrum Z = A + iB of rows (ya, ya+1)
// of slice z, rebuilt from the half spectra as PackedSpecLoad does.
__device__ __forceinline__ float2 packed_spec_g(const float2* __restrict__ S, const Geom& g,
                                                long long zo, int e) {
  const bool lo = e < g.nxh;
  const int k = lo ? e : g.nx - e;
  float4 w = __ldcg(reinterpret_cast<const float4*>(S + (long long)k * g.plane + zo));
  if (k == 0 || 2 * k == g.nx) {
    w.y = 0.f;
    w.w = 0.f;
  }
  return lo ? make_float2(w.x - w.w, w.y + w.z) : make_float2(w.x + w.w, w.z - w.y);
}

// Inverse transform of the packed spectra of the tile's pairs.  On return
// thread t < P*Q0 (pair p = t % P, k1 = t / P) holds z[e] = (row 2p, row
// 2p+1) at e = k1 + Q0*k2 in d[2*k2], d[2*k2+1] (already conjugated back).
template <class TP>
__device__ __forceinline__ void tc_inverse(TcWg& w, unsigned char* sm, const float2* S,
                                           const Geom& g, int z, int y0, float* d) {
  constexpr int Q0 = TP::Q0, Q1 = TP::Q1, P = TP::P;
  const float2* tw = reinterpret_cast<const float2*>(sm + TP::TW);
  const int t = w.t;
  if (t < P * Q1) {
    const int p = t % P, n2 = t / P;
    const int ya = y0 + 2 * p;
    const long long zo = (long long)z * g.nyp + ya;
    // every load of the vector first (the stores into A would otherwise
    // keep the compiler from moving later loads ahead of them)
    float2 v[Q0];
#pragma unroll
    for (int n1 = 0; n1 < Q0; ++n1)
      v[n1] = ya < g.ny ? packed_spec_g(S, g, zo, Q1 * n1 + n2) : make_float2(0.f, 0.f);
#pragma unroll
    for (int n1 = 0; n1 < Q0; ++n1) a_put<TP>(w, t, n1, conj2(v[n1]));
  }
  tc_stage<TP, TP::KP0, TP::NP0>(w, sm, TP::B0, d);
  if (t < P * Q1) {
    const int p = t % P, n2 = t / P;
    float2 c[Q0];
#pragma unroll
    for (int k1 = 0; k1 < Q0; ++k1) c[k1] = tw[n2 * TP::TWS + k1];
#pragma unroll
    for (int k1 = 0; k1 < Q0; ++k1)
      a_put<TP>(w, k1 * P + p, n2, cmul(make_float2(d[2 * k1], d[2 * k1 + 1]), c[k1]));
  }
  tc_stage<TP, TP::KP1, TP::NP1>(w, sm, TP::B1, d);
#pragma unroll
  for (int k2 = 0; k2 < Q1; ++k2) d[2 * k2 + 1] = -d[2 * k2 + 1];
}

// Forward transform whose stage-1 rows have been written (radices QA then
// QB, L = QA*QB, A rows m = n2*P + p with elements n1 < QA, n2 < QB).  Ends
// with the spectrum of each pair in the exchange tile X[p*LX + k], natural
// order, and a warpgroup barrier.  BA/BB: byte offsets of the DFT matrices
// of QA and QB; TWT: twiddle W_L^(n2*k1) is tw[k1*TWS + n2] when true (the
// table transposed), tw[n2*TWS + k1] when false.
template <class TP, int QA, int QB, int KPA, int NPA, int KPB, int NPB, bool TWT>
__device__ __forceinline__ void tc_forward_rest(TcWg& w, unsigned char* sm, unsigned BA,
                                                unsigned BB, float* d) {
  constexpr int P = TP::P;
  const float2* tw = reinterpret_cast<const float2*>(sm + TP::TW);
  const int t = w.t;
  tc_stage<TP, KPA, NPA>(w, sm, BA, d);
  if (t < P * QB) {
    const int p = t % P, n2 = t / P;
    float2 c[QA];
#pragma unroll
    for (int k1 = 0; k1 < QA; ++k1) c[k1] = TWT ? tw[k1 * TP::TWS + n2] : tw[n2 * TP::TWS + k1];
#pragma unroll
    for (int k1 = 0; k1 < QA; ++k1)
      a_put<TP>(w, k1 * P + p, n2, cmul(make_float2(d[2 * k1], d[2 * k1 + 1]), c[k1]));
  }
  tc_stage<TP, KPB, NPB>(w, sm, BB, d);
  // the last MMA has read A: the exchange tile may overwrite it
  tc::fence_proxy_async();
  if (t < P * QA) {
    const int p = t % P, k1 = t / P;
    float2* x = w.X + p * TP::LX;
#pragma unroll
    for (int k2 = 0; k2 < QB; ++k2) x[k1 + QA * k2] = make_float2(d[2 * k2], d[2 * k2 + 1]);
  }
  wg_bar(w.wg);
}

// Split the packed spectra in the exchange tile into half spectra and store
// them to S (as store_half_spectra), then a barrier before A is reused.
template <class TP>
__device__ __forceinline__ void tc_store_spectra(TcWg& w, const Geom& g, int z, int y0,
                                                 float2* S) {
  constexpr int P = TP::P, L = TP::L;
  for (int idx = w.t; idx < g.nxh * P; idx += 128) {
    const int k = idx / P, p = idx - (idx / P) * P;
    const int ya = y0 + 2 * p;
    if (ya >= g.ny) continue;
    const float2* x = w.X + p * TP::LX;
    const float2 zk = x[k];
    const float2 zm = x[k == 0 ? 0 : L - k];
    *reinterpret_cast<float4*>(S + (long long)k * g.plane + (long long)z * g.nyp + ya) =
        split_pair(zk, zm);
  }
  wg_bar(w.wg);
}

// ---------------------------------------------------------------- kernels
// Forward x pass (k_x_fwd's contract): Y from X, X_{k-1} and lambda
// (written over Xm1 when predict), then the R2C of row pairs into S.
template <class TP>
__global__ void __launch_bounds__(128 * TP::WG, TP::MINB)
k_xtc_fwd(Geom g, const float4* btab, const float4* twtab, const float* X, float* Xm1,
          const float* lam, int predict, float2* S, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  constexpr int Q0 = TP::Q0, Q1 = TP::Q1, P = TP::P;
  TcWg w = tc_setup<TP>(sm, btab, twtab);
  grid_dep_wait();
  grid_dep_launch();
  const float lamv = predict ? *lam : 0.f;
  const int tiles_y = (g.ny + 2 * P - 1) / (2 * P);
  const int ntiles = tiles_y * g.nz;
  float d[TP::NPM];
  for (int tile = blockIdx.x * TP::WG + w.wg; tile < ntiles; tile += gridDim.x * TP::WG) {
    const int z = tile / tiles_y;
    const int y0 = (tile - z * tiles_y) * 2 * P;
    const int t = w.t;
    if (t < P * Q1) {
      const int p = t % P, n2 = t / P;
      const int ya = y0 + 2 * p;
      const long long o = ((long long)z * g.ny + ya) * g.nx;
      const bool va = ya < g.ny, vb = ya + 1 < g.ny;
      // loads first, then the prediction, its stores and the A rows
      float2 xv[Q0], mv[Q0];
#pragma unroll
      for (int n1 = 0; n1 < Q0; ++n1) {
        const long long i = o + Q1 * n1 + n2;
        xv[n1] = make_float2(va ? __ldcs(X + i) : 0.f, vb ? __ldcs(X + i + g.nx) : 0.f);
        if (predict)
          mv[n1] = make_float2(va ? __ldcs(Xm1 + i) : 0.f, vb ? __ldcs(Xm1 + i + g.nx) : 0.f);
      }
#pragma unroll
      for (int n1 = 0; n1 < Q0; ++n1) {
        const long long i = o + Q1 * n1 + n2;
        float2 yv = xv[n1];
        if (predict) {
          yv.x = predict_y(yv.x, mv[n1].x, lamv);
          yv.y = predict_y(yv.y, mv[n1].y, lamv);
          if (va) __stcs(Xm1 + i, yv.x);
          if (vb) __stcs(Xm1 + i + g.nx, yv.y);
        }
        a_put<TP>(w, t, n1, yv);
      }
    }
    tc_forward_rest<TP, Q0, Q1, TP::KP0, TP::NP0, TP::KP1, TP::NP1, false>(w, sm, TP::B0, TP::B1,
                                                                          d);
    tc_store_spectra<TP>(w, g, z, y0, S);
    if (wg_bar_or(w.wg, w.fail)) break;
  }
  tc_teardown<TP>(sm, w.fail, err);
}

// Inverse x pass, RL ratio, forward x pass of the ratio (k_x_inv_ratio_fwd's
// contract).
template <class TP>
__global__ void __launch_bounds__(128 * TP::WG, TP::MINB)
k_xtc_ratio(Geom g, const float4* btab, const float4* twtab, float2* S, const float* raw,
            float eps, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  constexpr int Q0 = TP::Q0, Q1 = TP::Q1, P = TP::P;
  TcWg w = tc_setup<TP>(sm, btab, twtab);
  grid_dep_wait();
  grid_dep_launch();
  const int tiles_y = (g.ny + 2 * P - 1) / (2 * P);
  const int ntiles = tiles_y * g.nz;
  float d[TP::NPM];
  for (int tile = blockIdx.x * TP::WG + w.wg; tile < ntiles; tile += gridDim.x * TP::WG) {
    const int z = tile / tiles_y;
    const int y0 = (tile - z * tiles_y) * 2 * P;
    tc_inverse<TP>(w, sm, S, g, z, y0, d);
    const int t = w.t;
    if (t < P * Q0) {
      // ratio on elements e = k1 + Q0*k2, written as the forward stage-1
      // vector (p, n2 = k1) with elements n1 = k2 (radices Q1 then Q0)
      const int p = t % P, k1 = t / P;
      const int ya = y0 + 2 * p;
      const long long o = ((long long)z * g.ny + ya) * g.nx;
      const bool va = ya < g.ny, vb = ya + 1 < g.ny;
      float2 rv[Q1];
#pragma unroll
      for (int k2 = 0; k2 < Q1; ++k2) {
        const long long i = o + k1 + Q0 * k2;
        rv[k2] = make_float2(va ? __ldcs(raw + i) : 0.f, vb ? __ldcs(raw + i + g.nx) : 0.f);
      }
#pragma unroll
      for (int k2 = 0; k2 < Q1; ++k2) {
        float2 r = make_float2(0.f, 0.f);
        if (va) r.x = rl_ratio(d[2 * k2], rv[k2].x, eps);
        if (vb) r.y = rl_ratio(d[2 * k2 + 1], rv[k2].y, eps);
        a_put<TP>(w, t, k2, r);
      }
    }
    tc_forward_rest<TP, Q1, Q0, TP::KP1, TP::NP1, TP::KP0, TP::NP0, true>(w, sm, TP::B1, TP::B0,
                                                                         d);
    tc_store_spectra<TP>(w, g, z, y0, S);
    if (wg_bar_or(w.wg, w.fail)) break;
  }
  tc_teardown<TP>(sm, w.fail, err);
}

// Inverse x pass with the estimate update and the dot products
// (k_x_inv_update's contract; one float-float partial per CTA).
template <class TP>
__global__ void __launch_bounds__(128 * TP::WG, TP::MINB)
k_xtc_update(Geom g, const float4* btab, const float4* twtab, const float2* S, const float* Y,
             float* Xout, float* G, int dots, float4* partials, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ float4 red[32];
  constexpr int Q0 = TP::Q0, Q1 = TP::Q1, P = TP::P;
  TcWg w = tc_setup<TP>(sm, btab, twtab);
  grid_dep_wait();
  grid_dep_launch();
  const int tiles_y = (g.ny + 2 * P - 1) / (2 * P);
  const int ntiles = tiles_y * g.nz;
  float d[TP::NPM];
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int tile = blockIdx.x * TP::WG + w.wg; tile < ntiles; tile += gridDim.x * TP::WG) {
    const int z = tile / tiles_y;
    const int y0 = (tile - z * tiles_y) * 2 * P;
    tc_inverse<TP>(w, sm, S, g, z, y0, d);
    const int t = w.t;
    if (t < P * Q0) {
      const int p = t % P, k1 = t / P;
      const int ya = y0 + 2 * p;
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        if (ya + r >= g.ny) break;
        const long long o = ((long long)z * g.ny + ya + r) * g.nx + k1;
        // the row's loads first (Xout may alias Y, so a store would keep
        // later loads behind it)
        float yv[Q1], gv[Q1];
#pragma unroll
        for (int k2 = 0; k2 < Q1; ++k2) {
          yv[k2] = __ldcs(Y + o + Q0 * k2);
          gv[k2] = dots ? __ldcs(G + o + Q0 * k2) : 0.f;
        }
#pragma unroll
        for (int k2 = 0; k2 < Q1; ++k2) {
          const long long i = o + Q0 * k2;
          float xn = __fmul_rn(d[2 * k2 + r], yv[k2]);
          xn = xn > 0.f ? xn : 0.f;
          const float gn = __fsub_rn(xn, yv[k2]);
          if (dots) {
            acc_add(acc[0], acc[1], __fmul_rn(gn, gv[k2]));
            acc_add(acc[2], acc[3], __fmul_rn(gv[k2], gv[k2]));
          }
          Xout[i] = xn;
          __stcs(G + i, gn);
        }
      }
    }
    // the next tile rewrites A: every thread is past this tile's last MMA
    if (wg_bar_or(w.wg, w.fail)) break;
  }
  if (dots) {
    __syncthreads();
    const float4 s = block_sum2_ff(acc[0], acc[1], acc[2], acc[3], red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
  }
  tc_teardown<TP>(sm, w.fail, err);
}

// ---------------------------------------------------------------- host side
// Registry of the tensor-core row plans: length, radices Q0, Q1, warpgroups
// per CTA.
#define CDX_TC_PLANS(F) \
  F(256, 16, 16, 2)     \
  F(512, 16, 32, 1)     \
  F(756, 27, 28, 2)     \
  F(1024, 32, 32, 1)

#define CDX_TC_DEF(L, A, B, W) using TCP##L = TcPlan<A, B, W>;
CDX_TC_PLANS(CDX_TC_DEF)
#undef CDX_TC_DEF

bool tc_plan_radices(int L, int& q0, int& q1) {
  switch (L) {
#define CDX_TC_CASE(LL, A, B, W) \
  case LL:                       \
    q0 = A;                      \
    q1 = B;                      \
    return true;
    CDX_TC_PLANS(CDX_TC_CASE)
#undef CDX_TC_CASE
    default:
      return false;
  }
}

// Round to the nearest tf32 (11 significant bits), ties away from zero, as
// cvt.rna.tf32.f32 does.
static float host_tf32(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  u = (u + 0x1000u) & 0xffffe000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

// The real 2Q x 2Q form of the forward DFT matrix of radix Q as the B
// operand: row n = 2i + (0 real, 1 imaginary part of output i), column
// k = 2j + (0 real, 1 imaginary part of input j), padded to NP x KP with
// zeros; hi part, then lo part, each in the core-matrix layout.
static void host_dft_operand(int Q, int NP, int KP, std::vector<float>& out) {
  const size_t base = out.size();
  out.resize(base + 2 * (size_t)NP * KP, 0.f);
  const double two_pi = 6.283185307179586476925286766559;
  for (int i = 0; i < Q; ++i)
    for (int j = 0; j < Q; ++j) {
      const double a = two_pi * (double)((long long)i * j % Q) / (double)Q;
      const double c = cos(a), s = sin(a);
      // Re X_i = sum re_j c + im_j s;  Im X_i = sum -re_j s + im_j c
      const double v[2][2] = {{c, s}, {-s, c}};
      for (int ro = 0; ro < 2; ++ro)
        for (int co = 0; co < 2; ++co) {
          const double x = v[ro][co];
          const float hi = host_tf32((float)x);
          const float lo = host_tf32((float)(x - (double)hi));
          const unsigned off = tc::op_offset(2 * i + ro, 2 * j + co, KP) >> 2;
          out[base + off] = hi;
          out[base + (size_t)NP * KP + off] = lo;
        }
    }
}

template <class TP>
static int tc_build_tables(TcTables& t) {
  std::vector<float> b;
  host_dft_operand(TP::Q0, TP::NP0, TP::KP0, b);
  if (TP::Q1 != TP::Q0) host_dft_operand(TP::Q1, TP::NP1, TP::KP1, b);
  if (b.size() * 4 != TP::BEND) {
    set_error("tc_build_tables", "operand table size mismatch");
    return cudaErrorInvalidValue;
  }
  // twiddles W_L^(a*b), a < Q1 (rows, stride Q0+1), b < Q0
  std::vector<float2> tw((size_t)TP::Q1 * TP::TWS, make_float2(0.f, 0.f));
  const double two_pi = 6.283185307179586476925286766559;
  for (int a = 0; a < TP::Q1; ++a)
    for (int c = 0; c < TP::Q0; ++c) {
      const double ang = -two_pi * (double)((long long)a * c % TP::L) / (double)TP::L;
      tw[(size_t)a * TP::TWS + c] = make_float2((float)cos(ang), (float)sin(ang));
    }
  // pad the twiddle table to whole 16-byte groups
  const size_t twb = tc_align((unsigned)(tw.size() * 8), 16);
  CDX_CHECK(cudaMalloc(&t.d_b, b.size() * 4));
  CDX_CHECK(cudaMemcpy(t.d_b, b.data(), b.size() * 4, cudaMemcpyHostToDevice));
  CDX_CHECK(cudaMalloc(&t.d_tw, twb));
  CDX_CHECK(cudaMemset(t.d_tw, 0, twb));
  CDX_CHECK(cudaMemcpy(t.d_tw, tw.data(), tw.size() * 8, cudaMemcpyHostToDevice));
  t.q0 = TP::Q0;
  t.q1 = TP::Q1;
  return 0;
}

int tc_tables_init(TcTables& t, int L) {
  switch (L) {
#define CDX_TC_CASE(LL, A, B, W) \
  case LL:                       \
    return tc_build_tables<TCP##LL>(t);
    CDX_TC_PLANS(CDX_TC_CASE)
#undef CDX_TC_CASE
    default:
      set_error("tc_tables_init", "no tensor-core plan for this length");
      return cudaErrorInvalidValue;
  }
}

void tc_tables_free(TcTables& t) {
  if (t.d_b) cudaFree(t.d_b);
  if (t.d_tw) cudaFree(t.d_tw);
  if (t.d_err) cudaFree(t.d_err);
  t = TcTables{};
}

// Persistent grid: as many CTAs as fit on the device at once (the launch
// bounds' CTAs per SM, or fewer when shared memory holds fewer), at most one
// per group of WG tiles.
static int tc_grid(unsigned smem, int minb, int tiles, int wg, int* grid) {
  int dev = 0, sms = 0, smem_sm = 0;
  CDX_CHECK(cudaGetDevice(&dev));
  CDX_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CDX_CHECK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  int per = smem_sm / (int)(smem + 1024);
  if (per > minb) per = minb;
  if (per < 1) {
    set_error("tc_grid", "tensor-core kernel does not fit an SM");
    return cudaErrorInvalidConfiguration;
  }
  const int want = (tiles + wg - 1) / wg;
  *grid = std::min(want, sms * per);
  if (*grid < 1) *grid = 1;
  return 0;
}

template <class TP>
static int tc_fwd_go(const Geom& g, const TcTables& t, const float* X, float* Xm1, const float* lam,
                     int predict, float2* S, int* err, cudaStream_t st) {
  auto kern = k_xtc_fwd<TP>;
  const size_t smem = TP::BYTES;
  if (int rc = smem_optin(kern, smem)) return rc;
  const int tiles = ceil_div(g.ny, 2 * TP::P) * g.nz;
  int grid = 0;
  if (int rc = tc_grid(TP::BYTES, TP::MINB, tiles, TP::WG, &grid)) return rc;
  CDX_CHECK(launch_pdl(kern, dim3(grid), dim3(128 * TP::WG), smem, st, g,
                       (const float4*)t.d_b, (const float4*)t.d_tw, X, Xm1, lam, predict, S, err));
  CDX_LAUNCH_CHECK("k_xtc_fwd");
  return 0;
}

template <class TP>
static int tc_ratio_go(const Geom& g, const TcTables& t, float2* S, const float* raw, float eps,
                       int* err, cudaStream_t st) {
  auto kern = k_xtc_ratio<TP>;
  const size_t smem = TP::BYTES;
  if (int rc = smem_optin(kern, smem)) return rc;
  const int tiles = ceil_div(g.ny, 2 * TP::P) * g.nz;
  int grid = 0;
  if (int rc = tc_grid(TP::BYTES, TP::MINB, tiles, TP::WG, &grid)) return rc;
  CDX_CHECK(launch_pdl(kern, dim3(grid), dim3(128 * TP::WG), smem, st, g,
                       (const float4*)t.d_b, (const float4*)t.d_tw, S, raw, eps, err));
  CDX_LAUNCH_CHECK("k_xtc_ratio");
  return 0;
}

template <class TP>
static int tc_update_go(const Geom& g, const TcTables& t, const float2* S, const float* Y,
                        float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                        int* err, cudaStream_t st) {
  auto kern = k_xtc_update<TP>;
  const size_t smem = TP::BYTES;
  if (int rc = smem_optin(kern, smem)) return rc;
  const int tiles = ceil_div(g.ny, 2 * TP::P) * g.nz;
  int grid = 0;
  if (int rc = tc_grid(TP::BYTES, TP::MINB, tiles, TP::WG, &grid)) return rc;
  if (dots && grid > w.max_blocks) {
    set_error("launch_x_inv_update", "partials buffer too small");
    return cudaErrorInvalidValue;
  }
  float4* part = reinterpret_cast<float4*>(w.partials);
  CDX_CHECK(launch_pdl(kern, dim3(grid), dim3(128 * TP::WG), smem, st, g,
                       (const float4*)t.d_b, (const float4*)t.d_tw, S, Y, Xout, G, dots, part,
                       err));
  CDX_LAUNCH_CHECK("k_xtc_update");
  if (dots) return launch_lambda(part, grid, lam_next, eps, st);
  return 0;
}

int launch_xtc_fwd(const Geom& g, const TcTables& t, const float* X, float* Xm1, const float* lam,
                   int predict, float2* S, int* err, cudaStream_t st) {
  switch (g.nx) {
#define CDX_TC_CASE(LL, A, B, W) \
  case LL:                       \
    return tc_fwd_go<TCP##LL>(g, t, X, Xm1, lam, predict, S, err, st);
    CDX_TC_PLANS(CDX_TC_CASE)
#undef CDX_TC_CASE
    default:
      set_error("launch_xtc_fwd", "no tensor-core plan for this length");
      return cudaErrorInvalidValue;
  }
}

int launch_xtc_ratio(const Geom& g, const TcTables& t, float2* S, const float* raw, float eps,
                     int* err, cudaStream_t st) {
  switch (g.nx) {
#define CDX_TC_CASE(LL, A, B, W) \
  case LL:                       \
    return tc_ratio_go<TCP##LL>(g, t, S, raw, eps, err, st);
    CDX_TC_PLANS(CDX_TC_CASE)
#undef CDX_TC_CASE
    default:
      set_error("launch_xtc_ratio", "no tensor-core plan for this length");
      return cudaErrorInvalidValue;
  }
}

int launch_xtc_update(const Geom& g, const TcTables& t, const float2* S, const float* Y,
                      float* Xout, float* G, int dots, RLWork& w, float* lam_next, float eps,
                      int* err, cudaStream_t st) {
  switch (g.nx) {
#define CDX_TC_CASE(LL, A, B, W) \
  case LL:                       \
    return tc_update_go<TCP##LL>(g, t, S, Y, Xout, G, dots, w, lam_next, eps, err, st);
    CDX_TC_PLANS(CDX_TC_CASE)
#undef CDX_TC_CASE
    default:
      set_error("launch_xtc_update", "no tensor-core plan for this length");
      return cudaErrorInvalidValue;
  }
}

}  // namespace cdx
