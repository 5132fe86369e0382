// z pass: forward FFT along z, OTF multiply (interpolated on the fly),
// inverse FFT along z.
#include "decon_common.cuh"

namespace cdx {

// ---------------------------------------------------------------- z pass
// Columns (consecutive y) per z tile: 16 (128-byte runs) while the tile fits
// kMaxThreads * kEpt elements, fewer for long z.
static int z_cols(int nz) {
  int w = (kMaxThreads * kEpt) / nz;
  if (w > 16) w = 16;
  if (w < 1) w = 1;
  return w;
}

// Last forward stage of the static z pass: multiply element e (= kz) of the
// thread's column by the OTF (conjugated when CONJ), interpolated from the
// kz-resampled radial table at the column's radius (MODE 0: pair e of the
// column at tz[e * nr + ir], radius computed once per thread) or read from
// the precomputed 3D array (MODE 1: full[e * nyp]).
template <class IO, int MODE, bool CONJ>
struct OtfColMulStore {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  IO io;
  const float4* lo4;  // MODE 0: table column ir
  const float2* lo2;  // MODE 1: the column of the 3D array
  float ar;
  int valid, stride;
  __device__ __forceinline__ void st(int v, int e, float2 x) const {
    float2 o = make_float2(0.f, 0.f);
    if constexpr (MODE == 1) {
      o = __ldg(lo2 + e * stride);
    } else if (valid) {
      o = otf_lerp(__ldg(lo4 + e * stride), ar);
    }
    io.st(v, e, CONJ ? cmulconj(x, o) : cmul(x, o));
  }
};

// Runtime-width interleaved tile of W columns: element e of column v at
// sm[e * W + v] (the staged input of the generic z pass).
struct ColIOr {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  float2* sm;
  int W;
  __device__ __forceinline__ float2 ld(int v, int e) const { return sm[e * W + v]; }
};

// Last forward stage of the generic z pass: multiply element e (= kz) of
// column v by the OTF, interpolated from the kz-resampled radial table at the
// column's precomputed radius (mode 0: table column cir[v], fraction car[v];
// -1 outside the table) or read from the 3D array (mode 1), conjugated when
// conj; same arithmetic as OtfColMulStore.
struct OtfColMulStoreG {
  static constexpr bool kSmem = true;
  static constexpr bool kGroup = false;
  SmemIO io;
  const float4* tz;
  const float2* full;  // mode 1: the plane's column y0
  const int* cir;
  const float* car;
  int nr, nyp, ncols, mode, conj;
  __device__ __forceinline__ void st(int v, int e, float2 x) const {
    float2 o = make_float2(0.f, 0.f);
    if (mode == 1) {
      if (v < ncols) o = __ldg(full + (long long)e * nyp + v);
    } else {
      const int ir = cir[v];
      if (ir >= 0) o = otf_lerp(__ldg(tz + (long long)e * nr + ir), car[v]);
    }
    io.st(v, e, conj ? cmulconj(x, o) : cmul(x, o));
  }
};

// MODE and CONJ: the OTF mode and the conjugation as compile-time constants
// (static plans), or -1 to read them from otf.mode and conj (generic engine).
template <class Run, int MODE, int CONJ>
__global__ void __launch_bounds__(Run::kThreads, Run::template min_blocks<8>())
k_z_pass(Geom g, FftDev fz, float2* __restrict__ S, OtfDev otf, int conj, int fwd_only, int Wa) {
  const int W = tile_vectors<Run>(Wa);
  extern __shared__ __align__(16) float2 smem[];
  const int nz = g.nz;
  const int kx = blockIdx.y;
  const int y0 = blockIdx.x * W;
  float2* stw = smem;
  const float invW = 1.f / (float)W;
  const SpecColIO gio{S + (long long)kx * g.plane, y0, g.ny, g.nyp};
  if constexpr (Run::kStatic) {
    // The tile (W columns of nz elements, interleaved) is copied with
    // cp.async: one contiguous run of W complex values per z.
    const auto io = Run::col_tile(smem + (nz + (nz & 1)), W);
    constexpr int kChunks = Run::kV / 2;  // 16-byte chunks per z row
    const float2* src = S + (long long)kx * g.plane + y0;
    load_twiddles(fz, stw);
    grid_dep_wait();
    grid_dep_launch();
    for (int idx = threadIdx.x; idx < nz * kChunks; idx += blockDim.x) {
      const int z = idx / kChunks;
      const int c = idx - z * kChunks;
      if (y0 + 2 * c < g.ny) cp_async16(io.sm + z * W + 2 * c, src + (long long)z * g.nyp + 2 * c);
    }
    cp_async_commit();
    // the OTF of this thread's column (the column is fixed across stages)
    const int v = threadIdx.x % Run::kV;
    const int y = y0 + v;
    const float4* lo4 = otf.tz;
    const float2* lo2 = otf.full;
    float ar = 0.f;
    int valid = 0;
    if (MODE == 1) {
      lo2 = otf.full + (long long)kx * g.plane + (y < g.ny ? y : 0);
    } else if (y < g.ny) {
      int ir = 0;
      if (otf_radius(otf, kx, y, g.ny, ir, ar)) {
        lo4 = otf.tz + ir;
        valid = 1;
      }
    }
    cp_async_wait_all();
    __syncthreads();
    if (fwd_only) {
      Run::template run<false>(fz, W, invW, true, stw, io, io, gio);
      return;
    }
    const OtfColMulStore<decltype(io), MODE, CONJ == 1> ost{io, lo4, lo2, ar, valid,
                                                            MODE == 1 ? g.nyp : otf.nr};
    Run::template run<false>(fz, W, invW, true, stw, io, io, ost);
    Run::template run<true>(fz, W, invW, true, stw, io, io, gio);
  } else {
    // Generic engine: the tile (W columns of nz elements) is copied with
    // cp.async into an unpadded interleaved stage at the start of the padded
    // transform tile; the first stage reads it before its barrier, so the
    // two may alias.  The OTF radius is computed once per column.
    const int zoff = nz + (nz & 1);
    const SmemIO io{smem + zoff, W, 1};
    int* cir = reinterpret_cast<int*>(smem + zoff + spad_size(W * nz));
    float* car = reinterpret_cast<float*>(cir + W);
    const float2* src = S + (long long)kx * g.plane + y0;
    load_twiddles(fz, stw);
    for (int v = threadIdx.x; v < W; v += blockDim.x) {
      const int y = y0 + v;
      int ir = -1;
      float ar = 0.f;
      if (y < g.ny && otf.mode == 0) {
        int i = 0;
        if (otf_radius(otf, kx, y, g.ny, i, ar)) ir = i;
      }
      cir[v] = ir;
      car[v] = ar;
    }
    grid_dep_wait();
    grid_dep_launch();
    if ((W & 1) == 0) {
      // column pairs: 16-byte copies (y0 and the row pitch are even)
      const int half = W >> 1;
      for (int idx = threadIdx.x; idx < nz * half; idx += blockDim.x) {
        int z, c;
        divmod_small<0>(idx, half, 1.f / (float)half, z, c);
        if (y0 + 2 * c < g.ny)
          cp_async16(io.sm + z * W + 2 * c, src + (long long)z * g.nyp + 2 * c);
      }
    } else {
      for (int idx = threadIdx.x; idx < nz * W; idx += blockDim.x) {
        int z, c;
        divmod_small<0>(idx, W, invW, z, c);
        if (y0 + c < g.ny) cp_async8(io.sm + z * W + c, src + (long long)z * g.nyp + c);
      }
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    const ColIOr stg{io.sm, W};
    if (fwd_only) {
      Run::template run<false>(fz, W, invW, true, stw, io, stg, gio);
      return;
    }
    const float2* full = otf.mode == 1 ? otf.full + (long long)kx * g.plane + y0 : nullptr;
    const OtfColMulStoreG ost{io, otf.tz, full, cir, car, otf.nr, g.nyp, g.ny - y0, otf.mode,
                              conj};
    Run::template run<false>(fz, W, invW, true, stw, io, stg, ost);
    Run::template run<true>(fz, W, invW, true, stw, io, io, gio);
  }
}

template <class Run, int MODE, int CONJ>
static int z_go(const Geom& g, const FftDev& f, float2* S, const OtfDev& otf, bool conj,
                bool fwd_only, int W, int T, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, W), g.nxh);
  // static: twiddles + unpadded tile; generic: twiddles + padded tile +
  // per-column OTF radius (index and fraction)
  size_t smem = Run::kStatic
                    ? sizeof(float2) * ((size_t)(g.nz + (g.nz & 1)) + (size_t)W * g.nz)
                    : sizeof(float2) * ((size_t)(g.nz + (g.nz & 1)) + spad_size(W * g.nz) + W);
  auto kern = k_z_pass<Run, MODE, CONJ>;
  if (int rc = smem_optin(kern, smem)) return rc;
  CDX_CHECK(launch_pdl(kern, grid, dim3(T), smem, st, g, f, S, otf, conj ? 1 : 0,
                       fwd_only ? 1 : 0, W));
  CDX_LAUNCH_CHECK("k_z_pass");
  return 0;
}

// Static plans: one instantiation per OTF mode and conjugation.
template <class Run>
static int z_go_static(const Geom& g, const FftDev& f, float2* S, const OtfDev& otf, bool conj,
                       bool fwd_only, int W, int T, cudaStream_t st) {
  if (otf.mode == 1)
    return conj ? z_go<Run, 1, 1>(g, f, S, otf, conj, fwd_only, W, T, st)
                : z_go<Run, 1, 0>(g, f, S, otf, conj, fwd_only, W, T, st);
  return conj ? z_go<Run, 0, 1>(g, f, S, otf, conj, fwd_only, W, T, st)
              : z_go<Run, 0, 0>(g, f, S, otf, conj, fwd_only, W, T, st);
}

int launch_z_pass(const Geom& g, const FftLen& fz, float2* S, const OtfDev& otf, bool conj,
                  cudaStream_t st, bool fwd_only) {
  if (fz.has_static) switch (g.nz) {
#define CDX_CASE(L, WW)                                                                    \
  case L:                                                                                  \
    return z_go_static<StaticRunner<SP##L, WW, true>>(g, fz.sdev, S, otf, conj, fwd_only, WW, \
                                                       splan_threads<SP##L, WW>(), st);
      CDX_Z_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  if (fz.has_gz && otf.mode == 0) switch (g.nz) {
#define CDX_GCASE(L, WW, RR)                                                                  \
  case L:                                                                                     \
    return conj ? z_go<StaticRunner<SPZ##L, WW, true, false, RR>, 0, 1>(                      \
                      g, fz.gzdev, S, otf, conj, fwd_only, WW, splan_threads<SPZ##L, WW>(), st) \
                : z_go<StaticRunner<SPZ##L, WW, true, false, RR>, 0, 0>(                      \
                      g, fz.gzdev, S, otf, conj, fwd_only, WW, splan_threads<SPZ##L, WW>(), st);
      CDX_Z_GEN_PLANS(CDX_GCASE)
#undef CDX_GCASE
      default:
        break;
    }
  const int W = z_cols(g.nz);
  return z_go<GenericRunner, -1, -1>(g, fz.dev, S, otf, conj, fwd_only, W,
                                     threads_for((long long)W * g.nz), st);
}

}  // namespace cdx
