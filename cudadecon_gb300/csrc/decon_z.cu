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
    const SmemIO io{smem + nz, W, 1};
    float2* otf_tile = smem + nz + spad_size(W * nz);
    load_twiddles(fz, stw);
    grid_dep_wait();
    grid_dep_launch();
    if (fwd_only) {
      __syncthreads();
      Run::template run<false>(fz, W, invW, true, stw, io, gio, gio);
      return;
    }
    // OTF of every (y, z) of the tile, interpolated on the fly from the
    // kz-resampled radial table (dev_otfinterpolate RA branch,
    // RLgpuImpl.cu:238-273: kr = sqrt(kx^2 + ky^2), zero at kr >= nr-1) or
    // read from the precomputed 3D array
    for (int idx = threadIdx.x; idx < W * nz; idx += blockDim.x) {
      int w, z;
      divmod_small<Run::kV>(idx, W, invW, z, w);
      const int y = y0 + w;
      float2 o = make_float2(0.f, 0.f);
      if (y < g.ny) {
        if (otf.mode == 1) {
          o = __ldg(otf.full + (long long)kx * g.plane + (long long)z * g.nyp + y);
        } else {
          int ir = 0;
          float ar = 0.f;
          if (otf_radius(otf, kx, y, g.ny, ir, ar))
            o = otf_lerp(__ldg(otf.tz + (long long)z * otf.nr + ir), ar);
        }
      }
      otf_tile[idx] = o;
    }
    __syncthreads();
    const OtfMulStore ost{io, otf_tile, W, conj};
    Run::template run<false>(fz, W, invW, true, stw, io, gio, ost);
    Run::template run<true>(fz, W, invW, true, stw, io, io, gio);
  }
}

template <class Run, int MODE, int CONJ>
static int z_go(const Geom& g, const FftDev& f, float2* S, const OtfDev& otf, bool conj,
                bool fwd_only, int W, int T, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, W), g.nxh);
  // static: twiddles + unpadded tile; generic: twiddles + padded tile + OTF tile
  size_t smem = Run::kStatic
                    ? sizeof(float2) * ((size_t)(g.nz + (g.nz & 1)) + (size_t)W * g.nz)
                    : fft_smem(g.nz, (long long)W * g.nz, (long long)W * g.nz);
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
  const int W = z_cols(g.nz);
  return z_go<GenericRunner, -1, -1>(g, fz.dev, S, otf, conj, fwd_only, W,
                                     threads_for((long long)W * g.nz), st);
}

}  // namespace cdx
