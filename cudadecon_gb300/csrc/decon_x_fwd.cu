// Forward x pass of the RL iteration (prediction prologue + R2C along x) and
// the plain inverse x pass used by the convolution test hook.
#include "decon_common.cuh"

namespace cdx {

// ---------------------------------------------------------------- x forward
template <class Run>
__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_fwd(Geom g, FftDev fx, const float* __restrict__ X, const float* __restrict__ Xm1,
        const float* __restrict__ lamp, int predict, float2* __restrict__ S, int P) {
  extern __shared__ float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  load_twiddles(fx, stw);
  __syncthreads();
  const RowPairLoad ld{X, Xm1, predict ? __ldg(lamp) : 0.f, predict, (long long)z * g.ny * nx,
                       y0, g.ny, nx};
  Run::template run<false>(fx, P, 1.f, false, stw, io, ld, io);
  store_half_spectra(g, io, P, z, y0, S);
}

template <class Run>
static int x_fwd_go(const Geom& g, const FftDev& f, const float* X, const float* Xm1,
                    const float* lam, int predict, float2* S, int P, int T, cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  size_t smem = fft_smem(g.nx, (long long)P * g.nx);
  if (int rc = smem_optin(k_x_fwd<Run>, smem)) return rc;
  k_x_fwd<Run><<<grid, T, smem, st>>>(g, f, X, Xm1, lam, predict, S, P);
  CDX_LAUNCH_CHECK("k_x_fwd");
  return 0;
}

int launch_x_fwd(const Geom& g, const FftLen& fx, const float* X, const float* Xm1,
                 const float* lam, int predict, float2* S, cudaStream_t st) {
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP)                                                                      \
  case L:                                                                                    \
    return x_fwd_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, X, Xm1, lam, predict, S, PP, \
                                                    splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  const int P = x_pairs(g.nx);
  return x_fwd_go<GenericRunner>(g, fx.dev, X, Xm1, lam, predict, S, P,
                                 threads_for((long long)P * g.nx), st);
}


template <class Run>
__global__ void __launch_bounds__(kMaxThreads, 1)
k_x_inv_plain(Geom g, FftDev fx, const float2* __restrict__ S, float* __restrict__ out, int P) {
  extern __shared__ float2 smem[];
  const int nx = g.nx;
  float2* stw = smem;
  const SmemIO io{smem + nx, 1, nx};
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * P;
  load_twiddles(fx, stw);
  load_packed_spectra(g, S, io, P, z, y0);
  __syncthreads();
  const PlainRowStore ps{out, (long long)z * g.ny * nx, y0, g.ny, nx};
  Run::template run<true>(fx, P, 1.f, false, stw, io, io, ps);
}

template <class Run>
static int x_plain_go(const Geom& g, const FftDev& f, const float2* S, float* out, int P, int T,
                      cudaStream_t st) {
  dim3 grid(ceil_div(g.ny, 2 * P), g.nz);
  size_t smem = fft_smem(g.nx, (long long)P * g.nx);
  if (int rc = smem_optin(k_x_inv_plain<Run>, smem)) return rc;
  k_x_inv_plain<Run><<<grid, T, smem, st>>>(g, f, S, out, P);
  CDX_LAUNCH_CHECK("k_x_inv_plain");
  return 0;
}

int launch_x_inv_plain(const Geom& g, const FftLen& fx, const float2* S, float* out,
                       cudaStream_t st) {
  if (fx.has_static) switch (g.nx) {
#define CDX_CASE(L, PP) \
  case L:               \
    return x_plain_go<StaticRunner<SP##L, PP, false>>(g, fx.sdev, S, out, PP, splan_threads<SP##L, PP>(), st);
      CDX_X_PLANS(CDX_CASE)
#undef CDX_CASE
      default:
        break;
    }
  const int P = x_pairs(g.nx);
  return x_plain_go<GenericRunner>(g, fx.dev, S, out, P, threads_for((long long)P * g.nx), st);
}

}  // namespace cdx
