// Y tiling and maximum-intensity projections of the reference's CLI
// (linearDecon.cpp:497-566 tiling, 1175-1245 stitching, 1434-1473 MaxIntProj).
#include "kernels.h"

namespace cdx {

// Rows yoff .. yoff+tny-1 of a (nx, ny, nz) raw stack, rows past either end
// repeating the nearest edge row (the CLI's get_crop with boundary
// conditions, linearDecon.cpp:548-556), into a (nx, tny, nz) tile.
__global__ void k_tile_rows(const unsigned short* __restrict__ raw, unsigned short* __restrict__ tile,
                            int nx, int ny, int tny, int yoff) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  const int z = blockIdx.z;
  if (x >= nx) return;
  const int ys = min(max(yoff + y, 0), ny - 1);
  tile[((long long)z * tny + y) * nx + x] = raw[((long long)z * ny + ys) * nx + x];
}

int launch_tile_rows(const unsigned short* raw, unsigned short* tile, int nx, int ny, int nz,
                     int tny, int yoff, cudaStream_t st) {
  dim3 grid(ceil_div(nx, 128), tny, nz);
  k_tile_rows<<<grid, 128, 0, st>>>(raw, tile, nx, ny, tny, yoff);
  CDX_LAUNCH_CHECK("k_tile_rows");
  return 0;
}

// Stitch one deconvolved tile (nx, tny, nz) into the output (nx, ny_out, nz) at
// rows y + yoff, with the CLI's rules: zones of a tile near its ends are left
// to the neighbouring tile, a blend zone mixes linearly (BlendTileOverlap),
// and weight marks output voxels already written (linearDecon.cpp:1186-1237).
__global__ void k_stitch(const float* __restrict__ tile, float* out, unsigned char* weight, int nx,
                         int tny, int nz, int ny_out, int yoff, double overlap, int no_zone,
                         int blend_zone, int first, int last, int blend_on) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  const int z = blockIdx.z;
  if (x >= nx || y + yoff >= ny_out) return;
  float blend = 1;
  if (first && y <= overlap)
    blend = 1;
  else if (last && y >= tny - overlap)
    blend = 1;
  else {
    if (y <= no_zone)
      blend = 0;
    else if (y > no_zone && y <= no_zone + blend_zone)
      blend = (double)(y - no_zone) / blend_zone;
    else if (y >= tny - no_zone)
      blend = 0;
    else
      blend = 1;
  }
  const float v = tile[((long long)z * tny + y) * nx + x];
  const long long o = ((long long)z * ny_out + (y + yoff)) * nx + x;
  if (blend_on) {
    const bool w = weight[o] > 0;
    if (blend > 0 && blend < 1 && w)
      out[o] = (float)__dadd_rn((double)__fmul_rn(v, blend),
                                 __dmul_rn((double)out[o], 1.0 - (double)blend));
    else if (blend > 0 && !w)
      out[o] = v;
    else if (blend == 1)
      out[o] = v;
    if (blend > 0) weight[o] = 1;
  } else {
    const bool past_front = (y >= floor((float)overlap / 2.0) || first);
    const bool before_end = (y < floor(tny - (float)overlap / 2.0) || last);
    if (past_front && before_end) out[o] = v;
  }
}

int launch_stitch(const float* tile, float* out, unsigned char* weight, int nx, int tny, int nz,
                  int ny_out, int yoff, double overlap, int no_zone, int blend_zone, bool first,
                  bool last, bool blend, cudaStream_t st) {
  dim3 grid(ceil_div(nx, 128), tny, nz);
  k_stitch<<<grid, 128, 0, st>>>(tile, out, weight, nx, tny, nz, ny_out, yoff, overlap, no_zone,
                                 blend_zone, first ? 1 : 0, last ? 1 : 0, blend ? 1 : 0);
  CDX_LAUNCH_CHECK("k_stitch");
  return 0;
}

// MaxIntProj (linearDecon.cpp:1434-1473): maximum along axis 0 (x), 1 (y) or
// 2 (z), starting from -1e10; outputs (ny, nz), (nx, nz), (nx, ny) images,
// first size fastest.
__global__ void k_mip(const float* __restrict__ in, int nx, int ny, int nz, int axis,
                      float* __restrict__ out) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;  // fastest output index
  const int b = blockIdx.y;
  float m = -1e10f;
  if (axis == 0) {
    if (a >= ny) return;
    const float* p = in + ((long long)b * ny + a) * nx;
    for (int x = 0; x < nx; ++x)
      if (p[x] > m) m = p[x];
    out[(long long)b * ny + a] = m;
  } else if (axis == 1) {
    if (a >= nx) return;
    const float* p = in + (long long)b * ny * nx + a;
    for (int y = 0; y < ny; ++y)
      if (p[(long long)y * nx] > m) m = p[(long long)y * nx];
    out[(long long)b * nx + a] = m;
  } else {
    if (a >= nx) return;
    const float* p = in + (long long)b * nx + a;
    for (int z = 0; z < nz; ++z)
      if (p[(long long)z * ny * nx] > m) m = p[(long long)z * ny * nx];
    out[(long long)b * nx + a] = m;
  }
}

int launch_mip(const float* in, int nx, int ny, int nz, int axis, float* out, cudaStream_t st) {
  if (axis < 0 || axis > 2) {
    set_error("mip", "axis must be 0, 1 or 2");
    return cudaErrorInvalidValue;
  }
  const int fast = axis == 0 ? ny : nx;
  const int slow = axis == 2 ? ny : nz;
  dim3 grid(ceil_div(fast, 128), slow);
  k_mip<<<grid, 128, 0, st>>>(in, nx, ny, nz, axis, out);
  CDX_LAUNCH_CHECK("k_mip");
  return 0;
}

}  // namespace cdx
