// Affine resampling with hardware trilinear texture filtering.
//
// The reference's transformKernel / transformKernelRA
// (src/geometryTransform.cu:183-253) sample a 3D float texture with linear
// filtering and border (zero) addressing.  The texture unit computes the
// interpolation weights in reduced-precision fixed point, so a software
// trilinear interpolation would not reproduce the reference's values; this
// kernel uses the same texture path and the same coordinate arithmetic.
// The input is staged once into a 3D CUDA array (block-linear layout gives
// the texture cache 3D locality); the matrix is passed by value.
#include "kernels.h"

#include <string.h>

namespace cdx {

struct Mat12 {
  float m[12];
};

__global__ void k_affine(float* __restrict__ output, int nx, int ny, int nz, Mat12 M,
                         cudaTextureObject_t texObj) {
  const unsigned int x = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned int y = blockIdx.y * blockDim.y + threadIdx.y;
  const unsigned int z = blockIdx.z * blockDim.z + threadIdx.z;
  if (x >= (unsigned)nx || y >= (unsigned)ny || z >= (unsigned)nz) return;
  const float* mat = M.m;
  float u = x;
  float v = y;
  float w = z;
  float tu = mat[0] * u + mat[1] * v + mat[2] * w + mat[3] + 0.5f;
  float tv = mat[4] * u + mat[5] * v + mat[6] * w + mat[7] + 0.5f;
  float tw = mat[8] * u + mat[9] * v + mat[10] * w + mat[11] + 0.5f;
  const size_t idx = ((size_t)z * ny + y) * nx + x;
  output[idx] = tex3D<float>(texObj, tu, tv, tw);
}

__global__ void k_affine_ra(float* __restrict__ output, int nx, int ny, int nz, float dx, float dy,
                            float dz, Mat12 M, cudaTextureObject_t texObj) {
  const unsigned int x = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned int y = blockIdx.y * blockDim.y + threadIdx.y;
  const unsigned int z = blockIdx.z * blockDim.z + threadIdx.z;
  if (x >= (unsigned)nx || y >= (unsigned)ny || z >= (unsigned)nz) return;
  const float* mat = M.m;
  float u = x;
  float v = y;
  float w = z;
  // voxel to world coordinates
  u = 0.5 + (u - 0.5) * dx;
  v = 0.5 + (v - 0.5) * dy;
  w = 0.5 + (w - 0.5) * dz;
  float tu = mat[0] * u + mat[1] * v + mat[2] * w + mat[3];
  float tv = mat[4] * u + mat[5] * v + mat[6] * w + mat[7];
  float tw = mat[8] * u + mat[9] * v + mat[10] * w + mat[11];
  // world to voxel coordinates
  tu = 0.5 + (tu - 0.5) / dx;
  tv = 0.5 + (tv - 0.5) / dy;
  tw = 0.5 + (tw - 0.5) / dz;
  const size_t idx = ((size_t)z * ny + y) * nx + x;
  output[idx] = tex3D<float>(texObj, tu, tv, tw);
}

// Host-to-host affine transform; ra selects the world-coordinate variant.
int affine_host(const float* in, int nx, int ny, int nz, const float* mat16, bool ra, float dx,
                float dy, float dz, float* out, cudaStream_t st) {
  cudaArray_t arr = nullptr;
  cudaTextureObject_t tex = 0;
  float* d_out = nullptr;
  int rc = 0;
  cudaChannelFormatDesc cd = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
  cudaExtent ext = make_cudaExtent(nx, ny, nz);
  Mat12 M;
  memcpy(M.m, mat16, sizeof(M.m));
  cudaError_t e = cudaMalloc3DArray(&arr, &cd, ext, cudaArrayDefault);
  if (e == cudaSuccess) {
    cudaMemcpy3DParms prm;
    memset(&prm, 0, sizeof(prm));
    prm.srcPtr = make_cudaPitchedPtr((void*)in, nx * sizeof(float), nx, ny);
    prm.dstArray = arr;
    prm.extent = ext;
    prm.kind = cudaMemcpyHostToDevice;
    e = cudaMemcpy3DAsync(&prm, st);
  }
  if (e == cudaSuccess) {
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    td.readMode = cudaReadModeElementType;
    td.addressMode[0] = cudaAddressModeBorder;
    td.addressMode[1] = cudaAddressModeBorder;
    td.addressMode[2] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.normalizedCoords = 0;
    e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
  }
  const size_t n = (size_t)nx * ny * nz;
  if (e == cudaSuccess) e = cudaMalloc(&d_out, n * sizeof(float));
  if (e == cudaSuccess) {
    dim3 blk(32, 8, 2);
    dim3 grd(ceil_div(nx, blk.x), ceil_div(ny, blk.y), ceil_div(nz, blk.z));
    if (ra)
      k_affine_ra<<<grd, blk, 0, st>>>(d_out, nx, ny, nz, dx, dy, dz, M, tex);
    else
      k_affine<<<grd, blk, 0, st>>>(d_out, nx, ny, nz, M, tex);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, n * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_cuda_error("affine", e);
    rc = e;
  }
  if (tex) cudaDestroyTextureObject(tex);
  if (arr) cudaFreeArray(arr);
  if (d_out) cudaFree(d_out);
  return rc;
}

}  // namespace cdx
