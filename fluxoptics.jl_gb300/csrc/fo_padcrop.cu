// Padding and cropping of a batch of fields (PadCropOperator, pad, crop).
//
// pad: every px x py field of dst is pad_val except the nx x ny block at column ox, row
// oy, which is the field of src (utilities/pad_crop_operators.jl:1-16, pad! with offset
// and pad_val).  crop: every nx x ny field of dst is the block at (ox, oy) of the
// px x py field of src (pad_crop_operators.jl:61-79, crop!).  One thread per output
// element over a grid-stride loop: writes are coalesced along x, and so are the reads
// of each output row.
#include <cuda_runtime.h>

#include <string>

#include "../../include/fluxoptics_gb300.h"
#include "fo_internal.h"

namespace fo {
namespace {

constexpr int kPcThreads = 256;

unsigned pc_grid(long long n) {
  long long g = (n + kPcThreads - 1) / kPcThreads;
  if (g > 152LL * 16) g = 152LL * 16;
  return (unsigned)(g < 1 ? 1 : g);
}

__global__ void pad_kernel(const float2* __restrict__ src, int nx, int ny, float2* __restrict__ dst, int px, int py,
                           int batch, int ox, int oy, float2 fill) {
  const long long plane = (long long)px * py, n = plane * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const long long b = q / plane;
    const long long r = q - b * plane;
    const int y = (int)(r / px) - oy, x = (int)(r % px) - ox;
    dst[q] = (x >= 0 && x < nx && y >= 0 && y < ny) ? src[(b * ny + y) * nx + x] : fill;
  }
}

__global__ void crop_kernel(const float2* __restrict__ src, int px, int py, float2* __restrict__ dst, int nx, int ny,
                            int batch, int ox, int oy) {
  const long long plane = (long long)nx * ny, n = plane * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const long long b = q / plane;
    const long long r = q - b * plane;
    const int y = (int)(r / nx), x = (int)(r % nx);
    dst[q] = src[(b * py + y + oy) * (long long)px + x + ox];
  }
}

int check_pc(const void* src, const void* dst, int nx, int ny, int px, int py, int batch, int ox, int oy) {
  if (!src || !dst) return fail(FO_ERR_ARG, "src and dst must not be NULL");
  if (src == dst) return fail(FO_ERR_ARG, "src and dst must be different buffers");
  if (nx <= 0 || ny <= 0 || px <= 0 || py <= 0 || batch <= 0)
    return fail(FO_ERR_SHAPE, "grid sizes and batch must be positive");
  if (ox < 0 || oy < 0) return fail(FO_ERR_ARG, "offsets must be non-negative");
  if (ox + nx > px || oy + ny > py)
    return fail(FO_ERR_SHAPE, "the " + std::to_string(nx) + " x " + std::to_string(ny) + " block at (" +
                                  std::to_string(ox) + ", " + std::to_string(oy) + ") does not fit in " +
                                  std::to_string(px) + " x " + std::to_string(py));
  return FO_OK;
}

}  // namespace
}  // namespace fo

using namespace fo;

extern "C" {

FO_API int fo_pad(const void* src, int nx, int ny, void* dst, int px, int py, int batch, int ox, int oy,
                  double pad_re, double pad_im, void* stream) {
  const int rc = check_pc(src, dst, nx, ny, px, py, batch, ox, oy);
  if (rc != FO_OK) return rc;
  const long long n = (long long)px * py * batch;
  pad_kernel<<<pc_grid(n), kPcThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(src), nx, ny, reinterpret_cast<float2*>(dst), px, py, batch, ox, oy,
      make_float2((float)pad_re, (float)pad_im));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "pad_kernel launch");
}

FO_API int fo_crop(const void* src, int px, int py, void* dst, int nx, int ny, int batch, int ox, int oy,
                   void* stream) {
  const int rc = check_pc(src, dst, nx, ny, px, py, batch, ox, oy);
  if (rc != FO_OK) return rc;
  const long long n = (long long)nx * ny * batch;
  crop_kernel<<<pc_grid(n), kPcThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(src), px, py, reinterpret_cast<float2*>(dst), nx, ny, batch, ox, oy);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "crop_kernel launch");
}

}  // extern "C"
