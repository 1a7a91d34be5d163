// SquaredIntensityDifference loss for callers that cannot allocate device memory.
//
// Some hosts of this library must not call cudaMalloc: plug-ins whose device
// memory is owned by a pool allocator of the host application, or real-time loops
// where a device allocation (an implicit synchronisation) is not allowed.
// fo_sid_loss_noalloc
// gives them the metric's loss values without any allocation: the per-block
// partial sums live in a fixed array compiled into this library.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/fluxoptics_gb300.h"
#include "fo_internal.h"

namespace fo {
namespace {

constexpr int kNoAllocBlocks = 1024;    // fixed grid of the partial-sum kernel
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxTargets = 64;  // FO_SID_NOALLOC_MAX_TARGETS

// Partial sums, one slot per (block, target slice): 1024 x 64 floats = 256 KiB.
// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) float g_sid_partials[kNoAllocBlocks * kNoAllocMaxTargets];

__device__ float nb_block_sum(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  float r = 0.f;
  if (threadIdx.x < 32) {
    r = (threadIdx.x < kNoAllocThreads / 32) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;
}

// Grid-stride over pixels: for each target slice t, I_t = sum over fields b with
// tidx[b] == t of |u_b|^2, and each block writes sum (I_t - target_t)^2 over its
// pixels to partials[block * T + t].  Every used slot is written before it is read.
__global__ void sid_noalloc_partials(const float2* u, const float* target, const int* tidx, int batch, int T,
                                     long long npix, float* partials) {
  __shared__ float red[kNoAllocThreads / 32];
  for (int t = 0; t < T; ++t) {
    float acc = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
      float inten = 0.f;
      for (int b = 0; b < batch; ++b) {
        if (tidx[b] != t) continue;
        const float2 x = u[(long long)b * npix + p];
        inten = fmaf(x.x, x.x, fmaf(x.y, x.y, inten));
      }
      const float r = inten - target[(long long)t * npix + p];
      acc = fmaf(r, r, acc);
    }
    const float s = nb_block_sum(acc, red);
    if (threadIdx.x == 0) partials[blockIdx.x * T + t] = s;
  }
}

// loss[t] = sum over blocks of partials[block * T + t], in block order.
__global__ void sid_noalloc_finalize(const float* partials, int nblocks, int T, float* loss) {
  __shared__ float red[kNoAllocThreads / 32];
  const int t = blockIdx.x;
  float acc = 0.f;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partials[b * T + t];
  const float s = nb_block_sum(acc, red);
  if (threadIdx.x == 0) loss[t] = s;
}

// Device address of g_sid_partials, looked up once per device (the first call on
// that device) and kept for the life of the process: a cudaDeviceReset after it is
// not supported.  In host code the symbol names a host-side stand-in, not device
// memory, so kernels must be given the address returned by cudaGetSymbolAddress.
std::mutex g_mu;
float* g_addr[64] = {nullptr};

int partials_address(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(FO_ERR_UNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_sid_partials);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_sid_partials)");
    g_addr[dev] = static_cast<float*>(ptr);
  }
  *out = g_addr[dev];
  return FO_OK;
}

}  // namespace
}  // namespace fo

using namespace fo;

extern "C" FO_API int fo_sid_loss_noalloc(const void* u, const float* target, const int* target_index,
                                          int n_targets, int nx, int ny, int batch, float* loss,
                                          void* stream) {
  if (!u || !target || !target_index || !loss)
    return fail(FO_ERR_ARG, "u, target, target_index and loss must not be NULL");
  if (nx <= 0 || ny <= 0 || batch <= 0 || n_targets <= 0) return fail(FO_ERR_SHAPE, "sizes must be positive");
  if (n_targets > kNoAllocMaxTargets)
    return fail(FO_ERR_SHAPE, "fo_sid_loss_noalloc supports at most " + std::to_string(kNoAllocMaxTargets) +
                                  " target slices (got " + std::to_string(n_targets) + ")");
  float* partials = nullptr;
  int rc = partials_address(&partials);
  if (rc != FO_OK) return rc;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long long npix = (long long)nx * ny;
  long long blocks = (npix + kNoAllocThreads - 1) / kNoAllocThreads;
  if (blocks > kNoAllocBlocks) blocks = kNoAllocBlocks;
  sid_noalloc_partials<<<(unsigned)blocks, kNoAllocThreads, 0, st>>>(reinterpret_cast<const float2*>(u), target,
                                                                      target_index, batch, n_targets, npix,
                                                                      partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sid_noalloc_partials launch");
  sid_noalloc_finalize<<<n_targets, kNoAllocThreads, 0, st>>>(partials, (int)blocks, n_targets, loss);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sid_noalloc_finalize launch");
  return FO_OK;
}
