// Pointwise proximal operators IstaProx / PositiveProx, the gradient rules Descent /
// Momentum / Nesterov, and the SquaredFieldDifference metric.
//
// IstaProx(s, c) soft-thresholds every value towards c (ista_prox.jl:1-19, applied
// pointwise by PointwiseProx, pointwise_prox.jl:40-42); for complex parameters the
// reference shrinks the real and imaginary parts separately, each towards c, which is
// the same operation on the float pairs.  PositiveProx sets negative values to zero
// (positive_prox.jl:1-7).  SquaredFieldDifference gives per field b
// c_b = sum |u_b - v_b|^2 and the pull-back du = 2 dc_b (u_b - v_b)
// (metrics/squared_field_difference.jl:35-61).  Its sums are fixed-order: per field,
// every block reduces a fixed slice of the pixels, and one thread adds the block
// partials in FP64 in block order.
#include <cuda_runtime.h>

#include <string>

#include "../../include/fluxoptics_gb300.h"
#include "fo_internal.h"

namespace fo {
namespace {

constexpr int kPmThreads = 256;
constexpr int kSfdBlocks = 64;  // blocks per field of the metric's partial sums

unsigned pm_grid(long long n) {
  long long g = (n + kPmThreads - 1) / kPmThreads;
  if (g > 152LL * 32) g = 152LL * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

__global__ void ista_kernel(float* x, long long n, float s, float c) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = x[q];
    const float xc = v - c;
    x[q] = fabsf(xc) <= s ? c : (xc > s ? v - s : v + s);
  }
}

__global__ void positive_kernel(float* x, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    if (x[q] < 0.f) x[q] = 0.f;
}

// One step of Optimisers.jl's Descent / Momentum / Nesterov (Optimisers.jl 0.4, the
// version the reference pins; re-exported by OptimisersExt.jl:9), x <- x - newdx, in
// FP32 with the rule's operation order and no contraction into FMAs:
//   Descent:  newdx = eta dx
//   Momentum: v = rho v + eta dx;                      newdx = v
//   Nesterov: newdx = (-rho^2) v + ((1 + rho) eta) dx; v = rho v - eta dx
__global__ void rule_kernel(float* x, float* v, const float* dx, long long n, int rule, float eta, float rho) {
  const float a = -__fmul_rn(rho, rho), b = __fmul_rn(__fadd_rn(1.f, rho), eta);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float g = dx[q];
    float nd;
    if (rule == FO_RULE_DESCENT) {
      nd = __fmul_rn(eta, g);
    } else if (rule == FO_RULE_MOMENTUM) {
      nd = __fadd_rn(__fmul_rn(rho, v[q]), __fmul_rn(eta, g));
      v[q] = nd;
    } else {
      const float vq = v[q];
      nd = __fadd_rn(__fmul_rn(a, vq), __fmul_rn(b, g));
      v[q] = __fsub_rn(__fmul_rn(rho, vq), __fmul_rn(eta, g));
    }
    x[q] = __fsub_rn(x[q], nd);
  }
}

// partial[b * kSfdBlocks + blk] = sum over this block's pixels of |u_b - v_b|^2
__global__ void __launch_bounds__(kPmThreads) sfd_partial_kernel(const float2* u, const float2* v, long long npix,
                                                                 double* partial) {
  __shared__ float red[kPmThreads / 32];
  const int b = blockIdx.y;
  const float2* ub = u + (long long)b * npix;
  const float2* vb = v + (long long)b * npix;
  float acc = 0.f;
  for (long long q = blockIdx.x * (long long)kPmThreads + threadIdx.x; q < npix;
       q += (long long)gridDim.x * kPmThreads) {
    const float dx = ub[q].x - vb[q].x, dy = ub[q].y - vb[q].y;
    acc = fmaf(dx, dx, fmaf(dy, dy, acc));
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kPmThreads / 32; ++w) s += red[w];
    partial[(long long)b * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void sfd_finalize_kernel(const double* partial, int nblk, int batch, float* c) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  double s = 0.0;
  for (int k = 0; k < nblk; ++k) s += partial[(long long)b * nblk + k];
  c[b] = (float)s;
}

// du = 2 dc_b (u - v); dc NULL: all ones
__global__ void sfd_backward_kernel(const float2* u, const float2* v, const float* dc, long long npix, int batch,
                                    float2* du) {
  const long long n = npix * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float k = 2.f * (dc ? dc[q / npix] : 1.f);
    du[q] = make_float2(k * (u[q].x - v[q].x), k * (u[q].y - v[q].y));
  }
}

}  // namespace
}  // namespace fo

using namespace fo;


extern "C" {

FO_API int fo_ista(float* x, long long n, double s, double c, void* stream) {
  if (!x) return fail(FO_ERR_ARG, "x must not be NULL");
  if (n <= 0) return fail(FO_ERR_SHAPE, "n must be positive");
  if (!(s >= 0)) return fail(FO_ERR_ARG, "the threshold must be non-negative");
  ista_kernel<<<pm_grid(n), kPmThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(x, n, (float)s, (float)c);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "ista_kernel launch");
}

FO_API int fo_positive(float* x, long long n, void* stream) {
  if (!x) return fail(FO_ERR_ARG, "x must not be NULL");
  if (n <= 0) return fail(FO_ERR_SHAPE, "n must be positive");
  positive_kernel<<<pm_grid(n), kPmThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(x, n);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "positive_kernel launch");
}

FO_API int fo_rule_step(float* x, float* state, const float* dx, long long n, int rule, double eta, double rho,
                        void* stream) {
  if (!x || !dx) return fail(FO_ERR_ARG, "x and dx must not be NULL");
  if (n <= 0) return fail(FO_ERR_SHAPE, "n must be positive");
  if (rule != FO_RULE_DESCENT && rule != FO_RULE_MOMENTUM && rule != FO_RULE_NESTEROV)
    return fail(FO_ERR_ARG, "unknown rule");
  if (rule != FO_RULE_DESCENT && !state) return fail(FO_ERR_ARG, "Momentum and Nesterov need a velocity state");
  rule_kernel<<<pm_grid(n), kPmThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(x, state, dx, n, rule, (float)eta,
                                                                                      (float)rho);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "rule_kernel launch");
}

FO_API int fo_sfd_create(fo_sfd* sfd, int nx, int ny, int batch) {
  if (!sfd) return fail(FO_ERR_ARG, "sfd output pointer is NULL");
  *sfd = nullptr;
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  fo_sfd h = new fo_sfd_s();
  h->nx = nx;
  h->ny = ny;
  h->batch = batch;
  cudaError_t e = cudaMalloc(&h->partial, sizeof(double) * (size_t)batch * kSfdBlocks);
  if (e == cudaSuccess) e = cudaMalloc(&h->rows, sizeof(float) * (size_t)ny * batch);
  if (e != cudaSuccess) {
    cudaFree(h->partial);
    delete h;
    return fail(FO_ERR_ALLOC, "SquaredFieldDifference partials: " + std::string(cudaGetErrorString(e)));
  }
  *sfd = h;
  return FO_OK;
}

FO_API int fo_sfd_destroy(fo_sfd sfd) {
  if (sfd) {
    cudaFree(sfd->partial);
    cudaFree(sfd->rows);
    delete sfd;
  }
  return FO_OK;
}

FO_API int fo_sfd_forward(fo_sfd sfd, const void* u, const void* v, float* c, void* stream) {
  if (!sfd || !u || !v || !c) return fail(FO_ERR_ARG, "sfd, u, v and c must not be NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long long npix = (long long)sfd->nx * sfd->ny;
  sfd_partial_kernel<<<dim3(kSfdBlocks, sfd->batch), kPmThreads, 0, st>>>(
      reinterpret_cast<const float2*>(u), reinterpret_cast<const float2*>(v), npix, sfd->partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sfd_partial_kernel launch");
  sfd_finalize_kernel<<<(sfd->batch + 127) / 128, 128, 0, st>>>(sfd->partial, kSfdBlocks, sfd->batch, c);
  e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "sfd_finalize_kernel launch");
}

FO_API int fo_sfd_backward(fo_sfd sfd, const void* u, const void* v, const float* dc, void* du, void* stream) {
  if (!sfd || !u || !v || !du) return fail(FO_ERR_ARG, "sfd, u, v and du must not be NULL");
  const long long npix = (long long)sfd->nx * sfd->ny;
  sfd_backward_kernel<<<pm_grid(npix * sfd->batch), kPmThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(u), reinterpret_cast<const float2*>(v), dc, npix, sfd->batch,
      reinterpret_cast<float2*>(du));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FO_OK : cuda_fail(e, "sfd_backward_kernel launch");
}

}  // extern "C"
