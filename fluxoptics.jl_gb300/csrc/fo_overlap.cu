// Overlap metrics at the output plane: DotProduct and PowerCoupling
// (metrics/dot_product.jl:47-100, metrics/power_coupling.jl:48-66).
//
//   DotProduct, mode selective : c_b = dx dy sum_p u_b[p] conj(v_b[p])
//   DotProduct, full matrix    : c[i + j n] = dx dy sum_p conj(v_i[p]) u_j[p]
//   PowerCoupling              : |c|^2 against unit-power copies of v (made once)
// and their pull-backs du_b = v_b g_b, du_j = sum_i v_i G[i + j n], with g = dc
// (DotProduct) or 2 dc c (PowerCoupling, c from the last forward call).
//
// Reductions are deterministic: fixed-size block partials summed in a fixed order
// in FP64.  The matrix form stages 32-pixel tiles of every field of u and v in
// shared memory and keeps up to 16 (i, j) accumulators per thread.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/fluxoptics_gb300.h"
#include "fo_internal.h"

namespace fo {
namespace {

constexpr int OV_THREADS = 256;
constexpr int OV_BLOCKS = 304;  // partial sums per field (two per SM)
constexpr int OV_TILE = 32;     // pixels per shared-memory tile of the matrix form
constexpr int OV_MAX_N = 64;    // fields of the matrix form

__device__ __forceinline__ float2 ov_cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

template <typename T>
__device__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// partials[f * OV_BLOCKS + blk] = sum over this block's pixels of u_f conj(v_f)
__global__ void __launch_bounds__(OV_THREADS) ov_sel_partial_kernel(const float2* u, const float2* v,
                                                                   long long npix, float2* partials) {
  __shared__ float red[2][OV_THREADS / 32];
  const int f = blockIdx.y;
  const float2* uf = u + (long long)f * npix;
  const float2* vf = v + (long long)f * npix;
  float re = 0.f, im = 0.f;
  for (long long p = blockIdx.x * (long long)OV_THREADS + threadIdx.x; p < npix; p += (long long)OV_BLOCKS * OV_THREADS) {
    const float2 a = uf[p], b = vf[p];
    re = fmaf(a.x, b.x, fmaf(a.y, b.y, re));  // Re(a conj(b))
    im = fmaf(a.y, b.x, fmaf(-a.x, b.y, im));  // Im(a conj(b))
  }
  re = warp_sum(re);
  im = warp_sum(im);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = re;
    red[1][threadIdx.x >> 5] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float sr = 0.f, si = 0.f;
    for (int w = 0; w < OV_THREADS / 32; ++w) {
      sr += red[0][w];
      si += red[1][w];
    }
    partials[(long long)f * OV_BLOCKS + blockIdx.x] = make_float2(sr, si);
  }
}

// Matrix form: partials[blk * n^2 + i + j n] = sum over the block's pixels of conj(v_i) u_j.
__global__ void __launch_bounds__(OV_THREADS) ov_mat_partial_kernel(const float2* u, const float2* v,
                                                                   long long npix, int n, float2* partials) {
  __shared__ float2 su[OV_MAX_N][OV_TILE];
  __shared__ float2 sv[OV_MAX_N][OV_TILE];
  const int pairs = n * n;
  constexpr int PER = (OV_MAX_N * OV_MAX_N) / OV_THREADS;  // 16 accumulators per thread
  float2 acc[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) acc[k] = make_float2(0.f, 0.f);
  const long long tiles = (npix + OV_TILE - 1) / OV_TILE;
  for (long long tl = blockIdx.x; tl < tiles; tl += gridDim.x) {
    const long long p0 = tl * OV_TILE;
    __syncthreads();
    for (int e = threadIdx.x; e < n * OV_TILE; e += OV_THREADS) {
      const int f = e / OV_TILE, q = e % OV_TILE;
      const long long p = p0 + q;
      const bool ok = p < npix;
      su[f][q] = ok ? u[(long long)f * npix + p] : make_float2(0.f, 0.f);
      sv[f][q] = ok ? v[(long long)f * npix + p] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int pr = threadIdx.x + k * OV_THREADS;
      if (pr < pairs) {
        const int i = pr % n, j = pr / n;
        float re = acc[k].x, im = acc[k].y;
#pragma unroll 8
        for (int q = 0; q < OV_TILE; ++q) {
          const float2 b = sv[i][q], a = su[j][q];  // conj(b) a
          re = fmaf(b.x, a.x, fmaf(b.y, a.y, re));
          im = fmaf(b.x, a.y, fmaf(-b.y, a.x, im));
        }
        acc[k] = make_float2(re, im);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int pr = threadIdx.x + k * OV_THREADS;
    if (pr < pairs) partials[(long long)blockIdx.x * pairs + pr] = acc[k];
  }
}

// c[k] = scale * sum_blk partials[k, blk] (stride: element k of block blk at
// blk * bstride + k * kstride), in FP64 and block order; PowerCoupling also
// returns |c|^2 and keeps c for the pull-back.
__global__ void ov_finalize_kernel(const float2* partials, int nblk, int count, long long kstride,
                                   long long bstride, double scale, int power, float2* c_dot, void* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double re = 0.0, im = 0.0;
  for (int b = 0; b < nblk; ++b) {
    const float2 x = partials[(long long)b * bstride + (long long)k * kstride];
    re += x.x;
    im += x.y;
  }
  const float2 c = make_float2((float)(re * scale), (float)(im * scale));
  c_dot[k] = c;
  if (power)
    reinterpret_cast<float*>(out)[k] = (float)((re * scale) * (re * scale) + (im * scale) * (im * scale));
  else
    reinterpret_cast<float2*>(out)[k] = c;
}

// g[k] = dc[k] (DotProduct, complex) or 2 dc[k] c_dot[k] (PowerCoupling, real dc)
__global__ void ov_grad_coef_kernel(const void* dc, const float2* c_dot, int count, int power, float2* g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  if (power) {
    const float d = 2.f * reinterpret_cast<const float*>(dc)[k];
    g[k] = make_float2(d * c_dot[k].x, d * c_dot[k].y);
  } else {
    g[k] = reinterpret_cast<const float2*>(dc)[k];
  }
}

__global__ void ov_sel_backward_kernel(const float2* v, const float2* g, long long npix, int batch, float2* du) {
  const long long n = npix * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    du[q] = ov_cmul(v[q], g[q / npix]);
}

// du_j[p] = sum_i v_i[p] G[i + j n]; each thread one pixel, outputs in groups of 8
__global__ void __launch_bounds__(OV_THREADS) ov_mat_backward_kernel(const float2* v, const float2* G,
                                                                    long long npix, int n, float2* du) {
  __shared__ float2 sg[OV_MAX_N * OV_MAX_N];
  for (int e = threadIdx.x; e < n * n; e += OV_THREADS) sg[e] = G[e];
  __syncthreads();
  for (long long p = blockIdx.x * (long long)OV_THREADS + threadIdx.x; p < npix;
       p += (long long)gridDim.x * OV_THREADS) {
    for (int j0 = 0; j0 < n; j0 += 8) {
      float2 acc[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = make_float2(0.f, 0.f);
      for (int i = 0; i < n; ++i) {
        const float2 vi = v[(long long)i * npix + p];
#pragma unroll
        for (int t = 0; t < 8; ++t)
          if (j0 + t < n) {
            const float2 gg = sg[i + (j0 + t) * n];
            acc[t] = make_float2(fmaf(vi.x, gg.x, fmaf(-vi.y, gg.y, acc[t].x)),
                                 fmaf(vi.x, gg.y, fmaf(vi.y, gg.x, acc[t].y)));
          }
      }
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (j0 + t < n) du[(long long)(j0 + t) * npix + p] = acc[t];
    }
  }
}

// unit-power copy: vh_b = v_b / sqrt(dx dy sum |v_b|^2), one block per field (fixed order)
__global__ void __launch_bounds__(OV_THREADS) ov_normalize_kernel(const float2* v, long long npix, double area,
                                                                 float2* vh) {
  __shared__ double red[OV_THREADS / 32];
  const int f = blockIdx.x;
  const float2* vf = v + (long long)f * npix;
  double s = 0.0;
  for (long long p = threadIdx.x; p < npix; p += OV_THREADS) s += (double)vf[p].x * vf[p].x + (double)vf[p].y * vf[p].y;
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  __shared__ float inv;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < OV_THREADS / 32; ++w) t += red[w];
    inv = t > 0.0 ? (float)(1.0 / sqrt(t * area)) : 0.f;
  }
  __syncthreads();
  for (long long p = threadIdx.x; p < npix; p += OV_THREADS)
    vh[(long long)f * npix + p] = make_float2(vf[p].x * inv, vf[p].y * inv);
}

}  // namespace
}  // namespace fo

using namespace fo;

struct fo_overlap_s {
  int nx = 0, ny = 0, batch = 0;
  double area = 1.0;
  int selective = 1, power = 0;
  const float2* v = nullptr;  // reference fields (borrowed, or the owned unit-power copy)
  float2* vh = nullptr;       // owned unit-power copy (PowerCoupling)
  float2* partials = nullptr;
  float2* c_dot = nullptr;  // dot products of the last forward call
  float2* g = nullptr;      // pull-back coefficients
};

FO_API int fo_overlap_create(fo_overlap* ov, int nx, int ny, int batch, double dx, double dy, const void* v,
                             int mode_selective, int power) {
  if (!ov || !v) return fail(FO_ERR_ARG, "ov and v must not be NULL");
  *ov = nullptr;
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  if (!(dx > 0) || !(dy > 0)) return fail(FO_ERR_ARG, "dx and dy must be positive");
  if (!mode_selective && batch > OV_MAX_N)
    return fail(FO_ERR_SHAPE, "the overlap matrix form supports at most 64 fields");
  auto* o = new fo_overlap_s();
  o->nx = nx;
  o->ny = ny;
  o->batch = batch;
  o->area = dx * dy;
  o->selective = mode_selective ? 1 : 0;
  o->power = power ? 1 : 0;
  const long long npix = (long long)nx * ny;
  const int count = o->selective ? batch : batch * batch;
  const size_t nparts = o->selective ? (size_t)batch * OV_BLOCKS : (size_t)OV_BLOCKS * count;
  cudaError_t e = cudaMalloc(&o->partials, sizeof(float2) * nparts);
  if (e == cudaSuccess) e = cudaMalloc(&o->c_dot, sizeof(float2) * count);
  if (e == cudaSuccess) e = cudaMalloc(&o->g, sizeof(float2) * count);
  if (e == cudaSuccess && o->power) e = cudaMalloc(&o->vh, sizeof(float2) * npix * batch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fo_overlap_destroy(o);
    return fail(FO_ERR_ALLOC, "cudaMalloc failed for the overlap metric");
  }
  if (o->power) {
    ov_normalize_kernel<<<batch, OV_THREADS>>>(reinterpret_cast<const float2*>(v), npix, o->area, o->vh);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      fo_overlap_destroy(o);
      return cuda_fail(e, "normalising the PowerCoupling targets");
    }
    o->v = o->vh;
  } else {
    o->v = reinterpret_cast<const float2*>(v);
  }
  *ov = o;
  return FO_OK;
}

FO_API int fo_overlap_forward(fo_overlap ov, const void* u, void* c, void* stream) {
  if (!ov || !u || !c) return fail(FO_ERR_ARG, "ov, u and c must not be NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long long npix = (long long)ov->nx * ov->ny;
  const float2* uu = reinterpret_cast<const float2*>(u);
  if (ov->selective) {
    ov_sel_partial_kernel<<<dim3(OV_BLOCKS, ov->batch), OV_THREADS, 0, st>>>(uu, ov->v, npix, ov->partials);
    FO_CUDA_CHECK(cudaGetLastError());
    ov_finalize_kernel<<<(ov->batch + 127) / 128, 128, 0, st>>>(ov->partials, OV_BLOCKS, ov->batch, OV_BLOCKS, 1,
                                                               ov->area, ov->power, ov->c_dot, c);
  } else {
    const int n = ov->batch, pairs = n * n;
    ov_mat_partial_kernel<<<OV_BLOCKS, OV_THREADS, 0, st>>>(uu, ov->v, npix, n, ov->partials);
    FO_CUDA_CHECK(cudaGetLastError());
    ov_finalize_kernel<<<(pairs + 127) / 128, 128, 0, st>>>(ov->partials, OV_BLOCKS, pairs, 1, pairs, ov->area,
                                                            ov->power, ov->c_dot, c);
  }
  FO_CUDA_CHECK(cudaGetLastError());
  return FO_OK;
}

FO_API int fo_overlap_backward(fo_overlap ov, const void* dc, void* du, void* stream) {
  if (!ov || !dc || !du) return fail(FO_ERR_ARG, "ov, dc and du must not be NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long long npix = (long long)ov->nx * ov->ny;
  const int count = ov->selective ? ov->batch : ov->batch * ov->batch;
  ov_grad_coef_kernel<<<(count + 127) / 128, 128, 0, st>>>(dc, ov->c_dot, count, ov->power, ov->g);
  FO_CUDA_CHECK(cudaGetLastError());
  float2* d = reinterpret_cast<float2*>(du);
  if (ov->selective) {
    const long long n = npix * ov->batch;
    const unsigned grid = (unsigned)std::min<long long>((n + OV_THREADS - 1) / OV_THREADS, 152LL * 16);
    ov_sel_backward_kernel<<<grid, OV_THREADS, 0, st>>>(ov->v, ov->g, npix, ov->batch, d);
  } else {
    const unsigned grid = (unsigned)std::min<long long>((npix + OV_THREADS - 1) / OV_THREADS, 152LL * 8);
    ov_mat_backward_kernel<<<grid, OV_THREADS, 0, st>>>(ov->v, ov->g, npix, ov->batch, d);
  }
  FO_CUDA_CHECK(cudaGetLastError());
  return FO_OK;
}

FO_API int fo_overlap_destroy(fo_overlap ov) {
  if (!ov) return FO_OK;
  cudaFree(ov->partials);
  cudaFree(ov->c_dot);
  cudaFree(ov->g);
  cudaFree(ov->vh);
  delete ov;
  return FO_OK;
}
