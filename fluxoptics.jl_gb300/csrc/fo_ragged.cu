// Ragged batch: independent problems Phase(phi) -> ASProp(z) -> SquaredIntensityDifference
// on square grids of different sizes, forward pass, loss, adjoint and phase gradient of
// all of them in ONE persistent cooperative launch.
//
// The launch holds one 512-thread CTA per SM (all CTAs co-resident) and runs five
// passes separated by grid barriers; inside a pass the CTAs take work chunks from a
// shared counter, the largest grids first, so problems of every size share the SMs:
//   1 row    : v = u_in * cis(s*phi); FFT along x             -> u_out (scratch)
//   2 column : FFT along y, * H, IFFT along y                  (in place in u_out)
//   3 row    : IFFT along x -> u_out (the propagated field);
//              r = |u|^2 - t, loss partials sum r^2; du = 4 r u; FFT along x -> adj
//   4 column : FFT along y, * conj(H), IFFT along y            (in place in adj)
//   5 row    : IFFT along x -> dv; du = dv * cis(-s*phi);
//              dphi = s * Im(du * conj(u_in))                  -> grad
// and a final fixed-order sum of the loss partials of every problem.  Row chunks are
// 4096 elements (4096/n rows) taken by each 256-thread half of the CTA on its own
// (named barriers), column chunks are 8192 elements (a strip of 8192/n columns) taken
// by the whole CTA; strips and transfer functions move by one 4-D TMA instruction
// each, the next strip is fetched while the current one is transformed, and results
// leave by TMA tensor stores.  Every wait (mbarrier, grid barrier) is bounded by
// %globaltimer; on expiry the CTA sets a bit of the device error word and returns.
//
// Reference semantics per problem: Phase propagate!/backpropagate_with_gradient!
// (src/optical_components/modulators/phasemask.jl:90-150), ASProp
// (freespace_propagators/angular_spectrum.jl:1-12,193-234), SquaredIntensityDifference
// (metrics/squared_intensity_difference.jl:58-90), chained by the rrules of
// src/ChainRulesCoreExt.jl:21-111 under Zygote.withgradient.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fluxoptics_gb300.h"
#include "fo_aux.h"
#include "fo_fft.cuh"
#include "fo_internal.h"
#include "fo_passes.cuh"

namespace fo {
namespace {

constexpr int RG_THREADS = 512;
constexpr int RG_E = 16;
constexpr int RG_CHUNK = RG_THREADS * RG_E;    // column chunk: 8192 elements
constexpr int RG_HALF = RG_THREADS / 2;        // row passes: two independent halves
constexpr int RG_HCHUNK = RG_HALF * RG_E;      // row chunk: 4096 elements
constexpr int RG_HSLOTS = RG_HCHUNK + RG_HCHUNK / 16;  // padded exchange slots of one half
constexpr int RG_XSLOTS = RG_CHUNK + RG_CHUNK / 16;    // padded exchange slots of a strip
constexpr int RG_LG_MIN = 8, RG_LG_MAX = 12;           // n = 256 .. 4096
// dynamic shared memory: the column layout (strip, H strip, padded exchange) or the
// row layout (two padded exchange regions, then 4096 float2 + 4096 float of side
// inputs per half), whichever is larger
constexpr size_t RG_SMEM_COL = sizeof(float2) * ((size_t)2 * RG_CHUNK + RG_XSLOTS);
constexpr size_t RG_SMEM_ROW = sizeof(float2) * ((size_t)2 * RG_HSLOTS + 2 * (RG_HCHUNK + RG_HCHUNK / 2));
constexpr size_t RG_SMEM = 128 + (RG_SMEM_COL > RG_SMEM_ROW ? RG_SMEM_COL : RG_SMEM_ROW);

enum RgRowKind { RG_ROW_FWD = 0, RG_ROW_MID = 1, RG_ROW_GRAD = 2 };

struct RgProblem {  // aligned as CUtensorMap (64 bytes or more)
  CUtensorMap tm_fwd;  // 4-D view of u_out: strips of 8192/n columns
  CUtensorMap tm_adj;  // 4-D view of the adjoint scratch
  CUtensorMap tm_h;    // 4-D view of H
  const float2* u_in;
  const float* phase;
  const float* target;
  float2* u_out;
  float2* adj;
  float* grad;
  float* loss;
  int lg;         // n = 1 << lg
  int row_part0;  // index of this problem's first row chunk in `partials`
  int n_row;      // row chunks of this problem (n^2 / 4096)
  float s;        // direction sign of the phase (+1: Forward)
};

struct RgArgs {
  const RgProblem* probs;
  int count;
  const int2* row_items;  // (problem, chunk) in processing order
  int n_row_items;
  const int2* col_items;
  int n_col_items;
  const float2* tw[RG_LG_MAX - RG_LG_MIN + 1];  // E = 16 twiddle tables per size
  float* partials;
  unsigned* ctl;  // [0..4] chunk counters of the passes, [5] barrier arrivals, [6] barrier generation
  unsigned* err_word;
  unsigned long long wait_ns;
  unsigned long long* stamps;  // [6]: %globaltimer at the start and after every pass (CTA 0)
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;\n" ::: "memory");
}
// The tensor maps live in global memory (written by the host before the launch):
// acquire them for the tensor-map proxy before the copy that uses them.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap* m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(m) : "memory");
}
__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(n) : "memory");
}

// Grid-wide barrier of the co-resident CTAs: arrival counter + generation word, the
// wait bounded by wait_ns (bit 1 of the error word on expiry).  Returns false when the
// CTA must stop.
__device__ bool grid_sync(const RgArgs& a, int* s_flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned* count = a.ctl + 5;
    unsigned* gen = a.ctl + 6;
    const unsigned g = ld_acquire_u32(gen);
    fence_proxy_async_global();  // this CTA's completed TMA stores -> other CTAs' reads
    __threadfence();
    if (atomicAdd(count, 1u) == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else if (ld_acquire_u32(gen) == g) {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_u32(gen) == g) {
        if (global_ns() - t0 > a.wait_ns) {
          atomicOr(a.err_word, 2u);
          ok = 0;
          break;
        }
        __nanosleep(128);
      }
    }
    __threadfence();
    fence_proxy_async_global();  // generic writes before the barrier -> TMA reads after it
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

// 16-byte cp.async copies of `bytes` contiguous bytes (a multiple of 16) by the 256
// threads of a half.
__device__ __forceinline__ void half_copy16(void* dst, const void* src, int bytes, int ht) {
  char* d = reinterpret_cast<char*>(dst);
  const char* s = reinterpret_cast<const char*>(src);
  for (int o = ht * 16; o < bytes; o += RG_HALF * 16) cp_async16(d + o, s + o);
}

// One row chunk of problem P: 4096/N rows, T = N/16 threads per row, 256 threads.
// `side` (4096 float2 + 4096 float of this half) stages the inputs that are used
// after the transform, copied while it runs.
template <int N, int KIND>
__device__ __forceinline__ void row_chunk(const RgProblem& P, int chunk, int ht, float2* sm, int bar_id,
                                          const float2* __restrict__ tw, float* partials, float* red,
                                          float2* side) {
  constexpr int T = N / RG_E;
  constexpr int LANES = RG_HCHUNK / N;
  constexpr int SLOTS = SmemSize<N>::value;
  const int lane = ht / T;
  const int t = ht % T;
  const long long row = (long long)(chunk * LANES + lane) * N;
  float2* lsm = sm + lane * SLOTS;
  // the problem's pointers in registers (stores through them could alias the table)
  const float2* __restrict__ u_in = P.u_in;
  const float* __restrict__ phase = P.phase;
  float2* __restrict__ u_out = P.u_out;
  float2* __restrict__ adj = P.adj;
  const float s = P.s;
  const long long row0 = (long long)chunk * RG_HCHUNK;  // first element of the chunk
  float2* side_c = side;                                  // complex side input, chunk order
  float* side_r = reinterpret_cast<float*>(side + RG_HCHUNK);  // real side input
  const int loc = lane * N;                               // this lane's row inside the chunk
  float2 v[RG_E];
  if constexpr (KIND == RG_ROW_FWD) {
    float ph[RG_E];
#pragma unroll
    for (int i = 0; i < RG_E; ++i) {
      const int p = t + i * T;
      v[i] = u_in[row + p];
      ph[i] = phase[row + p];
    }
#pragma unroll
    for (int i = 0; i < RG_E; ++i) v[i] = cmul(v[i], cis_f(s * ph[i]));
    fft_forward<N, RG_E, 1>(v, t, tw, lsm, bar_id, RG_HALF);
#pragma unroll
    for (int i = 0; i < RG_E; ++i) u_out[row + t + i * T] = v[i];
  } else {
    const float2* src = (KIND == RG_ROW_MID) ? u_out : adj;
#pragma unroll
    for (int i = 0; i < RG_E; ++i) v[i] = cconj(src[row + t + i * T]);
    // side inputs of the chunk, copied while the inverse transform runs
    if constexpr (KIND == RG_ROW_MID) {
      half_copy16(side_r, P.target + row0, RG_HCHUNK * 4, ht);
    } else {
      half_copy16(side_c, u_in + row0, RG_HCHUNK * 8, ht);
      half_copy16(side_r, phase + row0, RG_HCHUNK * 4, ht);
    }
    cp_async_commit();
    fft_forward<N, RG_E, 1>(v, t, tw, lsm, bar_id, RG_HALF);
    cp_async_wait<0>();
    named_sync(bar_id, RG_HALF);
    if constexpr (KIND == RG_ROW_MID) {
      float part = 0.f;
#pragma unroll
      for (int i = 0; i < RG_E; ++i) {
        const int p = t + i * T;
        const float2 u = cconj(v[i]);
        u_out[row + p] = u;
        const float r = fmaf(u.x, u.x, u.y * u.y) - side_r[loc + p];
        part = fmaf(r, r, part);
        v[i] = cscale(u, 4.f * r);  // seed of the adjoint: 4 (I - t) u
      }
      // half-CTA sum in a fixed order: warp shuffles, then warp 0 of the half
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      if ((ht & 31) == 0) red[ht >> 5] = part;
      fft_forward<N, RG_E, 1>(v, t, tw, lsm, bar_id, RG_HALF);  // its barriers order red[] too
      if (ht == 0) {
        float acc = 0.f;
#pragma unroll
        for (int w = 0; w < RG_HALF / 32; ++w) acc += red[w];
        partials[P.row_part0 + chunk] = acc;
      }
#pragma unroll
      for (int i = 0; i < RG_E; ++i) adj[row + t + i * T] = v[i];
    } else {
      float* __restrict__ grad = P.grad;
#pragma unroll
      for (int i = 0; i < RG_E; ++i) {
        const int p = t + i * T;
        const float2 dv = cconj(v[i]);
        const float2 du = cmul(dv, cis_f(-s * side_r[loc + p]));
        const float2 us = side_c[loc + p];
        grad[row + p] = s * (du.y * us.x - du.x * us.y);  // s * Im(du * conj(u_in))
      }
    }
  }
}

template <int KIND>
__device__ void row_pass(const RgArgs& a, float2* smem, unsigned* counter, int* s_next, float* s_red) {
  const int half = threadIdx.x / RG_HALF;
  const int ht = threadIdx.x % RG_HALF;
  const int bar_id = 1 + half;
  float2* sm = smem + half * RG_HSLOTS;
  float* red = s_red + half * (RG_HALF / 32);
  // side inputs: 4096 float2 + 4096 float per half, after both exchange regions
  float2* side = smem + 2 * RG_HSLOTS + half * (RG_HCHUNK + RG_HCHUNK / 2);
  for (;;) {
    if (ht == 0) s_next[half] = (int)atomicAdd(counter, 1u);
    named_sync(bar_id, RG_HALF);
    const int k = s_next[half];
    named_sync(bar_id, RG_HALF);
    if (k >= a.n_row_items) break;
    const int2 it = a.row_items[k];
    const RgProblem& P = a.probs[it.x];
    switch (P.lg) {
      case 8: row_chunk<256, KIND>(P, it.y, ht, sm, bar_id, a.tw[0], a.partials, red, side); break;
      case 9: row_chunk<512, KIND>(P, it.y, ht, sm, bar_id, a.tw[1], a.partials, red, side); break;
      case 10: row_chunk<1024, KIND>(P, it.y, ht, sm, bar_id, a.tw[2], a.partials, red, side); break;
      case 11: row_chunk<2048, KIND>(P, it.y, ht, sm, bar_id, a.tw[3], a.partials, red, side); break;
      default: row_chunk<4096, KIND>(P, it.y, ht, sm, bar_id, a.tw[4], a.partials, red, side); break;
    }
  }
}

struct RgColState {
  unsigned long long* bar;  // [0] strip, [1] H
  unsigned ph0, ph1;        // parities expected next
  int* s_next;
  int* s_abort;
};

__device__ __forceinline__ void col_issue(const RgArgs& a, int k, bool adj, bool with_h, float2* stage, float2* hs,
                                          unsigned long long* bar) {
  const int2 it = a.col_items[k];
  const RgProblem* P = a.probs + it.x;
  const int W = RG_CHUNK >> P->lg;
  const int col0 = it.y * W;
  const CUtensorMap* m = adj ? &P->tm_adj : &P->tm_fwd;
  tmap_acquire(m);
  mbar_expect_tx(&bar[0], (unsigned)(RG_CHUNK * sizeof(float2)));
  tma_load_4d(stage, m, col0, 0, 0, 0, &bar[0]);
  if (with_h) {
    tmap_acquire(&P->tm_h);
    mbar_expect_tx(&bar[1], (unsigned)(RG_CHUNK * sizeof(float2)));
    tma_load_4d(hs, &P->tm_h, col0, 0, 0, 0, &bar[1]);
  }
}

// One column strip: W = 8192/N columns, T = N/16 threads per column.  Returns false
// when a bounded wait gave up (the whole CTA then stops).
template <int N>
__device__ __forceinline__ bool col_chunk(const RgArgs& a, const RgProblem& P, int chunk, int next, bool adj,
                                          float2* stage, float2* hs, float2* ex, RgColState& st) {
  constexpr int T = N / RG_E;
  constexpr int W = RG_CHUNK / N;
  const float2* __restrict__ tw = a.tw[ilog2c(N) - RG_LG_MIN];
  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  bool ok = mbar_wait_bounded(&st.bar[0], st.ph0, a.wait_ns);
  st.ph0 ^= 1u;
  if (!ok) *st.s_abort = 1;
  float2 v[RG_E];
#pragma unroll
  for (int i = 0; i < RG_E; ++i) v[i] = stage[(t + i * T) * W + c];
  if (threadIdx.x == 0) bulk_wait_read_all();  // the previous strip has left `ex`
  __syncthreads();                             // `stage` is free; abort decision is uniform
  if (*st.s_abort) return false;
  if (threadIdx.x == 0 && next < a.n_col_items) {
    fence_proxy_async();
    col_issue(a, next, adj, false, stage, hs, st.bar);
  }
  fft_forward<N, RG_E, W>(v, t, tw, ex + c);
  ok = mbar_wait_bounded(&st.bar[1], st.ph1, a.wait_ns);
  st.ph1 ^= 1u;
  if (!ok) *st.s_abort = 1;
  const float hsign = adj ? -1.f : 1.f;
#pragma unroll
  for (int i = 0; i < RG_E; ++i) {
    float2 hv = hs[(t + i * T) * W + c];
    hv.y *= hsign;
    // conj(X * H): the inverse transform runs as conj(FFT(conj(.)))
    v[i] = make_float2(fmaf(v[i].x, hv.x, -v[i].y * hv.y), -fmaf(v[i].x, hv.y, v[i].y * hv.x));
  }
  __syncthreads();  // `hs` is free
  if (*st.s_abort) return false;
  if (threadIdx.x == 0 && next < a.n_col_items) {
    const int2 it = a.col_items[next];
    const RgProblem* Pn = a.probs + it.x;
    const int Wn = RG_CHUNK >> Pn->lg;
    fence_proxy_async();
    tmap_acquire(&Pn->tm_h);
    mbar_expect_tx(&st.bar[1], (unsigned)(RG_CHUNK * sizeof(float2)));
    tma_load_4d(hs, &Pn->tm_h, it.y * Wn, 0, 0, 0, &st.bar[1]);
  }
  fft_forward<N, RG_E, W>(v, t, tw, ex + c);
  __syncthreads();  // the last stage has read `ex`
#pragma unroll
  for (int i = 0; i < RG_E; ++i) ex[(t + i * T) * W + c] = cconj(v[i]);
  fence_proxy_async();
  __syncthreads();
  if (threadIdx.x == 0) {
    const CUtensorMap* m = adj ? &P.tm_adj : &P.tm_fwd;
    tmap_acquire(m);
    tma_store_4d(m, chunk * W, 0, 0, 0, ex);
    bulk_commit();
  }
  return true;
}

__device__ bool col_pass(const RgArgs& a, float2* smem, unsigned* counter, bool adj, RgColState& st) {
  float2* stage = smem;
  float2* hs = stage + RG_CHUNK;
  float2* ex = hs + RG_CHUNK;
  if (threadIdx.x == 0) st.s_next[0] = (int)atomicAdd(counter, 1u);
  __syncthreads();
  int k = st.s_next[0];
  if (threadIdx.x == 0 && k < a.n_col_items) col_issue(a, k, adj, true, stage, hs, st.bar);
  bool ok = true;
  while (k < a.n_col_items) {
    if (threadIdx.x == 0) st.s_next[1] = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int next = st.s_next[1];
    const int2 it = a.col_items[k];
    const RgProblem& P = a.probs[it.x];
    switch (P.lg) {
      case 8: ok = col_chunk<256>(a, P, it.y, next, adj, stage, hs, ex, st); break;
      case 9: ok = col_chunk<512>(a, P, it.y, next, adj, stage, hs, ex, st); break;
      case 10: ok = col_chunk<1024>(a, P, it.y, next, adj, stage, hs, ex, st); break;
      case 11: ok = col_chunk<2048>(a, P, it.y, next, adj, stage, hs, ex, st); break;
      default: ok = col_chunk<4096>(a, P, it.y, next, adj, stage, hs, ex, st); break;
    }
    if (!ok) break;
    k = next;
  }
  if (threadIdx.x == 0) {
    if (!ok) {
      atomicOr(a.err_word, 1u);
      // copies of the next strip may still be in flight: let them land (bounded)
      mbar_wait_bounded(&st.bar[0], st.ph0, a.wait_ns);
      mbar_wait_bounded(&st.bar[1], st.ph1, a.wait_ns);
    }
    bulk_wait_all();  // the strips are in global memory before the grid barrier
  }
  return ok;
}

__global__ void __launch_bounds__(RG_THREADS, 1) ragged_kernel(const RgArgs a) {
  extern __shared__ float4 dsm4[];
  // 128-byte aligned, by pointer arithmetic on the shared array (keeps shared-memory accesses)
  float2* smem = reinterpret_cast<float2*>(reinterpret_cast<char*>(dsm4) + ((128u - (smem_u32(dsm4) & 127u)) & 127u));
  __shared__ unsigned long long bar[2];
  __shared__ int s_next[2], s_abort, s_flag;
  __shared__ float s_red[RG_THREADS / 32];
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    fence_proxy_async();
  }
  __syncthreads();
  RgColState st{bar, 0u, 0u, s_next, &s_abort};
  auto stamp = [&](int i) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.stamps[i] = global_ns();
  };

  stamp(0);
  row_pass<RG_ROW_FWD>(a, smem, a.ctl + 0, s_next, s_red);
  if (!grid_sync(a, &s_flag)) return;
  stamp(1);
  if (!col_pass(a, smem, a.ctl + 1, false, st)) return;
  if (!grid_sync(a, &s_flag)) return;
  stamp(2);
  row_pass<RG_ROW_MID>(a, smem, a.ctl + 2, s_next, s_red);
  if (!grid_sync(a, &s_flag)) return;
  stamp(3);
  if (!col_pass(a, smem, a.ctl + 3, true, st)) return;
  if (!grid_sync(a, &s_flag)) return;
  stamp(4);
  row_pass<RG_ROW_GRAD>(a, smem, a.ctl + 4, s_next, s_red);

  // loss of each problem: fixed-order sum of its row-chunk partials (written in pass 3,
  // complete since the third barrier)
  __shared__ double s_dred[RG_THREADS / 32];
  for (int p = blockIdx.x; p < a.count; p += gridDim.x) {
    const RgProblem& P = a.probs[p];
    double acc = 0.0;
    for (int k = threadIdx.x; k < P.n_row; k += RG_THREADS) acc += (double)a.partials[P.row_part0 + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_dred[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < RG_THREADS / 32; ++w) tot += s_dred[w];
      *P.loss = (float)tot;
    }
    __syncthreads();
  }
  stamp(5);
}

}  // namespace
}  // namespace fo

using namespace fo;

struct fo_ragged_s {
  int device = 0;
  int count = 0;
  int grid = 0;
  RgProblem* d_probs = nullptr;
  int2* d_items = nullptr;  // row items, then column items
  float* d_partials = nullptr;
  unsigned* d_ctl = nullptr;
  unsigned long long* d_stamps = nullptr;
  std::vector<void*> owned;  // H tables and adjoint scratch
  RgArgs args{};
  size_t ws_bytes = 0;
};

namespace {

void ragged_free(fo_ragged_plan p) {
  if (!p) return;
  for (void* q : p->owned) cudaFree(q);
  cudaFree(p->d_probs);
  cudaFree(p->d_items);
  cudaFree(p->d_partials);
  cudaFree(p->d_ctl);
  cudaFree(p->d_stamps);
  delete p;
}

int dev_alloc(void** ptr, size_t bytes, const char* what, size_t* total) {
  if (cudaMalloc(ptr, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(FO_ERR_ALLOC, std::string("cudaMalloc failed for ") + what + " (" + std::to_string(bytes) + " bytes)");
  }
  *total += bytes;
  return FO_OK;
}

}  // namespace

FO_API int fo_ragged_create(fo_ragged_plan* plan, const fo_ragged_problem* problems, int count, int flags) {
  (void)flags;
  if (!plan || !problems || count <= 0) return fail(FO_ERR_ARG, "plan, problems and count > 0 are required");
  *plan = nullptr;
  for (int i = 0; i < count; ++i) {
    const fo_ragged_problem& q = problems[i];
    int lg = 0;
    while ((1 << lg) < q.n) ++lg;
    if ((1 << lg) != q.n || lg < RG_LG_MIN || lg > RG_LG_MAX)
      return fail(FO_ERR_SHAPE, "ragged problem " + std::to_string(i) + ": n must be a power of two from 256 to 4096");
    if (!q.u_in || !q.phase || !q.target || !q.u_out || !q.grad_phase || !q.loss)
      return fail(FO_ERR_ARG, "ragged problem " + std::to_string(i) + ": every pointer is required");
    if (q.u_in == q.u_out)
      return fail(FO_ERR_ARG, "ragged problem " + std::to_string(i) + ": u_in must not alias u_out (it is the saved input)");
    if (!(q.lambda > 0.0) || !(q.dx > 0.0) || !(q.dy > 0.0))
      return fail(FO_ERR_ARG, "ragged problem " + std::to_string(i) + ": lambda, dx, dy must be positive");
  }
  auto* p = new fo_ragged_s();
  cudaGetDevice(&p->device);
  p->count = count;
  int rc = FO_OK;
  auto bail = [&](int code) {
    ragged_free(p);
    return code;
  };

  // occupancy: the cooperative launch needs every CTA resident
  if (cudaFuncSetAttribute(ragged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RG_SMEM) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(FO_ERR_UNSUPPORTED, "the ragged kernel's shared memory does not fit on this device"));
  }
  int per_sm = 0, sms = 0, coop = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ragged_kernel, RG_THREADS, RG_SMEM);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, p->device);
  if (per_sm < 1 || sms < 1 || !coop) return bail(fail(FO_ERR_UNSUPPORTED, "cooperative ragged launch not possible"));
  p->grid = per_sm * sms;

  std::vector<RgProblem> hp(count);
  std::vector<int> order(count);
  int n_row = 0, n_col = 0;
  for (int i = 0; i < count; ++i) {
    const fo_ragged_problem& q = problems[i];
    RgProblem& P = hp[i];
    std::memset(&P, 0, sizeof(P));
    int lg = 0;
    while ((1 << lg) < q.n) ++lg;
    const int n = q.n;
    const size_t n2 = (size_t)n * n;
    P.lg = lg;
    P.s = 1.f;
    P.u_in = reinterpret_cast<const float2*>(q.u_in);
    P.phase = q.phase;
    P.target = q.target;
    P.u_out = reinterpret_cast<float2*>(q.u_out);
    P.grad = q.grad_phase;
    P.loss = q.loss;
    P.row_part0 = n_row;
    P.n_row = (int)(n2 / RG_HCHUNK);
    n_row += P.n_row;
    n_col += (int)(n2 / RG_CHUNK);
    void* H = nullptr;
    void* adj = nullptr;
    if ((rc = dev_alloc(&H, n2 * sizeof(float2), "a ragged transfer function", &p->ws_bytes)) != FO_OK) return bail(rc);
    p->owned.push_back(H);
    if ((rc = dev_alloc(&adj, n2 * sizeof(float2), "a ragged adjoint buffer", &p->ws_bytes)) != FO_OK) return bail(rc);
    p->owned.push_back(adj);
    P.adj = reinterpret_cast<float2*>(adj);
    cudaError_t e = launch_as_h(reinterpret_cast<float2*>(H), n, n, q.dx, q.dy, q.lambda, q.n0 > 0.0 ? q.n0 : 1.0, q.z,
                                1.0 / ((double)n * (double)n), 0);
    if (e != cudaSuccess) return bail(cuda_fail(e, "transfer function of a ragged problem"));
    const int W = RG_CHUNK / n;
    if ((rc = encode_tmap_4d(&P.tm_fwd, q.u_out, 1, n, n, n, W)) != FO_OK) return bail(rc);
    if ((rc = encode_tmap_4d(&P.tm_adj, adj, 1, n, n, n, W)) != FO_OK) return bail(rc);
    if ((rc = encode_tmap_4d(&P.tm_h, H, 1, n, n, n, W)) != FO_OK) return bail(rc);
    order[i] = i;
  }
  // chunk lists, largest grids first (they take longest; small ones fill the tail)
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hp[x].lg > hp[y].lg; });
  std::vector<int2> items;
  items.reserve((size_t)n_row + n_col);
  for (int i : order)
    for (int c = 0; c < hp[i].n_row; ++c) items.push_back(make_int2(i, c));
  for (int i : order)
    for (int c = 0; c < (1 << (2 * hp[i].lg)) / RG_CHUNK; ++c) items.push_back(make_int2(i, c));

  int trc = FO_OK;
  for (int lg = RG_LG_MIN; lg <= RG_LG_MAX; ++lg) {
    p->args.tw[lg - RG_LG_MIN] = twiddles(1 << lg, RG_E, &trc);
    if (!p->args.tw[lg - RG_LG_MIN]) return bail(trc);
  }
  if ((rc = dev_alloc(reinterpret_cast<void**>(&p->d_probs), sizeof(RgProblem) * count, "ragged problems",
                      &p->ws_bytes)) != FO_OK)
    return bail(rc);
  if ((rc = dev_alloc(reinterpret_cast<void**>(&p->d_items), sizeof(int2) * items.size(), "ragged work lists",
                      &p->ws_bytes)) != FO_OK)
    return bail(rc);
  if ((rc = dev_alloc(reinterpret_cast<void**>(&p->d_partials), sizeof(float) * n_row, "ragged loss partials",
                      &p->ws_bytes)) != FO_OK)
    return bail(rc);
  if ((rc = dev_alloc(reinterpret_cast<void**>(&p->d_ctl), sizeof(unsigned) * 8, "ragged counters", &p->ws_bytes)) !=
      FO_OK)
    return bail(rc);
  if ((rc = dev_alloc(reinterpret_cast<void**>(&p->d_stamps), sizeof(unsigned long long) * 8, "ragged stamps",
                      &p->ws_bytes)) != FO_OK)
    return bail(rc);
  cudaError_t e = cudaMemcpy(p->d_probs, hp.data(), sizeof(RgProblem) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->d_ctl, 0, sizeof(unsigned) * 8);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return bail(cuda_fail(e, "uploading the ragged plan"));

  p->args.probs = p->d_probs;
  p->args.count = count;
  p->args.row_items = p->d_items;
  p->args.n_row_items = n_row;
  p->args.col_items = p->d_items + n_row;
  p->args.n_col_items = n_col;
  p->args.partials = p->d_partials;
  p->args.ctl = p->d_ctl;
  p->args.stamps = p->d_stamps;
  p->args.err_word = device_error_word(&rc);
  if (!p->args.err_word) return bail(rc);
  const char* w = getenv("FO_WAIT_NS");
  p->args.wait_ns = w ? strtoull(w, nullptr, 10) : 1000000000ull;
  *plan = p;
  return FO_OK;
}

FO_API int fo_ragged_batch(fo_ragged_plan plan, void* stream) {
  if (!plan) return fail(FO_ERR_ARG, "plan is NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // chunk counters and the barrier words start from zero on every run
  cudaError_t e = cudaMemsetAsync(plan->d_ctl, 0, sizeof(unsigned) * 8, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync (ragged counters)");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(plan->grid);
  cfg.blockDim = dim3(RG_THREADS);
  cfg.dynamicSmemBytes = RG_SMEM;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, ragged_kernel, plan->args);
  if (e != cudaSuccess) return cuda_fail(e, "cooperative launch of the ragged kernel");
  return FO_OK;
}

FO_API int fo_ragged_info(fo_ragged_plan plan, int* grid_ctas, size_t* workspace_bytes) {
  if (!plan) return fail(FO_ERR_ARG, "plan is NULL");
  if (grid_ctas) *grid_ctas = plan->grid;
  if (workspace_bytes) *workspace_bytes = plan->ws_bytes;
  return FO_OK;
}

FO_API int fo_ragged_pass_ms(fo_ragged_plan plan, double* ms) {
  if (!plan || !ms) return fail(FO_ERR_ARG, "plan and ms are required");
  unsigned long long t[6];
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(t, plan->d_stamps, sizeof(t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the ragged pass stamps");
  for (int i = 0; i < 5; ++i) ms[i] = (double)(t[i + 1] - t[i]) * 1e-6;
  return FO_OK;
}

FO_API int fo_ragged_destroy(fo_ragged_plan plan) {
  ragged_free(plan);
  return FO_OK;
}
