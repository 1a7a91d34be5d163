// Row and column passes of the fused 2-D propagation pipeline (templates).
//
// A propagation u <- IFFT2(H . FFT2(u)) over a batch of fields is split into
//   row pass    : FFT along x                      (fused with the modulation before it)
//   column pass : FFT along y, * H, IFFT along y    (one read + one write of the field)
//   row pass    : IFFT along x                     (fused with the next modulation and,
//                                                  inside a chain, the next FFT along x)
// so a chain of K propagations costs 2K+1 passes over the field, each reading and
// writing it once.  Zero padding (RSProp) is never materialised: rows are loaded
// with zeros past the valid extent and the column pass never reads the padded
// rows, which are identically zero after the row transform.
//
// Every CTA loops over several fields of the same rows (row pass) or the same
// column tile (column pass).  Per-pixel factors that do not depend on the field
// (the modulation, the transfer function of one wavelength) are loaded once per
// CTA, and with PF the next field is copied into shared memory with cp.async
// while the current one is transformed, so loads overlap the FFT arithmetic.
// The staging buffer of the current field doubles as the FFT exchange buffer.
#pragma once

#include "fo_fft.cuh"
#include "fo_internal.h"

namespace fo {

// Minimum resident CTAs per SM requested from the compiler: caps registers at 64
// per thread for E <= 8 and at 128 for E = 16.
__host__ __device__ constexpr int min_blocks(int threads, int E) {
  return (65536 / (threads * (E <= 8 ? 64 : 128))) > 0 ? 65536 / (threads * (E <= 8 ? 64 : 128)) : 1;
}

__device__ __forceinline__ float2 cis_f(float a) {
  float s, c;
  sincosf(a, &s, &c);
  return make_float2(c, s);
}

__device__ __forceinline__ void cp_async8(float2* dst, const float2* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory");
}

// --------------------------------------------------------------------------
// Row pass.  GK: gradient accumulator (0 none, 1 real: phase / dn, 2 complex: mask).
// PF: stage the next field's row through cp.async (needs load_n == N).
// Shared memory: 2 * LANES * SLOTS float2 (PF) or LANES * SLOTS float2.
// --------------------------------------------------------------------------
template <int N, int E, int LANES, int GK, bool PF>
__global__ void __launch_bounds__(LANES*(N / E), min_blocks(LANES*(N / E), E))
    row_pass_kernel(const RowPassArgs a, const float2* __restrict__ tw) {
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  extern __shared__ float2 dsm[];

  const int t = threadIdx.x % T;
  const int lane = threadIdx.x / T;
  const int y = blockIdx.y * LANES + lane;
  const bool row_ok = y < a.nrows;
  float2* buf0 = dsm + lane * SLOTS;
  float2* buf1 = dsm + (LANES + lane) * SLOTS;

  const int load_n = a.inv_first ? N : a.n_valid;
  const int store_n = a.fwd_after ? N : a.n_valid;
  constexpr int GR = (GK == 1) ? E : 1;
  constexpr int GC = (GK == 2) ? E : 1;
  float gacc[GR];
  float2 gacc_c[GC];
#pragma unroll
  for (int i = 0; i < GR; ++i) gacc[i] = 0.f;
#pragma unroll
  for (int i = 0; i < GC; ++i) gacc_c[i] = make_float2(0.f, 0.f);

  // per-pixel modulation factor, cached across fields while the field factor is unchanged
  float2 wm[E];
  float wm_fb = -1.f;

  const int f0 = blockIdx.x * a.fields_per_cta;
  const int f1 = min(a.batch, f0 + a.fields_per_cta);
  auto field_of = [&](int f) { return a.field_list ? a.field_list[f] : f; };
  auto prefetch = [&](int f, float2* dst) {
    const float2* src = a.src + (long long)field_of(f) * a.src_bstride + (long long)y * a.src_ld;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int p = t + i * T;
      cp_async8(dst + spad(p), src + p);
    }
  };
  if constexpr (PF) {
    if (row_ok && f0 < f1) prefetch(f0, buf0);
    cp_async_commit();
  }

  for (int f = f0; f < f1; ++f) {
    const int b = field_of(f);
    float2* cur = ((f - f0) & 1) ? buf1 : buf0;
    float2 v[E];
    if constexpr (PF) {
      float2* nxt = ((f - f0) & 1) ? buf0 : buf1;
      if (row_ok && f + 1 < f1) prefetch(f + 1, nxt);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        const float2 x = row_ok ? cur[spad(p)] : make_float2(0.f, 0.f);
        v[i] = a.inv_first ? cconj(x) : x;
      }
    } else {
      const float2* src = a.src + (long long)b * a.src_bstride + (long long)y * a.src_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 x = make_float2(0.f, 0.f);
        if (row_ok && p < load_n) x = src[p];
        v[i] = a.inv_first ? cconj(x) : x;
      }
    }
    // loads whose latency the inverse transform can hide
    float2 sv[GK != 0 ? E : 1];
    if constexpr (GK != 0) {
      const float2* svp = a.saved + (long long)b * a.saved_bstride + (long long)y * a.saved_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        sv[i] = (row_ok && p < a.n_valid) ? svp[p] : make_float2(0.f, 0.f);
      }
    }
    const float fb = (a.mod_kind == MOD_DN) ? a.mod_scale * a.inv_lambda[b] : 1.f;
    if (a.mod_kind != MOD_NONE && row_ok && fb != wm_fb) {
      const float s = a.mod_sign;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 w = make_float2(1.f, 0.f);
        if (p < a.n_valid) {
          const long long q = (long long)y * a.param_ld + p;
          if (a.mod_kind == MOD_MASK) {
            w = reinterpret_cast<const float2*>(a.mod_param)[q];
            // forward: m (conj for s < 0); adjoint: conj(m) (m for s < 0)
            if ((s < 0.f) != (a.mod_bwd != 0)) w = cconj(w);
          } else {
            const float ph = reinterpret_cast<const float*>(a.mod_param)[q];
            w = cis_f((a.mod_bwd ? -s : s) * fb * ph);
          }
        }
        wm[i] = w;
      }
      wm_fb = fb;
    }

    if (a.inv_first) {
      fft_forward<N, E, 1>(v, t, tw, PF ? cur : buf0);
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (p < a.n_valid) ? cconj(v[i]) : make_float2(0.f, 0.f);  // crop / re-pad
      }
    }
    // ---- real-space operations at positions p = t + i*T, p < n_valid ----
    if (a.seed && row_ok) {
      const int tt = a.tidx[b];
      const float k4 = 4.f * a.dc[tt];
      const float* rr = a.resid + (long long)tt * a.resid_tstride + (long long)y * a.resid_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < a.n_valid) v[i] = cscale(v[i], k4 * rr[p]);
      }
    }
    if (a.mod_kind != MOD_NONE && row_ok) {
      if (!a.mod_bwd) {
        if (a.save) {
          float2* svw = a.save + (long long)b * a.save_bstride + (long long)y * a.save_ld;
#pragma unroll
          for (int i = 0; i < E; ++i) {
            const int p = t + i * T;
            if (p < a.n_valid) svw[p] = v[i];
          }
        }
#pragma unroll
        for (int i = 0; i < E; ++i) v[i] = cmul(v[i], wm[i]);
      } else {
        const float s = a.mod_sign;
#pragma unroll
        for (int i = 0; i < E; ++i) {
          if constexpr (GK == 2) {
            float2 g = cmul(v[i], cconj(sv[i]));
            if (s < 0.f) g = cconj(g);
            gacc_c[i] = cadd(gacc_c[i], g);
          }
          v[i] = cmul(v[i], wm[i]);
          if constexpr (GK == 1) {
            // Im(du * conj(u_saved))
            const float im = v[i].y * sv[i].x - v[i].x * sv[i].y;
            gacc[i] = fmaf(s * fb, im, gacc[i]);
          }
        }
      }
    }
    if (a.fwd_after) {
      fft_forward<N, E, 1>(v, t, tw, PF ? cur : buf0);
    }
    if (row_ok) {
      float2* dst = a.dst + (long long)b * a.dst_bstride + (long long)y * a.dst_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < store_n) dst[p] = v[i];
      }
    }
    __syncthreads();  // `cur` is refilled by the prefetch of the next iteration
  }
  if constexpr (GK != 0) {
    if (row_ok) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < a.n_valid) {
          const long long q = (long long)y * a.param_ld + p;
          if constexpr (GK == 2)
            reinterpret_cast<float2*>(a.grad)[q] = gacc_c[i];
          else
            reinterpret_cast<float*>(a.grad)[q] = gacc[i];
        }
      }
    }
  }
}

// --------------------------------------------------------------------------
// Column pass: CTA (work item, column tile).  A work item is a run of fields
// (from a.field_list) that share one transfer function; the H tile is loaded
// once into registers.  PF stages the next field's tile with cp.async.
// Shared memory: 2 * W * SLOTS float2 (PF) or W * SLOTS float2.
// --------------------------------------------------------------------------
template <int N, int E, int W, bool PF>
__global__ void __launch_bounds__(W*(N / E), min_blocks(W*(N / E), E))
    col_pass_kernel(const ColPassArgs a, const float2* __restrict__ tw) {
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  extern __shared__ float2 dsm[];

  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  const int col = blockIdx.y * W + c;
  const bool col_ok = col < a.ncols;
  const int f0 = a.item_start ? a.item_start[blockIdx.x] : blockIdx.x;
  const int f1 = a.item_start ? a.item_start[blockIdx.x + 1] : blockIdx.x + 1;
  float2* buf0 = dsm + c;
  float2* buf1 = dsm + W * SLOTS + c;
  auto field_of = [&](int f) { return a.field_list ? a.field_list[f] : f; };

  // one transfer function per work item, read through L1/L2 for every field
  const float2* H = a.fft_only ? nullptr : a.H + (long long)a.h_index[field_of(f0)] * a.h_stride + col;
  auto prefetch = [&](int f, float2* dst) {
    const float2* src = a.buf + (long long)field_of(f) * a.bstride + col;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int p = t + i * T;
      if (p < a.y_in) cp_async8(dst + spad(p) * W, src + (long long)p * a.ld);
    }
  };
  if constexpr (PF) {
    if (col_ok && f0 < f1) prefetch(f0, buf0);
    cp_async_commit();
  }
  for (int f = f0; f < f1; ++f) {
    float2* buf = a.buf + (long long)field_of(f) * a.bstride + col;
    float2* cur = ((f - f0) & 1) ? buf1 : buf0;
    float2 v[E];
    if constexpr (PF) {
      float2* nxt = ((f - f0) & 1) ? buf0 : buf1;
      if (col_ok && f + 1 < f1) prefetch(f + 1, nxt);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (col_ok && p < a.y_in) ? cur[spad(p) * W] : make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (col_ok && p < a.y_in) ? buf[(long long)p * a.ld] : make_float2(0.f, 0.f);
      }
    }
    fft_forward<N, E, W>(v, t, tw, PF ? cur : buf0);
    if (a.fft_only) {
      if (col_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (p < a.y_out) buf[(long long)p * a.ld] = v[i];
        }
      }
    } else {
      // spectrum at ky = p: v <- conj(H * X) (inverse via conj-FFT-conj; H carries 1/(Nx*Ny))
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 hv = col_ok ? __ldg(H + (long long)p * a.ncols) : make_float2(0.f, 0.f);
        if (a.conj_h) hv = cconj(hv);
        v[i] = cconj(cmul(v[i], hv));
      }
      fft_forward<N, E, W>(v, t, tw, PF ? cur : buf0);
      if (col_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (p < a.y_out) buf[(long long)p * a.ld] = cconj(v[i]);
        }
      }
    }
    __syncthreads();  // `cur` is refilled by the prefetch of the next iteration
  }
}

// --------------------------------------------------------------------------
// Launch helpers used by the per-size translation units.
// --------------------------------------------------------------------------
template <int N, int E, int LANES>
struct RowShape {
  static constexpr int threads = LANES * (N / E);
  static size_t smem(bool pf) { return sizeof(float2) * (size_t)(pf ? 2 : 1) * LANES * SmemSize<N>::value; }
};

template <typename K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int N, int E, int LANES>
cudaError_t row_launch_shape(const RowPassArgs& a, const float2* tw, cudaStream_t s, bool pf) {
  using SH = RowShape<N, E, LANES>;
  const size_t smem = SH::smem(pf);
  dim3 grid((a.batch + a.fields_per_cta - 1) / a.fields_per_cta, (a.nrows + LANES - 1) / LANES);
  const bool grad = a.mod_bwd && a.grad != nullptr && a.mod_kind != MOD_NONE;
  cudaError_t e = cudaSuccess;
#define FO_ROW_GO(GK, PFV)                                                      \
  do {                                                                          \
    e = set_smem(row_pass_kernel<N, E, LANES, GK, PFV>, smem);                  \
    if (e == cudaSuccess) row_pass_kernel<N, E, LANES, GK, PFV><<<grid, SH::threads, smem, s>>>(a, tw); \
  } while (0)
  if (!grad) {
    if (pf) FO_ROW_GO(0, true); else FO_ROW_GO(0, false);
  } else if (a.mod_kind == MOD_MASK) {
    FO_ROW_GO(2, false);
  } else {
    if (pf) FO_ROW_GO(1, true); else FO_ROW_GO(1, false);
  }
#undef FO_ROW_GO
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <int N, int E, int W>
cudaError_t col_launch_shape(const ColPassArgs& a, const float2* tw, cudaStream_t s, bool pf) {
  constexpr int threads = W * (N / E);
  const size_t smem = sizeof(float2) * (size_t)(pf ? 2 : 1) * W * SmemSize<N>::value;
  dim3 grid(a.n_items, (a.ncols + W - 1) / W);
  cudaError_t e;
  if (pf) {
    e = set_smem(col_pass_kernel<N, E, W, true>, smem);
    if (e == cudaSuccess) col_pass_kernel<N, E, W, true><<<grid, threads, smem, s>>>(a, tw);
  } else {
    e = set_smem(col_pass_kernel<N, E, W, false>, smem);
    if (e == cudaSuccess) col_pass_kernel<N, E, W, false><<<grid, threads, smem, s>>>(a, tw);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace fo
