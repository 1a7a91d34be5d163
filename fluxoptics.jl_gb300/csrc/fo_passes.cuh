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

#include <cuda.h>

#include <utility>

#include "fo_fft.cuh"
#include "fo_internal.h"

namespace fo {

// Register cap per thread of the E = 16 row passes without a gradient, and whether
// forward row passes keep their twiddles in registers (build-time settings).
#ifndef FO_ROW_E16_REG_CAP
#define FO_ROW_E16_REG_CAP 96
#endif
#ifndef FO_ROW_TWR
#define FO_ROW_TWR 0
#endif
// Register cap per thread of the row pass that shares the metric and the adjoint's seed
// (GK = 4) for E = 16 (build-time setting).
#ifndef FO_ROW_SEED_REG_CAP
#define FO_ROW_SEED_REG_CAP 128
#endif

// Minimum resident CTAs per SM requested from the compiler: caps registers near
// 96 per thread for E <= 8 and at 128 (cap16) for E = 16.
__host__ __device__ constexpr int min_blocks(int threads, int E, int cap16 = 128) {
  return (65536 / (threads * (E <= 8 ? 96 : cap16))) > 0 ? 65536 / (threads * (E <= 8 ? 96 : cap16)) : 1;
}

// Programmatic dependent launch: let the next pass be launched while this one
// drains, then wait until the previous pass has completed and flushed before
// touching global memory.  Both are no-ops when the launch carries no
// programmatic dependency.
__device__ __forceinline__ void pdl_prologue() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

// L2 eviction priorities for data that one pass writes and reads back soon
// (createpolicy / cache_hint, sm_80 and later).
__device__ __forceinline__ unsigned long long l2_evict_last_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_hint(float2* ptr, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;\n" ::"l"(ptr), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}
__device__ __forceinline__ float2 ld_hint(const float2* ptr, unsigned long long pol) {
  float2 v;
  asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;\n" : "=f"(v.x), "=f"(v.y) : "l"(ptr), "l"(pol)
               : "memory");
  return v;
}
// Whether the shared metric + seed pass marks the rows it writes back and reads again
// as evict-last / evict-first in L2 (build-time setting).
#ifndef FO_SEED_L2_HINTS
#define FO_SEED_L2_HINTS 1
#endif

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
// Row pass.  GK: gradient accumulator (0 none, 1 real: phase / dn, 2 complex: mask,
// 3: intensity of the output summed over the CTA's fields for the squared
// intensity difference, see RowPassArgs::sid_target; 4: the same followed by the
// seeded first pass of the adjoint sweep, see RowPassArgs::seed_dst).
// PF: stage the next field's row through cp.async (needs load_n == N).
// Shared memory: 2 * LANES * SLOTS float2 (PF) or LANES * SLOTS float2, plus
// LANES * N float2 for the modulation-factor cache when GK != 0.
// --------------------------------------------------------------------------
// FULL: the row count is a multiple of LANES and n_valid == N, so no
// per-element guards are needed.
// RP (passes without a gradient only): the next field's row is loaded into a second
// set of registers while the current one is transformed, so that every row keeps a
// load in flight (128-register cap).
template <int N, int E, int LANES, int GK, bool PF, bool FULL, bool RP = false>
__global__ void __launch_bounds__(LANES*(N / E),
                                  min_blocks(LANES*(N / E), E,
                                             RP                          ? 128
                                             : (GK == 0 || GK == 3)      ? FO_ROW_E16_REG_CAP
                                             : ((GK == 4 || GK == 5) ? FO_ROW_SEED_REG_CAP : 128)))
    row_pass_kernel(const RowPassArgs a, const float2* __restrict__ tw) {
  static_assert(!RP || (GK == 0 && !PF), "register prefetch is for passes without a gradient or staging");
  pdl_prologue();
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  extern __shared__ float2 dsm[];

  const int t = threadIdx.x % T;
  const int lane = threadIdx.x / T;
  const int y = blockIdx.y * LANES + lane;
  const bool row_ok = FULL || y < a.nrows;
  float2* buf0 = dsm + lane * SLOTS;
  float2* buf1 = dsm + (LANES + lane) * SLOTS;

  const int n_valid = FULL ? N : a.n_valid;
  const int load_n = a.inv_first ? N : n_valid;
  const int store_n = a.fwd_after ? N : n_valid;
  constexpr int GR = (GK == 1 || GK == 3) ? E : 1;
  constexpr int GC = (GK == 2) ? E : 1;
  float gacc[GR];
  float2 gacc_c[GC];
#pragma unroll
  for (int i = 0; i < GR; ++i) gacc[i] = 0.f;
#pragma unroll
  for (int i = 0; i < GC; ++i) gacc_c[i] = make_float2(0.f, 0.f);

  // per-pixel modulation factor, cached across fields while the field factor is
  // unchanged: in registers, or for the gradient passes (which already hold the
  // saved input and the accumulator) in this thread's own shared-memory slots
  constexpr bool WMS = (GK != 0);
  float2 wm[WMS ? 1 : E];
  float2* wms = dsm + (PF ? 2 : 1) * LANES * SLOTS + lane * N;
  auto wm_set = [&](int i, float2 w) {
    if constexpr (WMS)
      wms[t + i * T] = w;
    else
      wm[i] = w;
  };
  auto wm_get = [&](int i) -> float2 {
    if constexpr (WMS)
      return wms[t + i * T];
    else
      return wm[i];
  };
  float wm_fb = -1.f;
  float2 wm_amp = make_float2(1.f, 0.f);

  // Passes without a gradient accumulator have the registers to keep this
  // thread's twiddles for all the CTA's fields.
  constexpr bool TWR = FO_ROW_TWR && (GK == 0) && (E == 16) && FULL && TwRegs<N, E>::total <= 24;
  float2 wr[TwRegs<N, E>::size];
  if constexpr (TWR) load_twiddles<N, E>(wr, t, tw);
  auto fft = [&](float2(&x)[E], float2* sm) {
    if constexpr (TWR)
      fft_forward_r<N, E, 1>(x, t, wr, sm);
    else
      fft_forward<N, E, 1>(x, t, tw, sm);
  };

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
  if constexpr (GK == 5) {
    // The chain's last forward pass, SquaredFieldDifference and the first pass of the
    // adjoint sweep in one launch.  Each field is independent: its spectrum row is
    // inverse-transformed along x (the output row, written to a.dst when set), the
    // difference d = u - v to the reference field gives the row's sum of |d|^2
    // (fixed-order reduction) and the seed 2 dc_b d, which is forward-transformed and
    // written over the spectrum row.  The same arithmetic as the forward pass, the
    // metric's pull-back (fo_sfd_backward) and the adjoint's first pass, so the seeds
    // and the gradients are the same bit for bit.
    float* red = reinterpret_cast<float*>(dsm + LANES * SLOTS) + lane * 32;  // past the exchange tiles
    for (int f = f0; f < f1; ++f) {
      const int b = field_of(f);
      float2* row = a.seed_dst + (long long)b * a.seed_bstride + (long long)y * a.seed_ld;
      float2 v[E];
#pragma unroll
      for (int i = 0; i < E; ++i) v[i] = row_ok ? cconj(row[t + i * T]) : make_float2(0.f, 0.f);
      fft(v, buf0);
      const float2* vr = a.sfd_v + (long long)b * a.dst_bstride + (long long)y * a.dst_ld;
      float2* dst = a.dst ? a.dst + (long long)b * a.dst_bstride + (long long)y * a.dst_ld : nullptr;
      const float k2 = 2.f * (a.sfd_dc ? a.sfd_dc[b] : 1.f);
      float r2 = 0.f;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 d = make_float2(0.f, 0.f);
        if (row_ok && p < n_valid) {
          const float2 uo = cconj(v[i]);
          if (dst) dst[p] = uo;
          const float2 w = vr[p];
          d = make_float2(uo.x - w.x, uo.y - w.y);
          r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, r2));
        }
        v[i] = make_float2(k2 * d.x, k2 * d.y);
      }
      constexpr int G = T < 32 ? T : 32;
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
      if constexpr (T > 32) {
        if ((t & 31) == 0) red[t >> 5] = r2;
        __syncthreads();
        if (t == 0) {
          float acc = 0.f;
#pragma unroll
          for (int w = 0; w < T / 32; ++w) acc += red[w];
          r2 = acc;
        }
      }
      if (t == 0 && row_ok) a.sfd_rows[(long long)y * a.batch + b] = r2;
      fft(v, buf0);  // its first barrier also ends this field's reads of `red`
      if (row_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) row[t + i * T] = v[i];
      }
    }
    return;
  }
  if constexpr (GK == 4) {
    // The chain's last forward pass, SquaredIntensityDifference and the first pass of the
    // seeded adjoint sweep in one launch.  Loop 1 inverse-transforms the rows of the
    // CTA's fields (the fields of one target slice) along x, sums their intensities,
    // writes the output field when a.dst is set, and puts each real-space row back in
    // place of its spectrum row (a.seed_dst == a.src).  Loop 2 reads those rows back --
    // newest field first, so that most of them are still in L2 and the adjoint row that
    // overwrites each one leaves a single write to DRAM -- multiplies them by
    // 4 dc_t (I - t) and forward-transforms them in place.  No other CTA touches these
    // rows.  The arithmetic equals the GK = 3 pass followed by the seeded pass, so the
    // results are the same bit for bit.
    const int ts = a.tidx[field_of(f0)];
    float r[E];
#pragma unroll
    for (int i = 0; i < E; ++i) r[i] = 0.f;
    for (int f = f0; f < f1; ++f) {
      const int b = field_of(f);
      float2* row = a.seed_dst + (long long)b * a.seed_bstride + (long long)y * a.seed_ld;
      float2 v[E];
#pragma unroll
      for (int i = 0; i < E; ++i) v[i] = row_ok ? cconj(row[t + i * T]) : make_float2(0.f, 0.f);
      fft(v, buf0);
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (p < n_valid) ? cconj(v[i]) : make_float2(0.f, 0.f);  // crop / re-pad
        r[i] = fmaf(v[i].x, v[i].x, fmaf(v[i].y, v[i].y, r[i]));
      }
      if (row_ok) {
        if constexpr (FO_SEED_L2_HINTS) {
          const unsigned long long keep = l2_evict_last_policy();
#pragma unroll
          for (int i = 0; i < E; ++i) st_hint(row + t + i * T, v[i], keep);
        } else {
#pragma unroll
          for (int i = 0; i < E; ++i) row[t + i * T] = v[i];
        }
        if (a.dst) {
          float2* dst = a.dst + (long long)b * a.dst_bstride + (long long)y * a.dst_ld;
#pragma unroll
          for (int i = 0; i < E; ++i) {
            const int p = t + i * T;
            if (p < n_valid) dst[p] = v[i];
          }
        }
      }
    }
    // residual I - target of this row and the row's sum of squares (as GK = 3)
    float r2 = 0.f;
    {
      const long long off = (long long)ts * a.resid_tstride + (long long)y * a.resid_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float rr = 0.f;
        if (row_ok && p < n_valid) {
          rr = r[i] - a.sid_target[off + p];
          a.sid_resid[off + p] = rr;
          r2 = fmaf(rr, rr, r2);
        }
        r[i] = rr;
      }
    }
    constexpr int G = T < 32 ? T : 32;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    float* red = reinterpret_cast<float*>(buf0);
    if constexpr (T > 32) {
      __syncthreads();  // every warp is done with the last transform's reads of buf0
      if ((t & 31) == 0) red[t >> 5] = r2;
      __syncthreads();
      if (t == 0) {
        float acc = 0.f;
#pragma unroll
        for (int w = 0; w < T / 32; ++w) acc += red[w];
        r2 = acc;
      }
    }
    if (t == 0 && row_ok) a.sid_partials[(long long)y * a.sid_T + ts] = r2;
    const float k4 = 4.f * a.dc[ts];
    for (int f = f1 - 1; f >= f0; --f) {
      const int b = field_of(f);
      float2* row = a.seed_dst + (long long)b * a.seed_bstride + (long long)y * a.seed_ld;
      float2 v[E];
      if constexpr (FO_SEED_L2_HINTS) {
        const unsigned long long last_use = l2_evict_first_policy();
#pragma unroll
        for (int i = 0; i < E; ++i)
          v[i] = row_ok ? cscale(ld_hint(row + t + i * T, last_use), k4 * r[i]) : make_float2(0.f, 0.f);
      } else {
#pragma unroll
        for (int i = 0; i < E; ++i) v[i] = row_ok ? cscale(row[t + i * T], k4 * r[i]) : make_float2(0.f, 0.f);
      }
      fft(v, buf0);
      if (row_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) row[t + i * T] = v[i];
      }
    }
    return;
  }
  if constexpr (PF) {
    if (row_ok && f0 < f1) prefetch(f0, buf0);
    cp_async_commit();
  }
  float2 nxt[RP ? E : 1];
  auto load_next = [&](int f) {
    if constexpr (RP) {
      const float2* src = a.src + (long long)field_of(f) * a.src_bstride + (long long)y * a.src_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        nxt[i] = (row_ok && p < load_n) ? src[p] : make_float2(0.f, 0.f);
      }
    }
  };
  if constexpr (RP) {
    if (f0 < f1) load_next(f0);
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
    } else if constexpr (RP) {
#pragma unroll
      for (int i = 0; i < E; ++i) v[i] = a.inv_first ? cconj(nxt[i]) : nxt[i];
      if (f + 1 < f1) load_next(f + 1);  // another field's row: no overlap with this field's stores
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
    // the saved modulation input of the gradient passes, loaded where the inverse
    // transform hides the latency
    float2 sv[(GK == 1 || GK == 2) ? E : 1];
    if constexpr (GK == 1 || GK == 2) {
      const float2* svp = a.saved + (long long)b * a.saved_bstride + (long long)y * a.saved_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        sv[i] = (row_ok && p < n_valid) ? svp[p] : make_float2(0.f, 0.f);
      }
    }
    // per-field factor of the phase-like kinds (dn: kdz / lambda; TeaDOE: 2 pi dn(lambda) /
    // lambda) and TeaDOE's per-field amplitude r(lambda)
    float fb = 1.f;
    float2 famp = make_float2(1.f, 0.f);
    if (a.mod_kind == MOD_DN) {
      fb = a.mod_scale * a.inv_lambda[b];
    } else if (a.mod_kind == MOD_TEA) {
      const float4 fc = a.field_coef[b];
      fb = fc.x;
      famp = make_float2(fc.y, fc.z);
    }
    if (a.mod_kind != MOD_NONE && row_ok && (fb != wm_fb || famp.x != wm_amp.x || famp.y != wm_amp.y)) {
      const float s = a.mod_sign;
      // forward: r (conj for s < 0); adjoint: conj(r) (r for s < 0)
      const float2 amp = ((s < 0.f) != (a.mod_bwd != 0)) ? cconj(famp) : famp;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 w = make_float2(1.f, 0.f);
        if (p < n_valid) {
          const long long q = (long long)y * a.param_ld + p;
          if (a.mod_kind == MOD_MASK) {
            w = reinterpret_cast<const float2*>(a.mod_param)[q];
            // forward: m (conj for s < 0); adjoint: conj(m) (m for s < 0)
            if ((s < 0.f) != (a.mod_bwd != 0)) w = cconj(w);
          } else {
            const float ph = reinterpret_cast<const float*>(a.mod_param)[q];
            w = cis_f((a.mod_bwd ? -s : s) * fb * ph);
            if (a.mod_kind == MOD_TEA) w = cmul(w, amp);
          }
        }
        wm_set(i, w);
      }
      wm_fb = fb;
      wm_amp = famp;
    }

    if (a.inv_first) {
      fft(v, PF ? cur : buf0);
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (p < n_valid) ? cconj(v[i]) : make_float2(0.f, 0.f);  // crop / re-pad
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
        if (p < n_valid) v[i] = cscale(v[i], k4 * rr[p]);
      }
    }
    // field probes: the plane before and after this pass's modulation (forward only)
    auto probe_store = [&](float2* pr) {
      float2* pw = pr + (long long)b * a.save_bstride + (long long)y * a.save_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < n_valid) pw[p] = v[i];
      }
    };
    if (a.probe_pre && row_ok) probe_store(a.probe_pre);
    if (a.mod_kind != MOD_NONE && row_ok) {
      if (!a.mod_bwd) {
        if (a.save) {
          float2* svw = a.save + (long long)b * a.save_bstride + (long long)y * a.save_ld;
#pragma unroll
          for (int i = 0; i < E; ++i) {
            const int p = t + i * T;
            if (p < n_valid) svw[p] = v[i];
          }
        }
#pragma unroll
        for (int i = 0; i < E; ++i) v[i] = cmul(v[i], wm_get(i));
      } else {
        const float s = a.mod_sign;
#pragma unroll
        for (int i = 0; i < E; ++i) {
          if constexpr (GK == 2) {
            float2 g = cmul(v[i], cconj(sv[i]));
            if (s < 0.f) g = cconj(g);
            gacc_c[i] = cadd(gacc_c[i], g);
          }
          v[i] = cmul(v[i], wm_get(i));
          if constexpr (GK == 1) {
            // Im(du * conj(u_saved))
            const float im = v[i].y * sv[i].x - v[i].x * sv[i].y;
            gacc[i] = fmaf(s * fb, im, gacc[i]);
          }
        }
      }
    }
    if (a.probe_post && row_ok) probe_store(a.probe_post);
    if (a.fwd_after) fft(v, PF ? cur : buf0);
    if constexpr (GK == 3) {
#pragma unroll
      for (int i = 0; i < E; ++i) gacc[i] = fmaf(v[i].x, v[i].x, fmaf(v[i].y, v[i].y, gacc[i]));
    }
    if (row_ok && a.dst) {  // a null destination discards the pass output (gradients only)
      float2* dst = a.dst + (long long)b * a.dst_bstride + (long long)y * a.dst_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < store_n) dst[p] = v[i];
      }
    }
    __syncthreads();  // `cur` is refilled by the prefetch of the next iteration
  }
  if constexpr (GK == 3) {
    // residual I - target of this row for the CTA's target slice, and the row's sum
    // of squared residuals (fixed-order reduction)
    const int ts = a.tidx[field_of(f0)];
    float r2 = 0.f;
    if (row_ok) {
      const long long off = (long long)ts * a.resid_tstride + (long long)y * a.resid_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < n_valid) {
          const float r = gacc[i] - a.sid_target[off + p];
          a.sid_resid[off + p] = r;
          r2 = fmaf(r, r, r2);
        }
      }
    }
    constexpr int G = T < 32 ? T : 32;  // lanes of one row within a warp
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    float* red = reinterpret_cast<float*>(buf0);  // this row's staging slots are free now
    if constexpr (T > 32) {
      if ((t & 31) == 0) red[t >> 5] = r2;
      __syncthreads();
      if (t == 0) {
        float acc = 0.f;
#pragma unroll
        for (int w = 0; w < T / 32; ++w) acc += red[w];
        r2 = acc;
      }
    }
    if (t == 0 && row_ok) a.sid_partials[(long long)y * a.sid_T + ts] = r2;
  }
  if constexpr (GK == 1 || GK == 2) {
    if (row_ok) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < n_valid) {
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
// (from a.field_list) that share one transfer function.  HS stages the H tile of
// the item in shared memory once; PF stages the next field's tile with 16-byte
// cp.async copies while the current one is transformed.
// Shared memory: (PF ? 2 : 1) * W * SLOTS float2 [+ N * W float2 when HS].
// --------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

// FULL: every column of the tile exists and all N rows are read and written
// (y_in == y_out == N), so no per-element guards are needed.
template <int N, int E, int W, bool PF, bool HS, bool FULL>
__global__ void __launch_bounds__(W*(N / E), min_blocks(W*(N / E), E))
    col_pass_kernel(const ColPassArgs a, const float2* __restrict__ tw) {
  pdl_prologue();
  static_assert(W % 2 == 0, "16-byte staging needs an even tile width");
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  constexpr int THREADS = W * (N / E);
  constexpr int CHUNKS = N * W / 2;  // 16-byte chunks of one tile
  extern __shared__ float4 dsm4[];
  float2* dsm = reinterpret_cast<float2*>(dsm4);
  float2* st0 = dsm;
  float2* st1 = dsm + W * SLOTS;
  float2* hs = dsm + (PF ? 2 : 1) * W * SLOTS;

  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  const int col0 = blockIdx.y * W;
  const int col = col0 + c;
  const bool col_ok = FULL || col < a.ncols;
  const int y_in = FULL ? N : a.y_in;
  const int y_out = FULL ? N : a.y_out;
  const int ld = a.ld;
  const int f0 = a.item_start ? a.item_start[blockIdx.x] : blockIdx.x;
  const int f1 = a.item_start ? a.item_start[blockIdx.x + 1] : blockIdx.x + 1;
  auto field_of = [&](int f) { return a.field_list ? a.field_list[f] : f; };
  const float2* Hg = a.fft_only ? nullptr : a.H + (long long)a.h_index[field_of(f0)] * a.h_stride + col0;

  // tile (rows < y_in, columns col0 .. col0+W-1) -> padded smem, 16 bytes per copy
  auto prefetch = [&](int f, float2* dst) {
    const float2* src = a.buf + (long long)field_of(f) * a.bstride + col0;
#pragma unroll
    for (int k = 0; k < CHUNKS / THREADS; ++k) {
      const int q = threadIdx.x + k * THREADS;
      const int row = q / (W / 2), cp = q % (W / 2);
      if (FULL || (row < y_in && col0 + 2 * cp < a.ncols))
        cp_async16(dst + spad(row) * W + 2 * cp, src + row * ld + 2 * cp);
    }
  };
  if constexpr (HS) {
    if (!a.fft_only) {
#pragma unroll
      for (int k = 0; k < CHUNKS / THREADS; ++k) {
        const int q = threadIdx.x + k * THREADS;
        const int row = q / (W / 2), cp = q % (W / 2);
        if (FULL || col0 + 2 * cp < a.ncols) cp_async16(hs + row * W + 2 * cp, Hg + row * a.ncols + 2 * cp);
      }
    }
  }
  if constexpr (PF) {
    if (f0 < f1) prefetch(f0, st0);
  }
  cp_async_commit();
  if constexpr (!PF) {
    cp_async_wait<0>();
    __syncthreads();
  }
  const float2 hconj = make_float2(1.f, a.conj_h ? -1.f : 1.f);

  for (int f = f0; f < f1; ++f) {
    float2* buf = a.buf + (long long)field_of(f) * a.bstride + col;
    float2* cur = ((f - f0) & 1) ? st1 : st0;
    float2 v[E];
    if constexpr (PF) {
      float2* nxt = ((f - f0) & 1) ? st0 : st1;
      if (f + 1 < f1) prefetch(f + 1, nxt);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (FULL || (col_ok && p < y_in)) ? cur[spad(p) * W + c] : make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (FULL || (col_ok && p < y_in)) ? buf[p * ld] : make_float2(0.f, 0.f);
      }
    }
    float2* ex = (PF ? cur : st0) + c;
    fft_forward<N, E, W>(v, t, tw, ex);
    if (a.fft_only) {
      if (col_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (FULL || p < y_out) buf[p * ld] = v[i];
        }
      }
    } else {
      // spectrum at ky = p: v <- conj(H * X) (inverse via conj-FFT-conj; H carries 1/(Nx*Ny))
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 hv;
        if constexpr (HS)
          hv = hs[p * W + c];
        else
          hv = col_ok ? Hg[p * a.ncols + c] : make_float2(0.f, 0.f);
        hv.y *= hconj.y;  // conj(H) for the adjoint direction
        // conj(X * H) = (xr hr - xi hi, -(xr hi + xi hr))
        v[i] = make_float2(fmaf(v[i].x, hv.x, -v[i].y * hv.y), -fmaf(v[i].x, hv.y, v[i].y * hv.x));
      }
      fft_forward<N, E, W>(v, t, tw, ex);
      if (col_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (FULL || p < y_out) buf[p * ld] = cconj(v[i]);
        }
      }
    }
    __syncthreads();  // `cur` is refilled by the prefetch of the next iteration
  }
}

// --------------------------------------------------------------------------
// Paired column pass: each thread carries two adjacent columns (cf2), so global,
// shared-memory and twiddle accesses are shared by two independent transforms.
// Same shared-memory layout as col_pass_kernel (a padded tile of W columns).
// --------------------------------------------------------------------------
template <int N, int E, int W, bool PF, bool HS>
__global__ void __launch_bounds__((W / 2) * (N / E), min_blocks((W / 2) * (N / E), 2 * E))
    col_pass2_kernel(const ColPassArgs a, const float2* __restrict__ tw) {
  pdl_prologue();
  static_assert(W % 2 == 0, "paired columns need an even tile width");
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  constexpr int WP = W / 2;             // column pairs per tile
  constexpr int THREADS = WP * (N / E);
  constexpr int CHUNKS = N * WP;         // 16-byte chunks of one tile
  extern __shared__ float4 dsm4[];
  cf2* st0 = reinterpret_cast<cf2*>(dsm4);
  cf2* st1 = st0 + WP * SLOTS;
  cf2* hs = st0 + (PF ? 2 : 1) * WP * SLOTS;

  const int cp = threadIdx.x % WP;
  const int t = threadIdx.x / WP;
  const int col0 = blockIdx.y * W;
  const int col = col0 + 2 * cp;
  const bool col_ok = col < a.ncols;
  const int f0 = a.item_start ? a.item_start[blockIdx.x] : blockIdx.x;
  const int f1 = a.item_start ? a.item_start[blockIdx.x + 1] : blockIdx.x + 1;
  auto field_of = [&](int f) { return a.field_list ? a.field_list[f] : f; };
  const float2* Hg = a.fft_only ? nullptr : a.H + (long long)a.h_index[field_of(f0)] * a.h_stride + col0;

  auto prefetch = [&](int f, cf2* dst) {
    const float2* src = a.buf + (long long)field_of(f) * a.bstride + col0;
#pragma unroll
    for (int k = 0; k < CHUNKS / THREADS; ++k) {
      const int q = threadIdx.x + k * THREADS;
      const int row = q / WP, c2 = q % WP;
      if (row < a.y_in && col0 + 2 * c2 < a.ncols)
        cp_async16(dst + spad(row) * WP + c2, src + (long long)row * a.ld + 2 * c2);
    }
  };
  if constexpr (HS) {
    if (!a.fft_only) {
#pragma unroll
      for (int k = 0; k < CHUNKS / THREADS; ++k) {
        const int q = threadIdx.x + k * THREADS;
        const int row = q / WP, c2 = q % WP;
        if (col0 + 2 * c2 < a.ncols) cp_async16(hs + row * WP + c2, Hg + (long long)row * a.ncols + 2 * c2);
      }
    }
  }
  if constexpr (PF) {
    if (f0 < f1) prefetch(f0, st0);
  }
  cp_async_commit();
  if constexpr (!PF) {
    cp_async_wait<0>();
    __syncthreads();
  }

  for (int f = f0; f < f1; ++f) {
    cf2* buf = reinterpret_cast<cf2*>(a.buf + (long long)field_of(f) * a.bstride + col);
    const long long ldp = a.ld / 2;  // row stride in cf2 units (ld is even)
    cf2* cur = ((f - f0) & 1) ? st1 : st0;
    cf2 v[E];
    if constexpr (PF) {
      cf2* nxt = ((f - f0) & 1) ? st0 : st1;
      if (f + 1 < f1) prefetch(f + 1, nxt);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (col_ok && p < a.y_in) ? cur[spad(p) * WP + cp] : vzero<cf2>();
      }
    } else {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (col_ok && p < a.y_in) ? buf[(long long)p * ldp] : vzero<cf2>();
      }
    }
    cf2* ex = (PF ? cur : st0) + cp;
    fft_forward<N, E, WP>(v, t, tw, ex);
    if (a.fft_only) {
      if (col_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (p < a.y_out) buf[(long long)p * ldp] = v[i];
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        cf2 hv;
        if constexpr (HS) {
          hv = hs[p * WP + cp];
        } else {
          hv = col_ok ? *reinterpret_cast<const cf2*>(Hg + (long long)p * a.ncols + 2 * cp) : vzero<cf2>();
        }
        if (a.conj_h) hv = cconj(hv);
        v[i] = cf2{cconj(cmul(v[i].a, hv.a)), cconj(cmul(v[i].b, hv.b))};
      }
      fft_forward<N, E, WP>(v, t, tw, ex);
      if (col_ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (p < a.y_out) buf[(long long)p * ldp] = cconj(v[i]);
        }
      }
    }
    __syncthreads();  // `cur` is refilled by the prefetch of the next iteration
  }
}

// --------------------------------------------------------------------------
// Lane-major column pass: the T threads of lane c transform column col0 + c and
// synchronise among themselves only (named barrier c+1), like the row pass.
// Tiles move between global and shared memory with a row-major copy mapping
// (coalesced 32-byte row segments): cp.async in, shared-memory staging out.
// Shared memory: 2 * W * LS float2 (LS = SLOTS + 4, conflict-free lane stride)
// [+ W * (N + 4) float2 for the H tile when HS].
// --------------------------------------------------------------------------
template <int N>
struct LaneStride {
  static constexpr int value = SmemSize<N>::value + 4;
};

template <int N, int E, int W, bool HS>
__global__ void __launch_bounds__(W*(N / E), min_blocks(W*(N / E), E))
    col_lane_kernel(const ColPassArgs a, const float2* __restrict__ tw) {
  pdl_prologue();
  constexpr int T = N / E;
  static_assert(T % 32 == 0, "a lane must be whole warps");
  constexpr int LS = LaneStride<N>::value;
  constexpr int HLS = N + 4;
  constexpr int THREADS = W * T;
  extern __shared__ float4 dsm4[];
  float2* st0 = reinterpret_cast<float2*>(dsm4);
  float2* st1 = st0 + W * LS;
  float2* hs = st0 + 2 * W * LS;

  const int lane = threadIdx.x / T;
  const int t = threadIdx.x % T;
  const int col0 = blockIdx.y * W;
  const bool lane_ok = col0 + lane < a.ncols;
  const int f0 = a.item_start ? a.item_start[blockIdx.x] : blockIdx.x;
  const int f1 = a.item_start ? a.item_start[blockIdx.x + 1] : blockIdx.x + 1;
  auto field_of = [&](int f) { return a.field_list ? a.field_list[f] : f; };
  const float2* Hg = a.fft_only ? nullptr : a.H + (long long)a.h_index[field_of(f0)] * a.h_stride + col0;

  auto prefetch = [&](int f, float2* dst) {
    const float2* src = a.buf + (long long)field_of(f) * a.bstride + col0;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int q = threadIdx.x + k * THREADS;
      const int row = q / W, c = q % W;
      if (row < a.y_in && col0 + c < a.ncols) cp_async8(dst + c * LS + spad(row), src + (long long)row * a.ld + c);
    }
  };
  if constexpr (HS) {
    if (!a.fft_only) {
#pragma unroll
      for (int k = 0; k < E; ++k) {
        const int q = threadIdx.x + k * THREADS;
        const int row = q / W, c = q % W;
        if (col0 + c < a.ncols) cp_async8(hs + c * HLS + row, Hg + (long long)row * a.ncols + c);
      }
    }
  }
  if (f0 < f1) prefetch(f0, st0);
  cp_async_commit();

  for (int f = f0; f < f1; ++f) {
    float2* cur = ((f - f0) & 1) ? st1 : st0;
    float2* nxt = ((f - f0) & 1) ? st0 : st1;
    if (f + 1 < f1) prefetch(f + 1, nxt);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    float2* L = cur + lane * LS;
    float2 v[E];
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int p = t + i * T;
      v[i] = (lane_ok && p < a.y_in) ? L[spad(p)] : make_float2(0.f, 0.f);
    }
    fft_forward<N, E, 1>(v, t, tw, L, lane + 1, T);
    if (!a.fft_only) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        float2 hv;
        if constexpr (HS)
          hv = hs[lane * HLS + p];
        else
          hv = lane_ok ? Hg[(long long)p * a.ncols + lane] : make_float2(0.f, 0.f);
        if (a.conj_h) hv = cconj(hv);
        v[i] = cconj(cmul(v[i], hv));
      }
      fft_forward<N, E, 1>(v, t, tw, L, lane + 1, T);
#pragma unroll
      for (int i = 0; i < E; ++i) v[i] = cconj(v[i]);
    }
    fft_sync(lane + 1, T);  // the lane's last exchange reads are done
#pragma unroll
    for (int i = 0; i < E; ++i) L[spad(t + i * T)] = v[i];
    __syncthreads();
    float2* out = a.buf + (long long)field_of(f) * a.bstride + col0;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int q = threadIdx.x + k * THREADS;
      const int row = q / W, c = q % W;
      if (row < a.y_out && col0 + c < a.ncols) out[(long long)row * a.ld + c] = cur[c * LS + spad(row)];
    }
    __syncthreads();  // `cur` is refilled by the prefetch of the next iteration
  }
}

// --------------------------------------------------------------------------
// TMA column pass: the tile of the next field is fetched by the tensor-memory
// accelerator (cp.async.bulk.tensor, boxes of W columns x 256 rows x 1 field,
// completion on an mbarrier) into a dense staging buffer as soon as the current
// field's registers are loaded; the H tile of the work item is fetched the same
// way.  FFT exchanges use a separate padded buffer, which after the last stage
// also holds the result tile [N][W] for a TMA tensor store: the field leaves as
// whole boxes instead of W-column slivers of every row.  The field map is 3-D
// (columns, rows of one field, fields), so boxes are clipped at the field's last
// row: rows past it read as zeros and are never written.  Every mbarrier wait is
// bounded by %globaltimer: on expiry the CTA sets bit 0 of the device error word
// and returns (no copy is left in flight).
// Shared memory: 128 (alignment) + 2 * N * W + W * SLOTS float2 + 16 bytes.
// --------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for phase `parity` of `bar`: false when `limit_ns` elapsed first.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;  // the common case reads no timer
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) return false;
  }
  return true;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const void* tmap, int x, int y, int z, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const void* tmap, int x, int y, int z, int w,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_4d(const void* tmap, int x, int y, int z, int w, const void* src) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4, %5}], [%1];\n" ::"l"(
                   reinterpret_cast<unsigned long long>(tmap)),
               "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z), "r"(w)
               : "memory");
}
__device__ __forceinline__ void tma_store_3d(const void* tmap, int x, int y, int z, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];\n" ::"l"(
                   reinterpret_cast<unsigned long long>(tmap)),
               "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// The stores issued so far have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// The stores issued so far are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

template <int N, int E, int W, bool TWR>
__global__ void __launch_bounds__(W*(N / E), min_blocks(W*(N / E), E))
    col_tma_kernel(const ColPassArgs a, const float2* __restrict__ tw, const __grid_constant__ CUtensorMap tm_buf,
                   const __grid_constant__ CUtensorMap tm_h) {
  pdl_prologue();
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  constexpr int BOX = 256;
  extern __shared__ float4 dsm4[];
  // 128-byte aligned start, formed by pointer arithmetic on the shared array itself
  // so that every access below compiles to a shared-memory (not generic) access
  char* base = reinterpret_cast<char*>(dsm4) + ((128u - (smem_u32(dsm4) & 127u)) & 127u);
  float2* stage = reinterpret_cast<float2*>(base);  // dense [N][W]
  float2* hs = stage + N * W;                         // dense [N][W]
  float2* ex = hs + N * W;                            // padded exchange [SLOTS][W]
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(ex + W * SLOTS);  // [0] tile, [1] H
  __shared__ int s_abort;

  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  // A unit is a run [f0, f1) of field_list positions on the strip starting at col0:
  // the (item, strip) block of the 2-D launch, or entries of a.units.  With
  // a.persistent the CTA takes units blockIdx.x, blockIdx.x + gridDim.x, ... and
  // loads the next unit's first strip and H strip while it finishes the current one.
  struct Unit {
    int f0, f1, col0;
  };
  auto unit_at = [&](int k) -> Unit {
    const int4 u = a.units[k];
    return Unit{u.x, u.y, u.z * W};
  };
  Unit U;
  if (a.units) {
    U = unit_at(blockIdx.x);
  } else {
    U.f0 = a.item_start ? a.item_start[blockIdx.x] : blockIdx.x;
    U.f1 = a.item_start ? a.item_start[blockIdx.x + 1] : blockIdx.x + 1;
    U.col0 = blockIdx.y * W;
  }
  int uk = blockIdx.x;
  const int y_in = a.y_in, y_out = a.y_out;
  auto field_of = [&](int f) { return a.field_list ? a.field_list[f] : f; };
  const int nbox = (y_in + BOX - 1) / BOX;
  const unsigned tile_bytes = (unsigned)(nbox * BOX * W * sizeof(float2));

  auto issue_tile = [&](int f, int col0) {  // one thread
    mbar_expect_tx(&bar[0], tile_bytes);
    if (a.test_skip_copy) return;
    const int fz = field_of(f);
    if (a.tile4d)
      tma_load_4d(stage, &tm_buf, col0, 0, 0, fz, &bar[0]);
    else
      for (int k = 0; k < nbox; ++k) tma_load_3d(stage + k * BOX * W, &tm_buf, col0, k * BOX, fz, &bar[0]);
  };
  auto issue_h = [&](const Unit& u) {  // one thread
    mbar_expect_tx(&bar[1], (unsigned)(N * W * sizeof(float2)));
    const int hz = a.h_index[field_of(u.f0)];
    if (a.tile4d)
      tma_load_4d(hs, &tm_h, u.col0, 0, 0, hz, &bar[1]);
    else
      for (int k = 0; k < N / BOX; ++k) tma_load_2d(hs + k * BOX * W, &tm_h, u.col0, hz * N + k * BOX, &bar[1]);
  };
  const int nbox_out = (y_out + BOX - 1) / BOX;
  if (threadIdx.x == 0) {
    s_abort = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_proxy_async();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!a.fft_only) issue_h(U);
    if (U.f0 < U.f1) issue_tile(U.f0, U.col0);
  }
  float2 wr[TwRegs<N, E>::size];
  if constexpr (TWR) load_twiddles<N, E>(wr, t, tw);
  auto fft = [&](float2(&x)[E]) {
    if constexpr (TWR)
      fft_forward_r<N, E, W>(x, t, wr, ex + c);
    else
      fft_forward<N, E, W>(x, t, tw, ex + c);
  };
  bool ok = true;
  unsigned phase = 0, hphase = 0;
  const float hsign = a.conj_h ? -1.f : 1.f;

  while (true) {
    if (!a.fft_only) {
      if (ok) ok = mbar_wait_bounded(&bar[1], hphase, a.wait_ns);
      hphase ^= 1u;
    }
    const bool col_ok = U.col0 + c < a.ncols;
    const bool has_next = a.persistent && a.units && uk + (int)gridDim.x < a.n_units;
    Unit Un = U;
    if (has_next) Un = unit_at(uk + gridDim.x);

    for (int f = U.f0; f < U.f1; ++f) {
      const unsigned wait_phase = phase;
      if (ok) ok = mbar_wait_bounded(&bar[0], wait_phase, a.wait_ns);
      phase ^= 1u;
      if (!ok) s_abort = 1;
      float2 v[E];
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        v[i] = (col_ok && p < y_in) ? stage[p * W + c] : make_float2(0.f, 0.f);
      }
      __syncthreads();  // the staging buffer is free again; abort decision is uniform
      if (s_abort) {
        if (threadIdx.x == 0) {
          atomicOr(a.err_word, 1u);
          // let copies still in flight land (bounded) before the CTA's memory is released:
          // this field's strip and the current unit's H strip
          if (!a.test_skip_copy) mbar_wait_bounded(&bar[0], wait_phase, a.wait_ns);
          if (!a.fft_only) mbar_wait_bounded(&bar[1], hphase ^ 1u, a.wait_ns);
          bulk_wait_all();
        }
        return;
      }
      if (threadIdx.x == 0) {
        if (f + 1 < U.f1) {
          fence_proxy_async();
          issue_tile(f + 1, U.col0);
        } else if (has_next) {
          fence_proxy_async();
          issue_tile(Un.f0, Un.col0);
        }
      }
      // First transform.  Its radix-E stage runs in registers; only then does thread 0
      // wait until the previous field's result tile has been read out of `ex` (the
      // TMA store), and the first exchange's barrier publishes that to every thread.
      Dft<E>::run(v, 0);
      if (threadIdx.x == 0) bulk_wait_read_all();
      if constexpr (TWR)
        stages_from_r<N, E, 1, W>(v, t, wr, ex + c, 0, 0);
      else
        stages_from<N, E, 1, W>(v, t, tw, ex + c, 0, 0);
      fft_last_stage_order<E>(v);
      if (!a.fft_only) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          float2 hv = hs[(t + i * T) * W + c];
          hv.y *= hsign;
          // conj(X * H): the inverse transform runs as conj(FFT(conj(.)))
          v[i] = make_float2(fmaf(v[i].x, hv.x, -v[i].y * hv.y), -fmaf(v[i].x, hv.y, v[i].y * hv.x));
        }
        if (f + 1 == U.f1 && has_next) {
          __syncthreads();  // every thread has read this unit's H strip
          if (threadIdx.x == 0) {
            fence_proxy_async();
            issue_h(Un);
          }
        }
        fft(v);
      }
      const float osign = a.fft_only ? 1.f : -1.f;
      __syncthreads();  // the last stage has read `ex`
#pragma unroll
      for (int i = 0; i < E; ++i) ex[(t + i * T) * W + c] = make_float2(v[i].x, osign * v[i].y);
      fence_proxy_async();
      __syncthreads();
      if (threadIdx.x == 0 && !a.test_skip_copy) {
        const int fz = field_of(f);
        if (a.tile4d)
          tma_store_4d(&tm_buf, U.col0, 0, 0, fz, ex);
        else
          for (int k = 0; k < nbox_out; ++k) tma_store_3d(&tm_buf, U.col0, k * BOX, fz, ex + k * BOX * W);
        bulk_commit();
      }
    }
    if (!has_next) break;
    U = Un;
    uk += gridDim.x;
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

// --------------------------------------------------------------------------
// Launch helpers used by the per-size translation units.
// --------------------------------------------------------------------------
template <int N, int E, int LANES>
struct RowShape {
  static constexpr int threads = LANES * (N / E);
  // staging / exchange tiles, plus the modulation cache of the gradient passes
  static size_t smem(bool pf, bool grad) {
    return sizeof(float2) * ((size_t)(pf ? 2 : 1) * LANES * SmemSize<N>::value + (grad ? (size_t)LANES * N : 0));
  }
};

// Whether a pass over field_bytes of fields is launched with the programmatic-dependent-
// launch attribute (small passes; FO_PDL=1 / 0 force it for all).
bool pdl_for(long long field_bytes);

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pass(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                               cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <typename K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// staging: 0 none, 1 cp.async staging of the next field's row in shared memory (PF),
// 2 register prefetch of the next field's row (RP; passes without a gradient only,
// otherwise as 0)
template <int N, int E, int LANES>
cudaError_t row_launch_shape(const RowPassArgs& a, const float2* tw, cudaStream_t s, int staging) {
  using SH = RowShape<N, E, LANES>;
  dim3 grid((a.batch + a.fields_per_cta - 1) / a.fields_per_cta, (a.nrows + LANES - 1) / LANES);
  const bool pdl = pdl_for((long long)a.batch * a.nrows * N * (long long)sizeof(float2));
  const bool grad = a.mod_bwd && a.grad != nullptr && a.mod_kind != MOD_NONE;
  const bool sid = a.sid_partials != nullptr;  // GK 3 (no staging)
  const bool pf = staging == 1;
  const size_t smem = SH::smem(pf && !sid && !(grad && a.mod_kind == MOD_MASK), grad || sid);
  const bool full = a.n_valid == N && a.nrows % LANES == 0;
  cudaError_t e = cudaSuccess;
#define FO_ROW_GO(GK, PFV)                                                                        \
  do {                                                                                            \
    if (full) {                                                                                   \
      e = set_smem(row_pass_kernel<N, E, LANES, GK, PFV, true>, smem);                            \
      if (e == cudaSuccess) e = launch_pass(pdl, row_pass_kernel<N, E, LANES, GK, PFV, true>, grid, dim3(SH::threads), smem, s, a, tw); \
    } else {                                                                                      \
      e = set_smem(row_pass_kernel<N, E, LANES, GK, PFV, false>, smem);                           \
      if (e == cudaSuccess) e = launch_pass(pdl, row_pass_kernel<N, E, LANES, GK, PFV, false>, grid, dim3(SH::threads), smem, s, a, tw); \
    }                                                                                             \
  } while (0)
  if (a.sfd_rows) {
    // the exchange tiles and 32 floats of reduction scratch per row
    const size_t smem5 = SH::smem(false, false) + sizeof(float) * 32 * LANES;
    if (full) {
      e = set_smem(row_pass_kernel<N, E, LANES, 5, false, true>, smem5);
      if (e == cudaSuccess)
        e = launch_pass(pdl, row_pass_kernel<N, E, LANES, 5, false, true>, grid, dim3(SH::threads), smem5, s, a, tw);
    } else {
      e = set_smem(row_pass_kernel<N, E, LANES, 5, false, false>, smem5);
      if (e == cudaSuccess)
        e = launch_pass(pdl, row_pass_kernel<N, E, LANES, 5, false, false>, grid, dim3(SH::threads), smem5, s, a, tw);
    }
  } else if (sid && a.seed_dst) {
    FO_ROW_GO(4, false);
  } else if (sid) {
    FO_ROW_GO(3, false);
  } else if (!grad && staging == 2) {
    if (full) {
      e = set_smem(row_pass_kernel<N, E, LANES, 0, false, true, true>, smem);
      if (e == cudaSuccess)
        e = launch_pass(pdl, row_pass_kernel<N, E, LANES, 0, false, true, true>, grid, dim3(SH::threads), smem, s, a, tw);
    } else {
      e = set_smem(row_pass_kernel<N, E, LANES, 0, false, false, true>, smem);
      if (e == cudaSuccess)
        e = launch_pass(pdl, row_pass_kernel<N, E, LANES, 0, false, false, true>, grid, dim3(SH::threads), smem, s, a, tw);
    }
  } else if (!grad) {
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

// Column-pass shared memory: staging (1 or 2 padded tiles) plus, when it fits,
// the transfer-function tile.
template <int N, int W>
constexpr size_t col_smem(bool pf, bool hs) {
  return sizeof(float2) * ((size_t)(pf ? 2 : 1) * W * SmemSize<N>::value + (hs ? (size_t)N * W : 0));
}
constexpr size_t kMaxSmemPerCta = 227 * 1024;

template <int N, int E, int W, int P>
cudaError_t col_launch_shape(const ColPassArgs& a, const float2* tw, cudaStream_t s, bool pf) {
  constexpr int threads = (W / (P == 2 ? 2 : 1)) * (N / E);
  dim3 grid(a.n_items, (a.ncols + W - 1) / W);
  const bool pdl = pdl_for((long long)a.batch * a.ncols * N * (long long)sizeof(float2));
  const bool full = a.y_in == N && a.y_out == N && a.ncols % W == 0;
  cudaError_t e;
#define FO_COL_GO(PFV, HSV)                                                                     \
  do {                                                                                          \
    constexpr size_t smem = col_smem<N, W>(PFV, HSV);                                           \
    if constexpr (P == 2) {                                                                     \
      e = set_smem(col_pass2_kernel<N, E, W, PFV, HSV>, smem);                                  \
      if (e == cudaSuccess) e = launch_pass(pdl, col_pass2_kernel<N, E, W, PFV, HSV>, grid, dim3(threads), smem, s, a, tw); \
    } else if (full) {                                                                          \
      e = set_smem(col_pass_kernel<N, E, W, PFV, HSV, true>, smem);                             \
      if (e == cudaSuccess) e = launch_pass(pdl, col_pass_kernel<N, E, W, PFV, HSV, true>, grid, dim3(threads), smem, s, a, tw); \
    } else {                                                                                    \
      e = set_smem(col_pass_kernel<N, E, W, PFV, HSV, false>, smem);                            \
      if (e == cudaSuccess) e = launch_pass(pdl, col_pass_kernel<N, E, W, PFV, HSV, false>, grid, dim3(threads), smem, s, a, tw); \
    }                                                                                           \
  } while (0)
  if constexpr (P == 4 || P == 6) {
    constexpr bool TWR = (P == 6);
    constexpr size_t smem_t = 128 + sizeof(float2) * ((size_t)2 * N * W + (size_t)W * SmemSize<N>::value) + 16;
    static_assert(smem_t <= kMaxSmemPerCta, "TMA column variant does not fit");
    (void)pf;
    e = set_smem(col_tma_kernel<N, E, W, TWR>, smem_t);
    if (a.occupancy_out) {
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(a.occupancy_out, col_tma_kernel<N, E, W, TWR>, threads,
                                                          smem_t);
      return e;
    }
    if (!a.tmap_buf || !a.tmap_h) return cudaErrorInvalidValue;
    if (a.units) grid = dim3(a.persistent ? std::min(a.persistent, a.n_units) : a.n_units, 1);
    if (e == cudaSuccess)
      e = launch_pass(pdl, col_tma_kernel<N, E, W, TWR>, grid, dim3(threads), smem_t, s, a, tw,
                      *reinterpret_cast<const CUtensorMap*>(a.tmap_buf),
                      *reinterpret_cast<const CUtensorMap*>(a.tmap_h));
  } else if constexpr (P == 0) {
    constexpr int LS = LaneStride<N>::value;
    constexpr size_t smem_hs = sizeof(float2) * ((size_t)2 * W * LS + (size_t)W * (N + 4));
    constexpr size_t smem_nohs = sizeof(float2) * ((size_t)2 * W * LS);
    (void)pf;
    if constexpr (smem_hs <= kMaxSmemPerCta) {
      e = set_smem(col_lane_kernel<N, E, W, true>, smem_hs);
      if (e == cudaSuccess) e = launch_pass(pdl, col_lane_kernel<N, E, W, true>, grid, dim3(threads), smem_hs, s, a, tw);
    } else {
      e = set_smem(col_lane_kernel<N, E, W, false>, smem_nohs);
      if (e == cudaSuccess) e = launch_pass(pdl, col_lane_kernel<N, E, W, false>, grid, dim3(threads), smem_nohs, s, a, tw);
    }
  } else if (pf) {
    if constexpr (col_smem<N, W>(true, true) <= kMaxSmemPerCta) FO_COL_GO(true, true);
    else FO_COL_GO(true, false);
  } else {
    if constexpr (col_smem<N, W>(false, true) <= kMaxSmemPerCta) FO_COL_GO(false, true);
    else FO_COL_GO(false, false);
  }
#undef FO_COL_GO
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace fo
