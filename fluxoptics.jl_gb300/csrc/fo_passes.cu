// Row and column passes of the fused 2-D propagation pipeline.
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
#include "fo_fft.cuh"
#include "fo_internal.h"

namespace fo {

// --------------------------------------------------------------------------
// Per-size launch shapes.
// Row pass: ROWS rows per CTA, T = N/E threads per row.
// Column pass: W columns per CTA, T = N/E threads per column.
// --------------------------------------------------------------------------
template <int N>
struct RowCfg;
template <int N>
struct ColCfg;

#define FO_ROW_CFG(NN, EE, RR)                 \
  template <>                                  \
  struct RowCfg<NN> {                          \
    static constexpr int E = EE, ROWS = RR;    \
  };
#define FO_COL_CFG(NN, EE, WW)                 \
  template <>                                  \
  struct ColCfg<NN> {                          \
    static constexpr int E = EE, W = WW;       \
  };

FO_ROW_CFG(16, 4, 32)
FO_ROW_CFG(32, 4, 16)
FO_ROW_CFG(64, 8, 16)
FO_ROW_CFG(128, 8, 16)
FO_ROW_CFG(256, 16, 16)
FO_ROW_CFG(512, 8, 4)
FO_ROW_CFG(1024, 16, 4)
FO_ROW_CFG(2048, 16, 2)
FO_ROW_CFG(4096, 16, 1)

FO_COL_CFG(16, 4, 32)
FO_COL_CFG(32, 4, 16)
FO_COL_CFG(64, 8, 16)
FO_COL_CFG(128, 8, 16)
FO_COL_CFG(256, 16, 16)
FO_COL_CFG(512, 8, 8)
FO_COL_CFG(1024, 16, 8)
FO_COL_CFG(2048, 16, 4)
FO_COL_CFG(4096, 16, 4)

__device__ __forceinline__ float2 cis_f(float a) {
  float s, c;
  sincosf(a, &s, &c);
  return make_float2(c, s);
}

// --------------------------------------------------------------------------
// Row pass
// --------------------------------------------------------------------------
// GK selects the gradient accumulator: 0 none, 1 real (phase, dn), 2 complex (mask).
template <int N, int GK>
__global__ void __launch_bounds__(RowCfg<N>::ROWS*(N / RowCfg<N>::E))
    row_pass_kernel(const RowPassArgs a, const float2* __restrict__ tw) {
  constexpr int E = RowCfg<N>::E;
  constexpr int ROWS = RowCfg<N>::ROWS;
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  __shared__ float2 smem[ROWS * SLOTS];

  const int t = threadIdx.x % T;
  const int lane = threadIdx.x / T;
  const int y = blockIdx.y * ROWS + lane;
  const bool row_ok = y < a.nrows;
  float2* sm = smem + lane * SLOTS;

  const int load_n = a.inv_first ? N : a.n_valid;
  const int store_n = a.fwd_after ? N : a.n_valid;
  constexpr bool is_grad = GK != 0;
  constexpr int GR = (GK == 1) ? E : 1;
  constexpr int GC = (GK == 2) ? E : 1;
  float gacc[GR];
  float2 gacc_c[GC];
#pragma unroll
  for (int i = 0; i < GR; ++i) gacc[i] = 0.f;
#pragma unroll
  for (int i = 0; i < GC; ++i) gacc_c[i] = make_float2(0.f, 0.f);

  const int f0 = blockIdx.x * a.fields_per_cta;
  const int f1 = min(a.batch, f0 + a.fields_per_cta);
  for (int f = f0; f < f1; ++f) {
    const int b = a.field_list ? a.field_list[f] : f;
    const float2* src = a.src + (long long)b * a.src_bstride + (long long)y * a.src_ld;
    float2 v[E];
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int p = t + i * T;
      float2 x = make_float2(0.f, 0.f);
      if (row_ok && p < load_n) x = src[p];
      v[i] = a.inv_first ? cconj(x) : x;
    }
    if (a.inv_first) {
      fft_forward<N, E, 1>(v, t, tw, sm);
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
      const float s = a.mod_sign;
      const float fb = (a.mod_kind == MOD_DN) ? a.mod_scale * a.inv_lambda[b] : 1.f;
      if (!a.mod_bwd) {
        if (a.save) {
          float2* sv = a.save + (long long)b * a.save_bstride + (long long)y * a.save_ld;
#pragma unroll
          for (int i = 0; i < E; ++i) {
            const int p = t + i * T;
            if (p < a.n_valid) sv[p] = v[i];
          }
        }
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (p < a.n_valid) {
            const long long q = (long long)y * a.param_ld + p;
            if (a.mod_kind == MOD_MASK) {
              float2 m = reinterpret_cast<const float2*>(a.mod_param)[q];
              if (s < 0.f) m = cconj(m);
              v[i] = cmul(v[i], m);
            } else {
              const float ph = reinterpret_cast<const float*>(a.mod_param)[q];
              v[i] = cmul(v[i], cis_f(s * fb * ph));
            }
          }
        }
      } else {
        const float2* sv = a.saved ? a.saved + (long long)b * a.saved_bstride + (long long)y * a.saved_ld
                                   : nullptr;
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int p = t + i * T;
          if (p < a.n_valid) {
            const long long q = (long long)y * a.param_ld + p;
            if (a.mod_kind == MOD_MASK) {
              if constexpr (GK == 2) {
                float2 g = cmul(v[i], cconj(sv[p]));
                if (s < 0.f) g = cconj(g);
                gacc_c[i] = cadd(gacc_c[i], g);
              }
              float2 m = reinterpret_cast<const float2*>(a.mod_param)[q];
              if (s > 0.f) m = cconj(m);
              v[i] = cmul(v[i], m);
            } else {
              const float ph = reinterpret_cast<const float*>(a.mod_param)[q];
              v[i] = cmul(v[i], cis_f(-s * fb * ph));
              if constexpr (GK == 1) {
                const float2 u = sv[p];
                // Im(du * conj(u))
                const float im = v[i].y * u.x - v[i].x * u.y;
                gacc[i] = fmaf(s * fb, im, gacc[i]);
              }
            }
          }
        }
      }
    }
    if (a.fwd_after) {
      fft_forward<N, E, 1>(v, t, tw, sm);
    }
    if (row_ok) {
      float2* dst = a.dst + (long long)b * a.dst_bstride + (long long)y * a.dst_ld;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < store_n) dst[p] = v[i];
      }
    }
  }
  if (is_grad && row_ok) {
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int p = t + i * T;
      if (p < a.n_valid) {
        const long long q = (long long)y * a.param_ld + p;
        if constexpr (GK == 2)
          reinterpret_cast<float2*>(a.grad)[q] = gacc_c[i];
        else if constexpr (GK == 1)
          reinterpret_cast<float*>(a.grad)[q] = gacc[i];
      }
    }
  }
}

// --------------------------------------------------------------------------
// Column pass
// --------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(ColCfg<N>::W*(N / ColCfg<N>::E))
    col_pass_kernel(const ColPassArgs a, const float2* __restrict__ tw) {
  constexpr int E = ColCfg<N>::E;
  constexpr int W = ColCfg<N>::W;
  constexpr int T = N / E;
  constexpr int SLOTS = SmemSize<N>::value;
  extern __shared__ float2 smem_dyn[];

  const int c = threadIdx.x % W;
  const int t = threadIdx.x / W;
  const int col = blockIdx.y * W + c;
  const bool col_ok = col < a.ncols;
  const int f = blockIdx.x;
  const int b = a.field_list ? a.field_list[f] : f;
  float2* buf = a.buf + (long long)b * a.bstride + col;
  const float2* H = a.fft_only ? nullptr : a.H + (long long)a.h_index[b] * a.h_stride + col;
  (void)SLOTS;

  float2 v[E];
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int p = t + i * T;
    v[i] = (col_ok && p < a.y_in) ? buf[(long long)p * a.ld] : make_float2(0.f, 0.f);
  }
  fft_forward<N, E, W>(v, t, tw, smem_dyn + c);
  if (a.fft_only) {
    if (col_ok) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int p = t + i * T;
        if (p < a.y_out) buf[(long long)p * a.ld] = v[i];
      }
    }
    return;
  }
  // spectrum at ky = p: v <- conj(H * X) (inverse via conj-FFT-conj; H carries 1/(Nx*Ny))
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int p = t + i * T;
    float2 h = col_ok ? __ldg(H + (long long)p * a.ncols) : make_float2(0.f, 0.f);
    if (a.conj_h) h = cconj(h);
    v[i] = cconj(cmul(v[i], h));
  }
  fft_forward<N, E, W>(v, t, tw, smem_dyn + c);
  if (col_ok) {
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int p = t + i * T;
      if (p < a.y_out) buf[(long long)p * a.ld] = cconj(v[i]);
    }
  }
}

// --------------------------------------------------------------------------
// Launchers
// --------------------------------------------------------------------------
bool fft_size_supported(int n) {
  switch (n) {
    case 16: case 32: case 64: case 128: case 256: case 512: case 1024: case 2048: case 4096:
      return true;
    default:
      return false;
  }
}

int row_pass_rows_per_cta(int N) {
  switch (N) {
#define FO_CASE(NN) case NN: return RowCfg<NN>::ROWS;
    FO_CASE(16) FO_CASE(32) FO_CASE(64) FO_CASE(128) FO_CASE(256) FO_CASE(512) FO_CASE(1024)
    FO_CASE(2048) FO_CASE(4096)
#undef FO_CASE
    default: return 0;
  }
}

template <int N>
static cudaError_t row_launch(const RowPassArgs& a, const float2* tw, cudaStream_t s) {
  constexpr int ROWS = RowCfg<N>::ROWS;
  constexpr int threads = ROWS * (N / RowCfg<N>::E);
  // fields vary fastest across the grid: CTAs that run together share the rows of
  // the modulation parameters, which then stay in L2
  dim3 grid((a.batch + a.fields_per_cta - 1) / a.fields_per_cta, (a.nrows + ROWS - 1) / ROWS);
  const bool grad = a.mod_bwd && a.grad != nullptr && a.mod_kind != MOD_NONE;
  if (!grad)
    row_pass_kernel<N, 0><<<grid, threads, 0, s>>>(a, tw);
  else if (a.mod_kind == MOD_MASK)
    row_pass_kernel<N, 2><<<grid, threads, 0, s>>>(a, tw);
  else
    row_pass_kernel<N, 1><<<grid, threads, 0, s>>>(a, tw);
  return cudaGetLastError();
}

template <int N>
static cudaError_t col_launch(const ColPassArgs& a, const float2* tw, cudaStream_t s) {
  constexpr int W = ColCfg<N>::W;
  constexpr int threads = W * (N / ColCfg<N>::E);
  constexpr size_t smem = sizeof(float2) * (size_t)W * SmemSize<N>::value;
  static bool configured = false;  // per process; the attribute is per function
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(col_pass_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  // fields (sorted by wavelength) vary fastest: the CTAs of one column tile run
  // together and read the tile of their transfer function from L2
  dim3 grid(a.batch, (a.ncols + W - 1) / W);
  col_pass_kernel<N><<<grid, threads, smem, s>>>(a, tw);
  return cudaGetLastError();
}

cudaError_t launch_row_pass(int N, const RowPassArgs& a, const float2* tw, cudaStream_t s) {
  switch (N) {
#define FO_CASE(NN) case NN: return row_launch<NN>(a, tw, s);
    FO_CASE(16) FO_CASE(32) FO_CASE(64) FO_CASE(128) FO_CASE(256) FO_CASE(512) FO_CASE(1024)
    FO_CASE(2048) FO_CASE(4096)
#undef FO_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_col_pass(int N, const ColPassArgs& a, const float2* tw, cudaStream_t s) {
  switch (N) {
#define FO_CASE(NN) case NN: return col_launch<NN>(a, tw, s);
    FO_CASE(16) FO_CASE(32) FO_CASE(64) FO_CASE(128) FO_CASE(256) FO_CASE(512) FO_CASE(1024)
    FO_CASE(2048) FO_CASE(4096)
#undef FO_CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fo
