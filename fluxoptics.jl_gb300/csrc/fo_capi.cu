// C ABI of libfluxoptics_gb300: plans, the fused chain engine, AS_BPM with
// checkpointed adjoint, the metric and the optimiser entry points.
#include <math.h>

#include <cmath>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <tuple>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fluxoptics_gb300.h"
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fo_aux.h"
#include "fo_fft.cuh"
#include "fo_internal.h"
#include "fo_units.h"

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
namespace fo {

static thread_local std::string g_last_error;

void set_error(int code, const std::string& msg) {
  (void)code;
  g_last_error = msg;
}

int fail(int code, const std::string& msg) {
  set_error(code, msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(FO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

// ---------------------------------------------------------------------------
// Stage-major twiddle tables of the (N, E) schedule, one per (device, N, E),
// built in FP64 and rounded once to float.
// ---------------------------------------------------------------------------
static std::mutex g_tw_mu;
static std::map<std::tuple<int, int, int>, float2*> g_tw;

const float2* twiddles(int N, int E, int* err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *err = cuda_fail(e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto it = g_tw.find({dev, N, E});
  if (it != g_tw.end()) return it->second;
  const int n = std::max(1, stage_twiddle_count(N, E));
  std::vector<float2> h(n, make_float2(1.f, 0.f));
  for_each_stage_twiddle(N, E, [&](int idx, long long num, long long den) {
    const long long m = num % den;  // exact reduction of the angle
    const double a = -2.0 * M_PI * (double)m / (double)den;
    h[idx] = make_float2((float)cos(a), (float)sin(a));
  });
  float2* d = nullptr;
  e = cudaMalloc(&d, sizeof(float2) * n);
  if (e != cudaSuccess) {
    *err = fail(FO_ERR_ALLOC, "cudaMalloc twiddles failed");
    return nullptr;
  }
  e = cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    *err = cuda_fail(e, "cudaMemcpy twiddles");
    return nullptr;
  }
  g_tw[{dev, N, E}] = d;
  return d;
}

// ---------------------------------------------------------------------------
// Device error word (one per device): kernels with bounded waits set bit 0 when
// a wait gives up; fo_device_status reads and clears it.
// ---------------------------------------------------------------------------
static std::mutex g_err_mu;
static std::map<int, unsigned int*> g_err_words;

unsigned int* device_error_word(int* err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *err = cuda_fail(e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_err_mu);
  auto it = g_err_words.find(dev);
  if (it != g_err_words.end()) return it->second;
  unsigned int* w = nullptr;
  e = cudaMalloc(&w, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(w, 0, sizeof(unsigned int));
  if (e != cudaSuccess) {
    *err = cuda_fail(e, "device error word");
    return nullptr;
  }
  g_err_words[dev] = w;
  return w;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder(int* err) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!fn) *err = fail(FO_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  return fn;
}

int encode_tmap_2d(void* tmap, const void* base, long long rows, int cols, int ld, int box_cols, int box_rows) {
  int err = FO_OK;
  auto fn = tmap_encoder(&err);
  if (!fn) return err;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(FO_ERR_ARG, "TMA base address not 16-byte aligned");
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float2)};
  const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(reinterpret_cast<CUtensorMap*>(tmap), CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void*>(base),
                  dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(FO_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return FO_OK;
}

int encode_tmap_4d(void* tmap, const void* base, int fields, int rows, int cols, int ld, int box_cols) {
  int err = FO_OK;
  auto fn = tmap_encoder(&err);
  if (!fn) return err;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(FO_ERR_ARG, "TMA base address not 16-byte aligned");
  if (rows % 256 != 0 || rows / 256 > 256) return fail(FO_ERR_ARG, "4-D tile view needs rows = 256 k, k <= 256");
  const cuuint64_t dims[4] = {(cuuint64_t)cols, 256, (cuuint64_t)(rows / 256), (cuuint64_t)fields};
  const cuuint64_t row = (cuuint64_t)ld * sizeof(float2);
  const cuuint64_t strides[3] = {row, row * 256, row * rows};
  const cuuint32_t box[4] = {(cuuint32_t)box_cols, 256, (cuuint32_t)(rows / 256), 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(reinterpret_cast<CUtensorMap*>(tmap), CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<void*>(base),
                  dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(FO_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return FO_OK;
}

int encode_tmap_3d(void* tmap, const void* base, int fields, int rows, int cols, int ld, int box_cols, int box_rows) {
  int err = FO_OK;
  auto fn = tmap_encoder(&err);
  if (!fn) return err;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(FO_ERR_ARG, "TMA base address not 16-byte aligned");
  const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)fields};
  const cuuint64_t strides[2] = {(cuuint64_t)ld * sizeof(float2), (cuuint64_t)ld * rows * sizeof(float2)};
  const cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(reinterpret_cast<CUtensorMap*>(tmap), CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(base),
                  dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(FO_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return FO_OK;
}

}  // namespace fo

using namespace fo;

// ---------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------
namespace {

int next_pow2(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return (v && *v) ? atoi(v) : dflt;
}

int check_dir(int d) {
  if (d != FO_FORWARD && d != FO_BACKWARD) return fail(FO_ERR_ARG, "direction must be FO_FORWARD (1) or FO_BACKWARD (-1)");
  return FO_OK;
}

template <typename T>
int dalloc(T** p, size_t count, const char* what) {
  *p = nullptr;
  if (count == 0) return FO_OK;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(FO_ERR_ALLOC, std::string("cudaMalloc failed for ") + what + " (" +
                                  std::to_string(sizeof(T) * count) + " bytes)");
  }
  return FO_OK;
}

#define FO_TRY(expr)             \
  do {                           \
    int _rc = (expr);            \
    if (_rc != FO_OK) return _rc; \
  } while (0)

#define FO_LAUNCH(expr)                                   \
  do {                                                    \
    cudaError_t _e = (expr);                              \
    if (_e != cudaSuccess) return cuda_fail(_e, #expr);   \
  } while (0)

}  // namespace

// ---------------------------------------------------------------------------
// Propagator plans
// ---------------------------------------------------------------------------
struct fo_prop_plan_s {
  int kind = 0;  // 0 AS, 1 RS
  int nx = 0, ny = 0, batch = 0;
  int fx = 0, fy = 0;  // transform sizes
  double dx = 0, dy = 0, z = 0, n0 = 1;
  std::vector<double> lambdas;  // per field
  float2* spec_a = nullptr;      // gradient calls (Fourier modulators, ASPropZ): spectra
  float2* spec_b = nullptr;
  int h_mode = 0;                   // 0 on axis, 1 tilted, 2 paraxial
  std::vector<double> table_lambda; // wavelength of each transfer-function table
  double* zgrad_partials = nullptr; // ASPropZ gradient: block partial sums
  float4* zpar = nullptr;           // ASPropZ gradient: per field {n0 / lambda, f0x, f0y, lambda / n0}
  std::vector<std::array<double, 2>> table_theta;  // tilts of each table (tilted / paraxial kernels)
  int track = 0;                    // track_tilts of the tilted / paraxial kernels
  bool has_filter = false;          // the tables carry a frequency filter
  double2* filters = nullptr;       // n_tables x fy x fx filter values, kept for fo_prop_set_z
  int n_tables = 0;
  float2* H = nullptr;          // n_tables x fy x fx, scaled by 1/(fx*fy)
  int* h_index = nullptr;       // device, per field
  int* sorted_fields = nullptr; // device, fields ordered by transfer-function table
  int* items = nullptr;         // device, n_items+1 offsets into sorted_fields (runs of one table)
  int n_items = 0;
  std::vector<int> items_host;  // the same offsets on the host
  int4* units = nullptr;        // device, balanced column work units of the TMA variants (or null)
  int n_units = 0;
  int col_ctas = 0;             // persistent column launch: CTAs taking every col_ctas-th unit (0: off)
  int row_v = 0, col_v = 0;     // launch-shape variants (autotuned or default)
  int row_pf = 1;                // row staging: 0 none, 1 cp.async, 2 register prefetch
  bool col_pf = true;
  unsigned int* err_word = nullptr;         // device error word (bounded waits)
  unsigned long long wait_ns = 1000000000ull;  // limit of a bounded device wait
  float* inv_lambda = nullptr;  // device, per field
  const float2* tw_x = nullptr;
  const float2* tw_y = nullptr;
  float2* scratch = nullptr;    // RS: batch x ny x fx
  size_t ws_bytes = 0;
};

struct fo_sid_s {
  int nx = 0, ny = 0, batch = 0, T = 0;
  int group = 0;           // fields per target slice when every slice has the same count, else 0
  int* tidx = nullptr;     // device, per field
  int* order = nullptr;    // device, fields grouped by target slice
  int* offsets = nullptr;  // device, T+1
  float* resid = nullptr;  // device, T x ny x nx
  float* partials = nullptr;  // device, max(pixel blocks, ny) x T
  float* ones = nullptr;   // device, T
};

namespace {

void plan_free(fo_prop_plan p) {
  if (!p) return;
  cudaFree(p->H);
  cudaFree(p->h_index);
  cudaFree(p->sorted_fields);
  cudaFree(p->units);
  cudaFree(p->items);
  cudaFree(p->inv_lambda);
  cudaFree(p->scratch);
  cudaFree(p->spec_a);
  cudaFree(p->spec_b);
  cudaFree(p->zgrad_partials);
  cudaFree(p->zpar);
  cudaFree(p->filters);
  delete p;
}

struct Layout {
  int nx, ny, batch, fx, fy;
  bool padded;
  int row_v;
  int row_pf;
};

Layout layout_of(const fo_prop_plan_s* p) {
  return Layout{p->nx, p->ny, p->batch, p->fx, p->fy, p->kind == 1, p->row_v, p->row_pf};
}

bool same_layout(const Layout& a, const Layout& b) {
  return a.nx == b.nx && a.ny == b.ny && a.batch == b.batch && a.fx == b.fx && a.fy == b.fy &&
         a.padded == b.padded;
}

// Optional per-pass timing of eager calls: CUDA events around every pass launch,
// summed per pass kind (0 single row transform, 1 fused inverse+forward row
// pass, 2 column pass) by fo_profile_end.
struct ProfRec {
  int kind;
  cudaEvent_t a, b;
};
bool g_prof = false;
std::vector<ProfRec> g_prof_recs;

struct ProfScope {
  int kind;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(int k, cudaStream_t s) : kind(k), st(s) {
    if (!g_prof) return;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, st);
  }
  ~ProfScope() {
    if (!a) return;
    cudaEventRecord(b, st);
    g_prof_recs.push_back({kind, a, b});
  }
};

// Internal modulation description.
struct Mod {
  int kind = MOD_NONE;
  const void* param = nullptr;
  void* saved = nullptr;
  void* grad = nullptr;
  float scale = 1.f;
  const float4* field_coef = nullptr;
};

Mod mod_from(const fo_mod* m) {
  Mod r;
  if (!m) return r;
  r.kind = m->kind;
  r.param = m->param;
  r.saved = m->saved;
  r.grad = m->grad;
  r.scale = (float)m->scale;
  r.field_coef = reinterpret_cast<const float4*>(m->field_coef);
  return r;
}


struct SeedArgs {
  const float* resid = nullptr;
  const int* tidx = nullptr;
  const float* dc = nullptr;
};

int validate_mod(const Mod& m, bool backward) {
  if (m.kind < MOD_NONE || m.kind > MOD_TEA) return fail(FO_ERR_ARG, "unknown modulation kind");
  if (m.kind != MOD_NONE && !m.param) return fail(FO_ERR_ARG, "modulation parameter pointer is NULL");
  if (m.kind == MOD_TEA && !m.field_coef) return fail(FO_ERR_ARG, "FO_MOD_TEA needs field_coef");
  if (m.kind == MOD_TEA && (reinterpret_cast<uintptr_t>(m.field_coef) & 15) != 0)
    return fail(FO_ERR_ARG, "field_coef must be 16-byte aligned");
  if (backward && m.kind != MOD_NONE && m.grad && !m.saved)
    return fail(FO_ERR_ARG, "a gradient needs the saved forward input");
  return FO_OK;
}

// Fields a CTA of a row pass without a gradient loops over (the gradient passes take
// the whole batch): the per-pixel modulation factor is computed once per CTA.  The
// batch is cut into the fewest equal groups of at most FO_ROW_FIELDS fields (default
// 24): at 2048^2 x 48 fields, two groups of 24 measured 10.46 ms per iteration
// against 10.51 ms for three of 16, 10.59 ms for 32 + 16 and 10.50 ms for one of 48.
int row_fields_per_cta(int batch) {
  static const int cap = std::max(1, std::min(64, env_int("FO_ROW_FIELDS", 24)));
  if (batch <= cap) return std::max(1, batch);
  const int groups = (batch + cap - 1) / cap;
  return (batch + groups - 1) / groups;
}

// One row pass.  `src`/`dst` are real-space (ld nx) or spectral (ld fx) arrays as
// selected by the inv/fwd flags.
int row_pass(const Layout& L, const float2* src, float2* dst, bool inv_first, bool fwd_after,
             const Mod& mod, bool bwd, float s, const float* inv_lambda, const SeedArgs* seed,
             const float2* tw, cudaStream_t st, const fo_sid_s* sid = nullptr, const float* target = nullptr,
             float2* probe_pre = nullptr, float2* probe_post = nullptr) {
  RowPassArgs a;
  std::memset(&a, 0, sizeof(a));
  const long long real_bs = (long long)L.nx * L.ny, spec_bs = (long long)L.fx * L.ny;
  a.src = src;
  a.dst = dst;
  a.src_bstride = inv_first ? spec_bs : real_bs;
  a.src_ld = inv_first ? L.fx : L.nx;
  a.dst_bstride = fwd_after ? spec_bs : real_bs;
  a.dst_ld = fwd_after ? L.fx : L.nx;
  a.nrows = L.ny;
  a.n_valid = L.nx;
  a.batch = L.batch;
  const bool grad = bwd && mod.kind != MOD_NONE && mod.grad != nullptr;
  a.fields_per_cta = grad ? L.batch : row_fields_per_cta(L.batch);
  a.field_list = nullptr;
  a.inv_first = inv_first;
  a.fwd_after = fwd_after;
  a.mod_kind = mod.kind;
  a.mod_bwd = bwd;
  a.mod_sign = s;
  a.mod_param = mod.param;
  a.param_ld = L.nx;
  a.mod_scale = mod.scale;
  a.inv_lambda = inv_lambda;
  a.field_coef = mod.field_coef;
  if (!bwd) {
    a.save = reinterpret_cast<float2*>(mod.saved);
    a.save_bstride = real_bs;
    a.save_ld = L.nx;
    a.probe_pre = probe_pre;
    a.probe_post = probe_post;
  } else {
    a.saved = reinterpret_cast<const float2*>(mod.saved);
    a.saved_bstride = real_bs;
    a.saved_ld = L.nx;
    a.grad = mod.grad;
  }
  if (seed) {
    a.seed = 1;
    a.resid = seed->resid;
    a.resid_tstride = real_bs;
    a.resid_ld = L.nx;
    a.tidx = seed->tidx;
    a.dc = seed->dc;
  }
  if (sid) {  // the metric on this pass's output: one CTA per (target slice, rows)
    a.field_list = sid->order;
    a.fields_per_cta = sid->group;
    a.tidx = sid->tidx;
    a.resid_tstride = real_bs;
    a.resid_ld = L.nx;
    a.sid_target = target;
    a.sid_resid = sid->resid;
    a.sid_partials = sid->partials;
    a.sid_T = sid->T;
  }
  const int load_n = inv_first ? L.fx : L.nx;
  int staging = L.row_pf;
  if (staging == 1 && !(load_n == L.fx && row_prefetch_fits(L.fx, L.row_v) && !(grad && mod.kind == MOD_MASK) && !sid))
    staging = 0;
  ProfScope prof(inv_first && fwd_after ? 1 : 0, st);
  FO_LAUNCH(launch_row_pass(L.fx, L.row_v, staging, a, tw, st));
  return FO_OK;
}

int col_pass(const fo_prop_plan_s* p, float2* buf, bool conj_h, cudaStream_t st) {
  ColPassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.buf = buf;
  a.bstride = (long long)p->fx * p->ny;
  a.ld = p->fx;
  a.ncols = p->fx;
  a.y_in = p->ny;
  a.y_out = p->ny;
  a.H = p->H;
  a.h_stride = (long long)p->fx * p->fy;
  a.h_index = p->h_index;
  a.conj_h = conj_h;
  a.fft_only = 0;
  a.batch = p->batch;
  a.field_list = p->sorted_fields;
  a.units = p->units;
  a.n_units = p->n_units;
  a.persistent = p->col_ctas;
  a.item_start = p->items;
  a.n_items = p->n_items;
  int v = p->col_v;
  const float2* tw = p->tw_y;
  alignas(64) CUtensorMap tm_buf, tm_h;
  if (col_variant_uses_tma(p->fy, v)) {
    const int W = col_variant(p->fy, v).lanes;
    // whole tiles in one TMA instruction when the field height is a multiple of 256
    const bool t4 = p->ny % 256 == 0 && p->fy % 256 == 0 && env_int("FO_TILE4D", 1) != 0;
    int rc = t4 ? encode_tmap_4d(&tm_buf, buf, p->batch, p->ny, p->fx, p->fx, W)
                : encode_tmap_3d(&tm_buf, buf, p->batch, p->ny, p->fx, p->fx, W, 256);
    if (rc == FO_OK)
      rc = t4 ? encode_tmap_4d(&tm_h, p->H, p->n_tables, p->fy, p->fx, p->fx, W)
              : encode_tmap_2d(&tm_h, p->H, (long long)p->n_tables * p->fy, p->fx, p->fx, W, 256);
    a.tile4d = t4 ? 1 : 0;
    if (rc != FO_OK) {  // e.g. an unaligned caller buffer: use the cp.async variant
      v = 0;
      int trc = FO_OK;
      tw = twiddles(p->fy, col_variant(p->fy, 0).E, &trc);
      if (!tw) return trc;
    } else {
      a.tmap_buf = &tm_buf;
      a.tmap_h = &tm_h;
      a.err_word = p->err_word;
      a.wait_ns = p->wait_ns;
      a.test_skip_copy = env_int("FO_TEST_SKIP_COPY", 0);
    }
  }
  const bool pf = p->col_pf && col_prefetch_fits(p->fy, v);
  ProfScope prof(2, st);
  FO_LAUNCH(launch_col_pass(p->fy, v, pf, a, tw, st));
  return FO_OK;
}

// Forward sweep: mods[0] -> props[0] -> ... -> props[K-1] -> mods[K], in place on u.
// Forward sweep.  With `sid` (fused form only: every target slice has the same
// number of fields) the last pass also evaluates the metric on u against `target`
// and loss[T] receives the per-slice sums.
// With `probes`, probes[0][k] / probes[1][k] (k = 0..K, NULL entries skipped) receive the
// field before / after modulation slot k from the row pass that applies it.
int run_forward(const std::vector<fo_prop_plan>& props, float2* buf, float2* u, const Mod* mods, int s,
                cudaStream_t st, const float2* src = nullptr, const fo_sid_s* sid = nullptr,
                const float* target = nullptr, float* loss = nullptr,
                const std::vector<float2*>* probes = nullptr) {
  const int K = (int)props.size();
  const Layout L = layout_of(props[0]);
  const float* il = props[0]->inv_lambda;
  const float sf = (float)s;
  auto pre = [&](int k) { return probes ? probes[0][k] : nullptr; };
  auto post = [&](int k) { return probes ? probes[1][k] : nullptr; };
  FO_TRY(row_pass(L, src ? src : u, buf, false, true, mods[0], false, sf, il, nullptr, props[0]->tw_x, st, nullptr,
                  nullptr, pre(0), post(0)));
  for (int k = 0; k < K; ++k) {
    FO_TRY(col_pass(props[k], buf, s < 0, st));
    if (k + 1 < K)
      FO_TRY(row_pass(L, buf, buf, true, true, mods[k + 1], false, sf, il, nullptr, props[0]->tw_x, st, nullptr,
                      nullptr, pre(k + 1), post(k + 1)));
    else
      FO_TRY(row_pass(L, buf, u, true, false, mods[K], false, sf, il, nullptr, props[0]->tw_x, st, sid, target,
                      pre(K), post(K)));
  }
  if (sid) FO_LAUNCH(launch_sid_finalize(sid->partials, L.ny, sid->T, loss, st));
  return FO_OK;
}

// The chain's last forward row pass, the metric and the adjoint sweep's first row pass
// as one launch (row kernel GK = 4): the spectrum `spec` (after the last column pass)
// is inverse-transformed along x, the metric's residuals and row partials are formed,
// `u_out` (nullable) receives the output field, and the seeded adjoint spectrum
// replaces `spec` field by field.  No modulation: the chain's last slot is empty.
int row_pass_sid_seed(const Layout& L, float2* spec, float2* u_out, const fo_sid_s* sid, const float* target,
                      const float2* tw, cudaStream_t st) {
  RowPassArgs a;
  std::memset(&a, 0, sizeof(a));
  const long long real_bs = (long long)L.nx * L.ny, spec_bs = (long long)L.fx * L.ny;
  a.src = spec;
  a.src_bstride = spec_bs;
  a.src_ld = L.fx;
  a.dst = u_out;
  a.dst_bstride = real_bs;
  a.dst_ld = L.nx;
  a.nrows = L.ny;
  a.n_valid = L.nx;
  a.batch = L.batch;
  a.inv_first = 1;
  a.fwd_after = 0;
  a.mod_kind = MOD_NONE;
  a.field_list = sid->order;
  a.fields_per_cta = sid->group;
  a.tidx = sid->tidx;
  a.dc = sid->ones;
  a.resid_tstride = real_bs;
  a.resid_ld = L.nx;
  a.sid_target = target;
  a.sid_resid = sid->resid;
  a.sid_partials = sid->partials;
  a.sid_T = sid->T;
  a.seed_dst = spec;
  a.seed_bstride = spec_bs;
  a.seed_ld = L.fx;
  ProfScope prof(1, st);
  FO_LAUNCH(launch_row_pass(L.fx, L.row_v, 0, a, tw, st));
  return FO_OK;
}

// The chain's last forward row pass, SquaredFieldDifference against `v` and the adjoint
// sweep's first row pass as one launch (row kernel GK = 5), in place on the spectrum
// `spec`; the per-row sums go to sfd->rows and `c` receives the per-field values.
int row_pass_sfd_seed(const Layout& L, float2* spec, float2* u_out, const fo_sfd_s* sfd, const float2* v,
                      const float* dc, float* c, const float2* tw, cudaStream_t st) {
  RowPassArgs a;
  std::memset(&a, 0, sizeof(a));
  const long long real_bs = (long long)L.nx * L.ny, spec_bs = (long long)L.fx * L.ny;
  a.src = spec;
  a.src_bstride = spec_bs;
  a.src_ld = L.fx;
  a.dst = u_out;
  a.dst_bstride = real_bs;
  a.dst_ld = L.nx;
  a.nrows = L.ny;
  a.n_valid = L.nx;
  a.batch = L.batch;
  a.inv_first = 1;
  a.fwd_after = 0;
  a.mod_kind = MOD_NONE;
  a.fields_per_cta = row_fields_per_cta(L.batch);
  a.seed_dst = spec;
  a.seed_bstride = spec_bs;
  a.seed_ld = L.fx;
  a.sfd_v = v;
  a.sfd_rows = sfd->rows;
  a.sfd_dc = dc;
  ProfScope prof(1, st);
  FO_LAUNCH(launch_row_pass(L.fx, L.row_v, 0, a, tw, st));
  FO_LAUNCH(launch_sid_finalize(sfd->rows, L.ny, L.batch, c, st));
  return FO_OK;
}

// Forward sweep, metric and seeded adjoint sweep in one sequence of passes on the
// working buffer `w` (the chain scratch for padded layouts, else du): 2K + 1 forward
// passes and 2K + 1 adjoint passes share one row pass, `shared_pass(w)`, which ends the
// forward sweep with the metric and starts the adjoint sweep with its seed.  mods_f /
// mods_b are the forward and adjoint descriptions of the K + 1 slots; the last slot
// must be empty.
template <typename SharedPass>
int run_withgradient(const std::vector<fo_prop_plan>& props, float2* w, const float2* u_in, float2* du,
                     const Mod* mods_f, const Mod* mods_b, int s, cudaStream_t st, bool discard_input_grad,
                     SharedPass&& shared_pass) {
  const int K = (int)props.size();
  const Layout L = layout_of(props[0]);
  const float* il = props[0]->inv_lambda;
  const float sf = (float)s;
  const float2* tw = props[0]->tw_x;
  FO_TRY(row_pass(L, u_in, w, false, true, mods_f[0], false, sf, il, nullptr, tw, st));
  for (int k = 0; k < K; ++k) {
    FO_TRY(col_pass(props[k], w, s < 0, st));
    if (k + 1 < K) FO_TRY(row_pass(L, w, w, true, true, mods_f[k + 1], false, sf, il, nullptr, tw, st));
  }
  FO_TRY(shared_pass(L, tw));
  for (int k = K - 1; k >= 0; --k) {
    FO_TRY(col_pass(props[k], w, s > 0, st));
    if (k > 0)
      FO_TRY(row_pass(L, w, w, true, true, mods_b[k], true, sf, il, nullptr, tw, st));
    else
      FO_TRY(row_pass(L, w, discard_input_grad ? nullptr : du, true, false, mods_b[0], true, sf, il, nullptr, tw,
                      st));
  }
  return FO_OK;
}

// Adjoint sweep in reverse order, in place on du (src0 is du, or the forward
// output when the sweep is seeded by the metric).
int run_backward(const std::vector<fo_prop_plan>& props, float2* buf, float2* du, const float2* src0,
                 const Mod* mods, int s, const SeedArgs* seed, cudaStream_t st, bool discard_input_grad = false) {
  const int K = (int)props.size();
  const Layout L = layout_of(props[0]);
  const float* il = props[0]->inv_lambda;
  const float sf = (float)s;
  FO_TRY(row_pass(L, src0, buf, false, true, mods[K], true, sf, il, seed, props[0]->tw_x, st));
  for (int k = K - 1; k >= 0; --k) {
    FO_TRY(col_pass(props[k], buf, s > 0, st));
    if (k > 0)
      FO_TRY(row_pass(L, buf, buf, true, true, mods[k], true, sf, il, nullptr, props[0]->tw_x, st));
    else
      FO_TRY(row_pass(L, buf, discard_input_grad ? nullptr : du, true, false, mods[0], true, sf, il, nullptr,
                      props[0]->tw_x, st));
  }
  return FO_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: times every launch-shape variant (with and without cp.async
// staging) of the row and column passes on the plan's grid and keeps the
// fastest.  Results are cached per (kind, fx, fy, ny, fields) for the process.
// FO_ROW_VARIANT / FO_COL_VARIANT / FO_PREFETCH=0 override the choice.
// ---------------------------------------------------------------------------
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, std::tuple<int, int, int, bool>> g_tune;


// Best per-launch time of `reps` samples.  Launches shorter than about 0.25 ms are
// timed in back-to-back runs of that length, so that event resolution and launch
// latency do not decide between variants of a short pass.
float time_launches(const std::function<cudaError_t()>& fn, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  if (fn() != cudaSuccess) best = -1.f;  // warm-up (and a launch-failure probe)
  int runs = 1;
  for (int r = 0; r < reps + 1 && best >= 0.f; ++r) {
    cudaEventRecord(a, 0);
    for (int i = 0; i < runs && best >= 0.f; ++i)
      if (fn() != cudaSuccess) best = -1.f;
    if (best < 0.f) break;
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    ms /= runs;
    if (r == 0) {  // sizing sample
      runs = std::max(1, std::min(64, (int)std::ceil(0.25f / std::max(ms, 1e-3f))));
      if (runs == 1) best = ms;
      continue;
    }
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaGetLastError();
  return best;
}

// Column-pass work items: runs of at most this many fields sharing one table.
int fields_per_item() { return std::max(1, std::min(64, env_int("FO_FIELDS_PER_ITEM", 16))); }

int autotune_plan(fo_prop_plan p) {
  // Time the shapes on the plan's own batch (up to 2 GiB of fields) and with the
  // plan's work-item length, so that the number of CTAs and the last partial wave
  // are those of the real passes.
  const size_t field_bytes = sizeof(float2) * (size_t)p->ny * p->fx;
  const int cap = (int)std::max<size_t>(1, std::min<size_t>(64, (size_t(2) << 30) / field_bytes));
  const int nb = std::min(p->batch, cap);
  const auto key = std::make_tuple(p->kind, p->fx, p->fy, p->ny, nb);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      std::tie(p->row_v, p->row_pf, p->col_v, p->col_pf) = it->second;
      return FO_OK;
    }
  }
  float2* tmp = nullptr;
  int* idx = nullptr;
  FO_TRY(dalloc(&tmp, (size_t)nb * p->ny * p->fx, "autotune buffer"));
  if (dalloc(&idx, 2 * (size_t)nb + 2, "autotune indices") != FO_OK) {
    cudaFree(tmp);
    return FO_ERR_ALLOC;
  }
  std::vector<int> hidx(2 * nb + 2, 0);
  for (int i = 0; i < nb; ++i) hidx[i] = i;  // field list
  const int fpi = fields_per_item();
  int n_items = 0;  // runs of fpi fields (all on table 0)
  for (int f = 0; f < nb; f += fpi) hidx[nb + n_items++] = f;
  hidx[nb + n_items] = nb;
  cudaMemcpy(idx, hidx.data(), sizeof(int) * hidx.size(), cudaMemcpyHostToDevice);
  cudaMemset(tmp, 0, sizeof(float2) * (size_t)nb * p->ny * p->fx);
  float best = 1e30f;
  int bv = 0;
  int brs = 0;
  for (int v = 0; v < row_variant_count(p->fx); ++v) {
    for (int pf = 0; pf < 3; ++pf) {  // staging: none, cp.async, register prefetch
      if (pf == 1 && !row_prefetch_fits(p->fx, v)) continue;
      RowPassArgs a;
      std::memset(&a, 0, sizeof(a));
      a.src = tmp;
      a.dst = tmp;
      a.src_bstride = a.dst_bstride = (long long)p->fx * p->ny;
      a.src_ld = a.dst_ld = p->fx;
      a.nrows = p->ny;
      a.n_valid = p->nx;
      a.batch = nb;
      a.fields_per_cta = row_fields_per_cta(nb);
      a.inv_first = 1;
      a.fwd_after = 1;
      int trc = FO_OK;
      const float2* tw = twiddles(p->fx, row_variant(p->fx, v).E, &trc);
      if (!tw) continue;
      const float ms = time_launches([&] { return launch_row_pass(p->fx, v, pf, a, tw, 0); }, 3);
      if (env_int("FO_VERBOSE", 0) > 1)
        fprintf(stderr, "[fluxoptics_gb300] tune row N=%d v=%d (E=%d lanes=%d) pf=%d: %.4f ms\n", p->fx, v,
                row_variant(p->fx, v).E, row_variant(p->fx, v).lanes, pf, ms);
      if (ms >= 0.f && ms < best) {
        best = ms;
        bv = v;
        brs = pf;
      }
    }
  }
  p->row_v = bv;
  p->row_pf = brs;
  best = 1e30f;
  bv = 0;
  bool bpf = false;
  for (int v = 0; v < col_variant_count(p->fy); ++v) {
    for (int pf = 0; pf < 2; ++pf) {
      if (pf && !col_prefetch_fits(p->fy, v)) continue;
      ColPassArgs a;
      std::memset(&a, 0, sizeof(a));
      a.buf = tmp;
      a.bstride = (long long)p->fx * p->ny;
      a.ld = p->fx;
      a.ncols = p->fx;
      a.y_in = a.y_out = p->ny;
      a.H = p->H;
      a.h_stride = (long long)p->fx * p->fy;
      a.h_index = p->h_index;
      a.batch = nb;
      a.field_list = idx;
      a.item_start = idx + nb;
      a.n_items = n_items;
      alignas(64) CUtensorMap tm_buf, tm_h;
      if (col_variant_uses_tma(p->fy, v)) {
        if (pf) continue;  // staging is built in
        const int W = col_variant(p->fy, v).lanes;
        const bool t4 = p->ny % 256 == 0 && p->fy % 256 == 0 && env_int("FO_TILE4D", 1) != 0;
        if ((t4 ? encode_tmap_4d(&tm_buf, tmp, nb, p->ny, p->fx, p->fx, W)
                : encode_tmap_3d(&tm_buf, tmp, nb, p->ny, p->fx, p->fx, W, 256)) != FO_OK ||
            (t4 ? encode_tmap_4d(&tm_h, p->H, p->n_tables, p->fy, p->fx, p->fx, W)
                : encode_tmap_2d(&tm_h, p->H, (long long)p->n_tables * p->fy, p->fx, p->fx, W, 256)) != FO_OK)
          continue;
        a.tile4d = t4 ? 1 : 0;
        a.tmap_buf = &tm_buf;
        a.tmap_h = &tm_h;
        a.err_word = p->err_word;
        a.wait_ns = p->wait_ns;
      }
      int trc = FO_OK;
      const float2* tw = twiddles(p->fy, col_variant(p->fy, v).E, &trc);
      if (!tw) continue;
      const float ms = time_launches([&] { return launch_col_pass(p->fy, v, pf != 0, a, tw, 0); }, 3);
      if (env_int("FO_VERBOSE", 0) > 1)
        fprintf(stderr, "[fluxoptics_gb300] tune col N=%d v=%d (E=%d lanes=%d) pf=%d: %.4f ms\n", p->fy, v,
                col_variant(p->fy, v).E, col_variant(p->fy, v).lanes, pf, ms);
      if (ms >= 0.f && ms < best) {
        best = ms;
        bv = v;
        bpf = pf != 0;
      }
    }
  }
  p->col_v = bv;
  p->col_pf = bpf;
  cudaFree(tmp);
  cudaFree(idx);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "autotuning");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = std::make_tuple(p->row_v, p->row_pf, p->col_v, p->col_pf);
  return FO_OK;
}

// Work units of the TMA column variants.  The (strip, item) CTAs of the 2-D launch
// come in rounds of `slots` (SMs x CTAs per SM); when the last round is only partly
// filled, its units are cut into shorter runs of fields so that every slot takes
// a share and the pass ends about when the full rounds do.
int build_col_units(fo_prop_plan p) {
  cudaFree(p->units);
  p->units = nullptr;
  p->n_units = 0;
  p->col_ctas = 0;
  if (!col_variant_uses_tma(p->fy, p->col_v) || env_int("FO_COL_UNITS", 1) == 0) return FO_OK;
  const int W = col_variant(p->fy, p->col_v).lanes;
  ColPassArgs q;
  std::memset(&q, 0, sizeof(q));
  int occ = 0;
  q.occupancy_out = &occ;
  int dev = 0, sms = 0;
  if (launch_col_pass(p->fy, p->col_v, false, q, nullptr, 0) != cudaSuccess || occ < 1 ||
      cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
    cudaGetLastError();
    return FO_OK;  // keep the 2-D launch
  }
  const int slots = sms * occ;
  const int strips = (p->fx + W - 1) / W;
  const std::vector<ColUnit> list = balanced_col_units(p->items_host, strips, slots);
  if (list.empty()) return FO_OK;  // a single round: the 2-D launch
  std::vector<int4> units;
  units.reserve(list.size());
  for (const ColUnit& u : list) units.push_back(make_int4(u.first, u.end, u.strip, 0));
  int rc = dalloc(&p->units, units.size(), "column work units");
  if (rc != FO_OK) return rc;
  cudaError_t e = cudaMemcpy(p->units, units.data(), sizeof(int4) * units.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p->units);
    p->units = nullptr;
    return cuda_fail(e, "cudaMemcpy column work units");
  }
  p->n_units = (int)units.size();
  // One CTA per SM walks its share of the units, prefetching across unit
  // boundaries.  Only for shapes that fill an SM with one CTA: at 2048^2 with
  // 2-column strips (two CTAs per SM) the persistent walk measured 1.96 vs 1.06 ms,
  // while the hardware's own dispatch of the units is fine at any occupancy.
  if (occ == 1 && env_int("FO_COL_PERSIST", 1) != 0) p->col_ctas = slots;
  return FO_OK;
}

void apply_overrides(fo_prop_plan p) {
  const int rv = env_int("FO_ROW_VARIANT", -1), cv = env_int("FO_COL_VARIANT", -1);
  if (rv >= 0 && rv < row_variant_count(p->fx)) p->row_v = rv;
  if (cv >= 0 && cv < col_variant_count(p->fy)) p->col_v = cv;
  if (env_int("FO_PREFETCH", 1) == 0) {
    p->row_pf = 0;
    p->col_pf = false;
  }
  const int rpf = env_int("FO_ROW_PF", -1), cpf = env_int("FO_COL_PF", -1);
  if (rpf >= 0) p->row_pf = std::min(rpf, 2);
  if (cpf >= 0) p->col_pf = cpf != 0;
}

int make_plan(fo_prop_plan* out, int kind, int nx, int ny, int batch, double dx, double dy,
              const double* lambdas, int n_lambdas, double z, double n0, int flags,
              const fo_as_options* opt = nullptr) {
  if (!out) return fail(FO_ERR_ARG, "plan output pointer is NULL");
  *out = nullptr;
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  if (!(dx > 0) || !(dy > 0)) return fail(FO_ERR_ARG, "dx and dy must be positive");
  if (!lambdas || (n_lambdas != 1 && n_lambdas != batch))
    return fail(FO_ERR_ARG, "lambdas must hold 1 or batch wavelengths");
  for (int i = 0; i < n_lambdas; ++i)
    if (!(lambdas[i] > 0)) return fail(FO_ERR_ARG, "wavelengths must be positive");
  if (!std::isfinite(z)) return fail(FO_ERR_ARG, "z must be finite");
  if (kind == 0 && !(n0 > 0)) return fail(FO_ERR_ARG, "n0 must be positive");
  if (opt && opt->tilts && opt->n_tilts != 1 && opt->n_tilts != batch)
    return fail(FO_ERR_ARG, "tilts must hold 1 or batch (theta_x, theta_y) pairs");
  if (opt && opt->tilts)
    for (int i = 0; i < 2 * opt->n_tilts; ++i)
      if (!std::isfinite(opt->tilts[i])) return fail(FO_ERR_ARG, "tilt angles must be finite");
  // kind 0 ASProp, 1 RSProp (padded), 2 Fourier-domain modulator (multiplier set later)
  const int fx = kind == 1 ? next_pow2(2 * nx - 1) : nx;
  const int fy = kind == 1 ? next_pow2(2 * ny - 1) : ny;
  if (!fft_size_supported(fx) || !fft_size_supported(fy))
    return fail(FO_ERR_SHAPE, "transform size " + std::to_string(fx) + " x " + std::to_string(fy) +
                                  " is not supported (powers of two from 16 to 4096)");
  fo_prop_plan p = new fo_prop_plan_s();
  p->kind = kind;
  p->nx = nx;
  p->ny = ny;
  p->batch = batch;
  p->fx = fx;
  p->fy = fy;
  p->dx = dx;
  p->dy = dy;
  p->z = z;
  p->n0 = n0;
  p->lambdas.resize(batch);
  for (int b = 0; b < batch; ++b) p->lambdas[b] = lambdas[n_lambdas == 1 ? 0 : b];
  // transfer-function kind: on axis, tilted (any field with a non-zero tilt) or paraxial
  const bool paraxial = opt && opt->paraxial;
  std::vector<std::array<double, 2>> tilt(batch, {0.0, 0.0});
  bool tilted = false;
  if (opt && opt->tilts)
    for (int b = 0; b < batch; ++b) {
      const int t = opt->n_tilts == 1 ? 0 : b;
      tilt[b] = {opt->tilts[2 * t], opt->tilts[2 * t + 1]};
      tilted = tilted || tilt[b][0] != 0.0 || tilt[b][1] != 0.0;
    }
  const int h_mode = paraxial ? 2 : (tilted ? 1 : 0);
  // distinct (wavelength, tilts) -> one transfer function each
  std::vector<std::array<double, 3>> uniq;
  std::vector<int> hidx(batch);
  for (int b = 0; b < batch; ++b) {
    const std::array<double, 3> key{p->lambdas[b], h_mode ? tilt[b][0] : 0.0, h_mode ? tilt[b][1] : 0.0};
    auto it = std::find(uniq.begin(), uniq.end(), key);
    if (it == uniq.end()) {
      hidx[b] = (int)uniq.size();
      uniq.push_back(key);
    } else {
      hidx[b] = (int)(it - uniq.begin());
    }
  }
  p->n_tables = (int)uniq.size();
  p->h_mode = h_mode;
  for (const auto& k : uniq) {
    p->table_lambda.push_back(k[0]);
    p->table_theta.push_back({k[1], k[2]});
  }
  p->track = (opt && opt->track_tilts) ? 1 : 0;
  int rc = FO_OK;
  const size_t table = (size_t)fx * fy;
  if ((rc = dalloc(&p->H, table * p->n_tables, "transfer functions")) != FO_OK ||
      (rc = dalloc(&p->h_index, batch, "table index")) != FO_OK ||
      (rc = dalloc(&p->sorted_fields, batch, "field order")) != FO_OK ||
      (rc = dalloc(&p->items, batch + 1, "field runs")) != FO_OK ||
      (rc = dalloc(&p->inv_lambda, batch, "inverse wavelengths")) != FO_OK) {
    plan_free(p);
    return rc;
  }
  p->ws_bytes = sizeof(float2) * table * p->n_tables + (sizeof(int) + sizeof(float)) * batch;
  p->err_word = device_error_word(&rc);
  if (!p->err_word) {
    plan_free(p);
    return rc;
  }
  {
    const char* w = getenv("FO_WAIT_NS");
    if (w && *w) p->wait_ns = strtoull(w, nullptr, 10);
  }
  if (kind == 1) {
    if ((rc = dalloc(&p->scratch, (size_t)batch * ny * fx, "padded scratch")) != FO_OK) {
      plan_free(p);
      return rc;
    }
    p->ws_bytes += sizeof(float2) * (size_t)batch * ny * fx;
  }
  p->tw_x = twiddles(fx, row_variant(fx, 0).E, &rc);
  if (!p->tw_x) {
    plan_free(p);
    return rc;
  }
  p->tw_y = twiddles(fy, col_variant(fy, 0).E, &rc);
  if (!p->tw_y) {
    plan_free(p);
    return rc;
  }
  std::vector<float> il(batch);
  for (int b = 0; b < batch; ++b) il[b] = (float)(1.0 / p->lambdas[b]);
  std::vector<int> order(batch);
  for (int b = 0; b < batch; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hidx[a] < hidx[b]; });
  // column-pass work items: runs of at most kFieldsPerItem fields sharing one table
  const int kFieldsPerItem = fields_per_item();
  std::vector<int> items{0};
  for (int i = 1; i <= batch; ++i) {
    if (i == batch || hidx[order[i]] != hidx[order[i - 1]] || i - items.back() >= kFieldsPerItem)
      items.push_back(i);
  }
  p->n_items = (int)items.size() - 1;
  p->items_host = items;
  cudaError_t e = cudaMemcpy(p->h_index, hidx.data(), sizeof(int) * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->sorted_fields, order.data(), sizeof(int) * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->items, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->inv_lambda, il.data(), sizeof(float) * batch, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    plan_free(p);
    return cuda_fail(e, "cudaMemcpy plan tables");
  }
  const double scale = 1.0 / ((double)fx * (double)fy);
  double2* d_filter = nullptr;
  // plans whose distance is later set from device memory keep the filter values of
  // every table (the rebuild needs them); others fill one scratch table per table
  const bool keep_filter = kind == 0 && opt && opt->filter && (flags & (FO_FLAG_GRAD_SPECTRA | FO_FLAG_DEVICE_Z));
  if (kind == 0 && opt && opt->filter) {
    p->has_filter = true;
    if (keep_filter) {
      if ((rc = dalloc(&p->filters, table * p->n_tables, "filter values")) != FO_OK) {
        plan_free(p);
        return rc;
      }
      p->ws_bytes += sizeof(double2) * table * p->n_tables;
    } else if ((rc = dalloc(&d_filter, table, "filter values")) != FO_OK) {
      plan_free(p);
      return rc;
    }
  }
  std::vector<double> ffx, ffy, fre, fim;
  std::vector<double2> fval;
  if (kind == 2) e = cudaMemset(p->H, 0, sizeof(float2) * table * p->n_tables);
  for (int i = 0; i < p->n_tables && e == cudaSuccess && kind != 2; ++i) {
    float2* Hi = p->H + table * i;
    if (kind == 0) {
      const double lam = uniq[i][0];
      double2* fl = p->filters ? p->filters + table * i : d_filter;
      if (fl) {
        // the reference evaluates the filter at the (tilt-shifted for the tilted
        // kernel) frequencies: filter(fx + f0x, fy + f0y), f0 = sin(theta) n0 / lambda
        const double lm = lam / n0;
        const double f0x = h_mode == 1 ? sin(uniq[i][1]) / lm : 0.0, f0y = h_mode == 1 ? sin(uniq[i][2]) / lm : 0.0;
        ffx.resize(table);
        ffy.resize(table);
        fre.assign(table, 1.0);
        fim.assign(table, 0.0);
        for (int ky = 0; ky < fy; ++ky)
          for (int kx = 0; kx < fx; ++kx) {
            const size_t q = (size_t)ky * fx + kx;
            ffx[q] = (kx < (fx + 1) / 2 ? kx : kx - fx) / (fx * dx) + f0x;
            ffy[q] = (ky < (fy + 1) / 2 ? ky : ky - fy) / (fy * dy) + f0y;
          }
        opt->filter(ffx.data(), ffy.data(), (long long)table, fre.data(), fim.data(), opt->filter_ctx);
        fval.resize(table);
        for (size_t q = 0; q < table; ++q) fval[q] = make_double2(fre[q], fim[q]);
        e = cudaMemcpy(fl, fval.data(), sizeof(double2) * table, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) break;
      }
      if (h_mode == 0 && !fl)
        e = launch_as_h(Hi, fx, fy, dx, dy, lam, n0, z, scale, 0);
      else
        e = launch_as_h_general(Hi, fx, fy, dx, dy, lam, n0, z, scale, h_mode, uniq[i][1], uniq[i][2],
                                opt && opt->track_tilts ? 1 : 0, fl, 0);
      if (d_filter && e == cudaSuccess) e = cudaDeviceSynchronize();  // d_filter is refilled next
    } else {
      e = launch_rs_h_spatial(Hi, nx, ny, fx, fy, dx, dy, uniq[i][0], z, scale, 0);
      if (e == cudaSuccess) {
        // H_RS = FFT2(h): row transforms of all fy rows, then column transforms
        Layout L{fx, fy, 1, fx, fy, false, 0, 0};
        Mod none;
        rc = row_pass(L, Hi, Hi, false, true, none, false, 1.f, nullptr, nullptr, p->tw_x, 0);
        if (rc != FO_OK) {
          plan_free(p);
          return rc;
        }
        ColPassArgs a;
        std::memset(&a, 0, sizeof(a));
        a.buf = Hi;
        a.bstride = (long long)table;
        a.ld = fx;
        a.ncols = fx;
        a.y_in = fy;
        a.y_out = fy;
        a.fft_only = 1;
        a.batch = 1;
        a.n_items = 1;
        e = launch_col_pass(fy, 0, false, a, p->tw_y, 0);
      }
    }
  }
  if (e == cudaSuccess && kind == 0 && (flags & FO_FLAG_GRAD_SPECTRA)) {
    const size_t nf = (size_t)batch * fx * fy;
    if ((rc = dalloc(&p->spec_a, nf, "gradient spectra")) != FO_OK ||
        (rc = dalloc(&p->spec_b, nf, "gradient spectra")) != FO_OK ||
        (rc = dalloc(&p->zgrad_partials, (size_t)as_z_grad_blocks(), "z-gradient partials")) != FO_OK ||
        (rc = dalloc(&p->zpar, batch, "z-gradient field parameters")) != FO_OK) {
      if (d_filter) cudaFree(d_filter);
      plan_free(p);
      return rc;
    }
    p->ws_bytes += 2 * sizeof(float2) * nf;
    std::vector<float4> zp(batch);
    for (int b = 0; b < batch; ++b) {
      const double lm = p->lambdas[b] / n0;
      const double f0x = h_mode ? sin(tilt[b][0]) / lm : 0.0, f0y = h_mode ? sin(tilt[b][1]) / lm : 0.0;
      zp[b] = make_float4((float)(1.0 / lm), (float)f0x, (float)f0y, (float)lm);
    }
    e = cudaMemcpy(p->zpar, zp.data(), sizeof(float4) * batch, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (d_filter) cudaFree(d_filter);
  if (e != cudaSuccess) {
    plan_free(p);
    return cuda_fail(e, "building transfer functions");
  }
  // FO_AUTOTUNE=0 / =1 in the environment forces the tuner off / on
  const int tune_env = env_int("FO_AUTOTUNE", -1);
  if (tune_env == 1 || (tune_env != 0 && (flags & FO_FLAG_AUTOTUNE))) {
    rc = autotune_plan(p);
    if (rc != FO_OK) {
      plan_free(p);
      return rc;
    }
  }
  apply_overrides(p);
  p->tw_x = twiddles(fx, row_variant(fx, p->row_v).E, &rc);
  p->tw_y = p->tw_x ? twiddles(fy, col_variant(fy, p->col_v).E, &rc) : nullptr;
  if (!p->tw_x || !p->tw_y) {
    plan_free(p);
    return rc;
  }
  if ((rc = build_col_units(p)) != FO_OK) {
    plan_free(p);
    return rc;
  }
  if (env_int("FO_VERBOSE", 0))
    fprintf(stderr, "[fluxoptics_gb300] plan %s %dx%d (fft %dx%d) batch %d: row variant %d (E=%d, lanes=%d, pf=%d), col variant %d (E=%d, lanes=%d, pf=%d)\n",
            kind == 0 ? "AS" : "RS", nx, ny, fx, fy, batch, p->row_v, row_variant(fx, p->row_v).E,
            row_variant(fx, p->row_v).lanes, (int)p->row_pf, p->col_v, col_variant(fy, p->col_v).E,
            col_variant(fy, p->col_v).lanes, (int)p->col_pf);
  *out = p;
  return FO_OK;
}

}  // namespace

extern "C" {

FO_API int fo_version(void) { return 1 * 10000 + 0 * 100 + 0; }

FO_API const char* fo_last_error(void) { return g_last_error.c_str(); }

FO_API int fo_profile_begin(void) {
  g_prof = true;
  return FO_OK;
}

FO_API int fo_profile_end(double* ms, int* launches) {
  g_prof = false;
  double acc[3] = {0, 0, 0};
  int cnt[3] = {0, 0, 0};
  int rc = FO_OK;
  for (auto& r : g_prof_recs) {
    float t = 0.f;
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.a, r.b);
    if (e != cudaSuccess && rc == FO_OK) rc = cuda_fail(e, "cudaEventElapsedTime");
    acc[r.kind] += t;
    cnt[r.kind] += 1;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_prof_recs.clear();
  for (int k = 0; k < 3; ++k) {
    if (ms) ms[k] = acc[k];
    if (launches) launches[k] = cnt[k];
  }
  return rc;
}

FO_API int fo_device_status(void* stream) {
  cudaError_t e = cudaStreamSynchronize(S(stream));
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  int rc = FO_OK;
  unsigned int* w = device_error_word(&rc);
  if (!w) return rc;
  unsigned int h = 0;
  e = cudaMemcpy(&h, w, sizeof(h), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h) e = cudaMemset(w, 0, sizeof(unsigned int));
  if (e != cudaSuccess) return cuda_fail(e, "reading the device error word");
  if (h & 1u) return fail(FO_ERR_TIMEOUT, "a bounded device wait gave up (TMA copy did not complete in time)");
  if (h & 2u) return fail(FO_ERR_TIMEOUT, "a bounded device wait gave up (grid barrier of the ragged launch)");
  return FO_OK;
}

FO_API int fo_stream_synchronize(void* stream) {
  cudaError_t e = cudaStreamSynchronize(S(stream));
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  return FO_OK;
}

FO_API int fo_asprop_create(fo_prop_plan* plan, int nx, int ny, int batch, double dx, double dy,
                            const double* lambdas, int n_lambdas, double z, double n0, int flags) {
  return make_plan(plan, 0, nx, ny, batch, dx, dy, lambdas, n_lambdas, z, n0, flags);
}

FO_API int fo_asprop_create_ex(fo_prop_plan* plan, int nx, int ny, int batch, double dx, double dy,
                               const double* lambdas, int n_lambdas, double z, double n0,
                               const fo_as_options* options, int flags) {
  return make_plan(plan, 0, nx, ny, batch, dx, dy, lambdas, n_lambdas, z, n0, flags, options);
}

// Unnormalised 2-D FFT of every field of `src` into `dst` (row transforms, then
// column transforms with the plain cp.async column kernel).
static int fft2_into(const fo_prop_plan_s* p, const float2* src, float2* dst, cudaStream_t st) {
  Mod none;
  FO_TRY(row_pass(layout_of(p), src, dst, false, true, none, false, 1.f, p->inv_lambda, nullptr, p->tw_x, st));
  ColPassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.buf = dst;
  a.bstride = (long long)p->fx * p->ny;
  a.ld = p->fx;
  a.ncols = p->fx;
  a.y_in = a.y_out = p->ny;
  a.fft_only = 1;
  a.batch = p->batch;
  a.n_items = p->batch;
  int trc = FO_OK;
  const float2* tw = twiddles(p->fy, col_variant(p->fy, 0).E, &trc);
  if (!tw) return trc;
  FO_LAUNCH(launch_col_pass(p->fy, 0, false, a, tw, st));
  return FO_OK;
}

FO_API int fo_fft2(fo_prop_plan plan, void* u, int mode, void* stream) {
  if (!plan || !u) return fail(FO_ERR_ARG, "plan and u must not be NULL");
  if (mode < FO_FFT_FORWARD || mode > FO_FFT_INVERSE_ADJOINT) return fail(FO_ERR_ARG, "unknown fo_fft2 mode");
  if (plan->fx != plan->nx || plan->fy != plan->ny)
    return fail(FO_ERR_ARG, "fo_fft2 needs a plan on the field's own grid (ASProp or Fourier), not a padded one");
  float2* x = reinterpret_cast<float2*>(u);
  cudaStream_t st = S(stream);
  const long long n = (long long)plan->nx * plan->ny * plan->batch;
  const float inv_n = (float)(1.0 / ((double)plan->nx * (double)plan->ny));
  // the inverse directions run as conj(DFT(conj(x)))
  const bool conj = mode == FO_FFT_INVERSE || mode == FO_FFT_FORWARD_ADJOINT;
  if (conj) FO_LAUNCH(launch_conj_scale(x, n, 1.f, 1, st));
  FO_TRY(fft2_into(plan, x, x, st));
  if (conj || mode == FO_FFT_INVERSE_ADJOINT)
    FO_LAUNCH(launch_conj_scale(x, n, mode == FO_FFT_FORWARD_ADJOINT ? 1.f : inv_n, conj ? 1 : 0, st));
  return FO_OK;
}

FO_API int fo_prop_set_z(fo_prop_plan plan, const float* z, void* stream) {
  if (!plan || !z) return fail(FO_ERR_ARG, "plan and z must not be NULL");
  if (plan->kind != 0) return fail(FO_ERR_ARG, "fo_prop_set_z needs an ASProp plan");
  if (plan->has_filter && !plan->filters)
    return fail(FO_ERR_ARG, "a filtered plan needs FO_FLAG_DEVICE_Z (or FO_FLAG_GRAD_SPECTRA) for fo_prop_set_z");
  const double scale = 1.0 / ((double)plan->fx * (double)plan->fy);
  const size_t table = (size_t)plan->fx * plan->fy;
  for (int i = 0; i < plan->n_tables; ++i) {
    float2* Hi = plan->H + table * i;
    if (plan->h_mode == 0 && !plan->filters)
      FO_LAUNCH(launch_as_h_z(Hi, plan->fx, plan->fy, plan->dx, plan->dy, plan->table_lambda[i], plan->n0, z, scale,
                              S(stream)));
    else
      FO_LAUNCH(launch_as_h_general(Hi, plan->fx, plan->fy, plan->dx, plan->dy, plan->table_lambda[i], plan->n0,
                                    0.0, scale, plan->h_mode, plan->table_theta[i][0], plan->table_theta[i][1],
                                    plan->track, plan->filters ? plan->filters + table * i : nullptr, S(stream), z));
  }
  return FO_OK;
}

FO_API int fo_prop_z_gradient(fo_prop_plan plan, const float* z, const void* u_saved, const void* du, int direction,
                              float* dz, void* stream) {
  if (!plan || !z || !u_saved || !du || !dz) return fail(FO_ERR_ARG, "plan, z, u_saved, du and dz must not be NULL");
  if (plan->kind != 0 || !plan->spec_a)
    return fail(FO_ERR_ARG, "needs an ASProp plan created with FO_FLAG_GRAD_SPECTRA");
  FO_TRY(check_dir(direction));
  cudaStream_t st = S(stream);
  FO_TRY(fft2_into(plan, reinterpret_cast<const float2*>(u_saved), plan->spec_a, st));
  FO_TRY(fft2_into(plan, reinterpret_cast<const float2*>(du), plan->spec_b, st));
  FO_LAUNCH(launch_as_z_grad(plan->spec_a, plan->spec_b, plan->H, plan->h_index, plan->zpar, plan->h_mode,
                             plan->track, plan->fx, plan->fy, plan->dx, plan->dy, z, plan->batch, direction < 0,
                             plan->zgrad_partials, dz, st));
  return FO_OK;
}

FO_API int fo_fourier_create(fo_prop_plan* plan, int nx, int ny, int batch, int flags) {
  const double one = 1.0;
  int rc = make_plan(plan, 2, nx, ny, batch, 1.0, 1.0, &one, 1, 0.0, 1.0, flags & FO_FLAG_AUTOTUNE);
  if (rc != FO_OK) return rc;
  fo_prop_plan p = *plan;
  if (flags & FO_FOURIER_TRAINABLE) {
    const size_t n = (size_t)batch * nx * ny;
    if ((rc = dalloc(&p->spec_a, n, "Fourier gradient spectra")) != FO_OK ||
        (rc = dalloc(&p->spec_b, n, "Fourier gradient spectra")) != FO_OK) {
      plan_free(p);
      *plan = nullptr;
      return rc;
    }
    p->ws_bytes += 2 * sizeof(float2) * n;
  }
  return FO_OK;
}

FO_API int fo_fourier_set(fo_prop_plan plan, int kind, const void* param, void* stream) {
  if (!plan || !param) return fail(FO_ERR_ARG, "plan and param must not be NULL");
  if (plan->kind != 2) return fail(FO_ERR_ARG, "not a Fourier-modulator plan");
  if (kind != MOD_PHASE && kind != MOD_MASK) return fail(FO_ERR_ARG, "kind must be FO_MOD_PHASE or FO_MOD_MASK");
  FO_LAUNCH(launch_fourier_h(plan->H, kind, param, (long long)plan->fx * plan->fy,
                             1.0 / ((double)plan->fx * (double)plan->fy), S(stream)));
  return FO_OK;
}

FO_API int fo_fourier_gradient(fo_prop_plan plan, int kind, const void* param, const void* u_saved, const void* dv,
                               void* grad, int direction, void* stream) {
  if (!plan || !param || !u_saved || !dv || !grad)
    return fail(FO_ERR_ARG, "plan, param, u_saved, dv and grad must not be NULL");
  if (plan->kind != 2 || !plan->spec_a) return fail(FO_ERR_ARG, "needs a Fourier plan created with FO_FOURIER_TRAINABLE");
  if (kind != MOD_PHASE && kind != MOD_MASK) return fail(FO_ERR_ARG, "kind must be FO_MOD_PHASE or FO_MOD_MASK");
  FO_TRY(check_dir(direction));
  cudaStream_t st = S(stream);
  FO_TRY(fft2_into(plan, reinterpret_cast<const float2*>(u_saved), plan->spec_a, st));
  FO_TRY(fft2_into(plan, reinterpret_cast<const float2*>(dv), plan->spec_b, st));
  FO_LAUNCH(launch_fourier_grad(kind, param, plan->spec_a, plan->spec_b, grad, (long long)plan->fx * plan->fy,
                                plan->batch, (float)direction, st));
  return FO_OK;
}

FO_API int fo_rsprop_create(fo_prop_plan* plan, int nx, int ny, int batch, double dx, double dy,
                            const double* lambdas, int n_lambdas, double z, int flags) {
  return make_plan(plan, 1, nx, ny, batch, dx, dy, lambdas, n_lambdas, z, 1.0, flags);
}

FO_API int fo_prop_destroy(fo_prop_plan plan) {
  plan_free(plan);
  return FO_OK;
}

FO_API int fo_prop_info(fo_prop_plan plan, int* fft_nx, int* fft_ny, size_t* workspace_bytes) {
  if (!plan) return fail(FO_ERR_ARG, "plan is NULL");
  if (fft_nx) *fft_nx = plan->fx;
  if (fft_ny) *fft_ny = plan->fy;
  if (workspace_bytes) *workspace_bytes = plan->ws_bytes;
  return FO_OK;
}

FO_API int fo_prop_variants(fo_prop_plan plan, int* row_v, int* col_v, char* row_kernel, char* col_kernel,
                            int len) {
  if (!plan) return fail(FO_ERR_ARG, "plan is NULL");
  if (row_v) *row_v = plan->row_v;
  if (col_v) *col_v = plan->col_v;
  auto put = [len](char* dst, const std::string& s) {
    if (!dst || len <= 0) return;
    const size_t n = std::min((size_t)len - 1, s.size());
    std::memcpy(dst, s.data(), n);
    dst[n] = 0;
  };
  const PassVariant rv = row_variant(plan->fx, plan->row_v);
  const PassVariant cv = col_variant(plan->fy, plan->col_v);
  put(row_kernel, "row_pass_kernel<" + std::to_string(plan->fx) + ", E=" + std::to_string(rv.E) +
                      ", rows/CTA=" + std::to_string(rv.lanes) + (plan->row_pf == 1   ? ", cp.async staging>"
                       : plan->row_pf == 2 ? ", register prefetch>"
                                           : ">"));
  const char* form = cv.P == 6   ? "col_tma_kernel (TMA load/store, register twiddles)"
                     : cv.P == 4 ? "col_tma_kernel (TMA load/store)"
                     : cv.P == 2 ? "col_pass2_kernel (paired columns)"
                     : cv.P == 0 ? "col_lane_kernel (lane-major)"
                                 : (plan->col_pf ? "col_pass_kernel (cp.async staging)" : "col_pass_kernel");
  put(col_kernel, std::string(form) + "<" + std::to_string(plan->fy) + ", E=" + std::to_string(cv.E) +
                      ", columns/CTA=" + std::to_string(cv.lanes) + ">" +
                      (plan->units ? " over " + std::to_string(plan->n_units) + " balanced work units" : "") +
                      (plan->col_ctas ? " in " + std::to_string(plan->col_ctas) + " persistent CTAs" : ""));
  return FO_OK;
}

FO_API int fo_propagate(fo_prop_plan plan, void* u, int direction, void* stream) {
  if (!plan || !u) return fail(FO_ERR_ARG, "plan and u must not be NULL");
  FO_TRY(check_dir(direction));
  std::vector<fo_prop_plan> props{plan};
  Mod mods[2];
  float2* uu = reinterpret_cast<float2*>(u);
  float2* buf = plan->kind == 1 ? plan->scratch : uu;
  return run_forward(props, buf, uu, mods, direction, S(stream));
}

// ---------------------------------------------------------------------------
// Standalone modulators
// ---------------------------------------------------------------------------

FO_API int fo_phase_forward(void* u, const float* phi, void* u_saved, int nx, int ny, int batch,
                            int direction, void* stream) {
  if (!u || !phi) return fail(FO_ERR_ARG, "u and phi must not be NULL");
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  FO_TRY(check_dir(direction));
  FO_LAUNCH(launch_phase_fwd(reinterpret_cast<float2*>(u), phi, reinterpret_cast<float2*>(u_saved),
                             (long long)nx * ny, batch, (float)direction, S(stream)));
  return FO_OK;
}

FO_API int fo_phase_backward(void* dv, const float* phi, const void* u_saved, float* dphi, int nx,
                             int ny, int batch, int direction, void* stream) {
  if (!dv || !phi) return fail(FO_ERR_ARG, "dv and phi must not be NULL");
  if (dphi && !u_saved) return fail(FO_ERR_ARG, "dphi needs u_saved");
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  FO_TRY(check_dir(direction));
  FO_LAUNCH(launch_phase_bwd(reinterpret_cast<float2*>(dv), phi, reinterpret_cast<const float2*>(u_saved),
                             dphi, (long long)nx * ny, batch, (float)direction, S(stream)));
  return FO_OK;
}

FO_API int fo_tea_forward(void* u, const float* h, const void* field_coef, void* u_saved, int nx, int ny,
                          int batch, int direction, void* stream) {
  if (!u || !h || !field_coef) return fail(FO_ERR_ARG, "u, h and field_coef must not be NULL");
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  FO_TRY(check_dir(direction));
  FO_LAUNCH(launch_tea_fwd(reinterpret_cast<float2*>(u), h, reinterpret_cast<const float4*>(field_coef),
                           reinterpret_cast<float2*>(u_saved), (long long)nx * ny, batch, (float)direction,
                           S(stream)));
  return FO_OK;
}

FO_API int fo_tea_backward(void* dv, const float* h, const void* field_coef, const void* u_saved, float* dh,
                           int nx, int ny, int batch, int direction, void* stream) {
  if (!dv || !h || !field_coef) return fail(FO_ERR_ARG, "dv, h and field_coef must not be NULL");
  if (dh && !u_saved) return fail(FO_ERR_ARG, "dh needs u_saved");
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  FO_TRY(check_dir(direction));
  FO_LAUNCH(launch_tea_bwd(reinterpret_cast<float2*>(dv), h, reinterpret_cast<const float4*>(field_coef),
                           reinterpret_cast<const float2*>(u_saved), dh, (long long)nx * ny, batch,
                           (float)direction, S(stream)));
  return FO_OK;
}

FO_API int fo_mask_forward(void* u, const void* m, void* u_saved, int nx, int ny, int batch,
                           int direction, void* stream) {
  if (!u || !m) return fail(FO_ERR_ARG, "u and m must not be NULL");
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  FO_TRY(check_dir(direction));
  FO_LAUNCH(launch_mask_fwd(reinterpret_cast<float2*>(u), reinterpret_cast<const float2*>(m),
                            reinterpret_cast<float2*>(u_saved), (long long)nx * ny, batch,
                            direction < 0, S(stream)));
  return FO_OK;
}

FO_API int fo_mask_backward(void* dv, const void* m, const void* u_saved, void* dm, int nx, int ny,
                            int batch, int direction, void* stream) {
  if (!dv || !m) return fail(FO_ERR_ARG, "dv and m must not be NULL");
  if (dm && !u_saved) return fail(FO_ERR_ARG, "dm needs u_saved");
  if (nx <= 0 || ny <= 0 || batch <= 0) return fail(FO_ERR_SHAPE, "nx, ny and batch must be positive");
  FO_TRY(check_dir(direction));
  FO_LAUNCH(launch_mask_bwd(reinterpret_cast<float2*>(dv), reinterpret_cast<const float2*>(m),
                            reinterpret_cast<const float2*>(u_saved), reinterpret_cast<float2*>(dm),
                            (long long)nx * ny, batch, (float)direction, S(stream)));
  return FO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Chains
// ---------------------------------------------------------------------------
struct fo_chain_s {
  std::vector<fo_prop_plan> props;
  float2* scratch = nullptr;  // padded layouts only
  std::vector<float2*> probes[2];  // field probes before / after each modulation slot (empty: none)
  const std::vector<float2*>* probe_ptr() const { return probes[0].empty() ? nullptr : probes; }
};

extern "C" {

FO_API int fo_chain_create(fo_chain* chain, int n_props, const fo_prop_plan* props) {
  if (!chain) return fail(FO_ERR_ARG, "chain output pointer is NULL");
  *chain = nullptr;
  if (n_props < 1 || !props) return fail(FO_ERR_ARG, "a chain needs at least one propagator");
  for (int k = 0; k < n_props; ++k)
    if (!props[k]) return fail(FO_ERR_ARG, "propagator plan is NULL");
  const Layout L = layout_of(props[0]);
  for (int k = 1; k < n_props; ++k)
    if (!same_layout(L, layout_of(props[k])))
      return fail(FO_ERR_SHAPE, "all propagators of a chain must share grid, batch and padding");
  fo_chain c = new fo_chain_s();
  c->props.assign(props, props + n_props);
  if (L.padded) {
    int rc = dalloc(&c->scratch, (size_t)L.batch * L.ny * L.fx, "chain scratch");
    if (rc != FO_OK) {
      delete c;
      return rc;
    }
  }
  *chain = c;
  return FO_OK;
}

FO_API int fo_chain_destroy(fo_chain chain) {
  if (chain) {
    cudaFree(chain->scratch);
    delete chain;
  }
  return FO_OK;
}

FO_API int fo_chain_set_probes(fo_chain chain, void* const* pre, void* const* post) {
  if (!chain) return fail(FO_ERR_ARG, "chain is NULL");
  const int K = (int)chain->props.size();
  bool any = false;
  for (int k = 0; k <= K; ++k) any = any || (pre && pre[k]) || (post && post[k]);
  for (int h = 0; h < 2; ++h) chain->probes[h].clear();
  if (!any) return FO_OK;
  for (int h = 0; h < 2; ++h) {
    void* const* src = h == 0 ? pre : post;
    chain->probes[h].assign(K + 1, nullptr);
    for (int k = 0; k <= K; ++k) {
      void* q = src ? src[k] : nullptr;
      if (q && (reinterpret_cast<uintptr_t>(q) & 7) != 0) {
        chain->probes[0].clear();
        chain->probes[1].clear();
        return fail(FO_ERR_ARG, "probe buffers must be 8-byte aligned");
      }
      chain->probes[h][k] = reinterpret_cast<float2*>(q);
    }
  }
  return FO_OK;
}

FO_API int fo_chain_forward(fo_chain chain, void* u, const fo_mod* mods, int direction, void* stream) {
  if (!chain || !u || !mods) return fail(FO_ERR_ARG, "chain, u and mods must not be NULL");
  FO_TRY(check_dir(direction));
  const int K = (int)chain->props.size();
  std::vector<Mod> m(K + 1);
  for (int k = 0; k <= K; ++k) {
    m[k] = mod_from(&mods[k]);
    FO_TRY(validate_mod(m[k], false));
  }
  float2* uu = reinterpret_cast<float2*>(u);
  float2* buf = chain->scratch ? chain->scratch : uu;
  return run_forward(chain->props, buf, uu, m.data(), direction, S(stream), nullptr, nullptr, nullptr, nullptr,
                     chain->probe_ptr());
}

FO_API int fo_chain_forward_from(fo_chain chain, const void* u_in, void* u, const fo_mod* mods,
                                 int direction, void* stream) {
  if (!chain || !u_in || !u || !mods) return fail(FO_ERR_ARG, "chain, u_in, u and mods must not be NULL");
  FO_TRY(check_dir(direction));
  const int K = (int)chain->props.size();
  std::vector<Mod> m(K + 1);
  for (int k = 0; k <= K; ++k) {
    m[k] = mod_from(&mods[k]);
    FO_TRY(validate_mod(m[k], false));
  }
  float2* uu = reinterpret_cast<float2*>(u);
  float2* buf = chain->scratch ? chain->scratch : uu;
  return run_forward(chain->props, buf, uu, m.data(), direction, S(stream),
                     reinterpret_cast<const float2*>(u_in), nullptr, nullptr, nullptr, chain->probe_ptr());
}

FO_API int fo_chain_forward_sid(fo_chain chain, const void* u_in, void* u, const fo_mod* mods, int direction,
                                fo_sid sid, const float* target, float* loss, void* stream) {
  if (!chain || !u || !mods || !sid || !target || !loss)
    return fail(FO_ERR_ARG, "chain, u, mods, sid, target and loss must not be NULL");
  FO_TRY(check_dir(direction));
  const int K = (int)chain->props.size();
  const Layout L = layout_of(chain->props[0]);
  if (sid->nx != L.nx || sid->ny != L.ny || sid->batch != L.batch)
    return fail(FO_ERR_SHAPE, "metric and chain shapes differ");
  std::vector<Mod> m(K + 1);
  for (int k = 0; k <= K; ++k) {
    m[k] = mod_from(&mods[k]);
    FO_TRY(validate_mod(m[k], false));
  }
  float2* uu = reinterpret_cast<float2*>(u);
  float2* buf = chain->scratch ? chain->scratch : uu;
  const float2* src = reinterpret_cast<const float2*>(u_in);
  if (sid->group > 0)
    return run_forward(chain->props, buf, uu, m.data(), direction, S(stream), src, sid, target, loss,
                       chain->probe_ptr());
  // slices with different field counts: the metric runs as its own pass
  FO_TRY(run_forward(chain->props, buf, uu, m.data(), direction, S(stream), src, nullptr, nullptr, nullptr,
                     chain->probe_ptr()));
  return fo_sid_forward(sid, u, target, loss, stream);
}

FO_API int fo_chain_withgradient_sid(fo_chain chain, const void* u_in, void* u_out, void* du,
                                     const fo_mod* mods_fwd, const fo_mod* mods_bwd, int direction, fo_sid sid,
                                     const float* target, float* loss, int flags, void* stream) {
  if (!chain || !u_in || !du || !mods_fwd || !mods_bwd || !sid || !target || !loss)
    return fail(FO_ERR_ARG, "chain, u_in, du, mods_fwd, mods_bwd, sid, target and loss must not be NULL");
  FO_TRY(check_dir(direction));
  if (u_out == du) return fail(FO_ERR_ARG, "u_out and du must be different buffers");
  if (u_in == du || u_in == u_out)
    return fail(FO_ERR_ARG, "u_in must not alias u_out or du: the adjoint sweep reads it");
  const int K = (int)chain->props.size();
  const Layout L = layout_of(chain->props[0]);
  if (sid->nx != L.nx || sid->ny != L.ny || sid->batch != L.batch)
    return fail(FO_ERR_SHAPE, "metric and chain shapes differ");
  std::vector<Mod> mf(K + 1), mb(K + 1);
  for (int k = 0; k <= K; ++k) {
    mf[k] = mod_from(&mods_fwd[k]);
    mb[k] = mod_from(&mods_bwd[k]);
    FO_TRY(validate_mod(mf[k], false));
    FO_TRY(validate_mod(mb[k], true));
  }
  const bool discard = (flags & FO_BWD_DISCARD_INPUT_GRAD) != 0;
  if (mf[K].kind != MOD_NONE || mb[K].kind != MOD_NONE || sid->group <= 0 || chain->probe_ptr()) {
    // the shared pass does not apply: the separate forward and adjoint sweeps
    void* out = u_out ? u_out : du;
    FO_TRY(fo_chain_forward_sid(chain, u_in, out, mods_fwd, direction, sid, target, loss, stream));
    return fo_chain_backward_ex(chain, du, mods_bwd, direction, sid, out, flags, stream);
  }
  float2* d = reinterpret_cast<float2*>(du);
  float2* w = chain->scratch ? chain->scratch : d;
  cudaStream_t st = S(stream);
  return run_withgradient(chain->props, w, reinterpret_cast<const float2*>(u_in), d, mf.data(), mb.data(), direction,
                          st, discard, [&](const Layout& L, const float2* tw) {
                            FO_TRY(row_pass_sid_seed(L, w, reinterpret_cast<float2*>(u_out), sid, target, tw, st));
                            FO_LAUNCH(launch_sid_finalize(sid->partials, L.ny, sid->T, loss, st));
                            return FO_OK;
                          });
}

FO_API int fo_chain_withgradient_sfd(fo_chain chain, const void* u_in, void* u_out, void* du,
                                     const fo_mod* mods_fwd, const fo_mod* mods_bwd, int direction, fo_sfd sfd,
                                     const void* v, const float* dc, float* c, int flags, void* stream) {
  if (!chain || !u_in || !du || !mods_fwd || !mods_bwd || !sfd || !v || !c)
    return fail(FO_ERR_ARG, "chain, u_in, du, mods_fwd, mods_bwd, sfd, v and c must not be NULL");
  FO_TRY(check_dir(direction));
  if (u_out == du) return fail(FO_ERR_ARG, "u_out and du must be different buffers");
  if (u_in == du || u_in == u_out)
    return fail(FO_ERR_ARG, "u_in must not alias u_out or du: the adjoint sweep reads it");
  if (v == du || v == u_out) return fail(FO_ERR_ARG, "v must not alias u_out or du");
  const int K = (int)chain->props.size();
  const Layout L = layout_of(chain->props[0]);
  if (sfd->nx != L.nx || sfd->ny != L.ny || sfd->batch != L.batch)
    return fail(FO_ERR_SHAPE, "metric and chain shapes differ");
  std::vector<Mod> mf(K + 1), mb(K + 1);
  for (int k = 0; k <= K; ++k) {
    mf[k] = mod_from(&mods_fwd[k]);
    mb[k] = mod_from(&mods_bwd[k]);
    FO_TRY(validate_mod(mf[k], false));
    FO_TRY(validate_mod(mb[k], true));
  }
  if (mf[K].kind != MOD_NONE || mb[K].kind != MOD_NONE || chain->probe_ptr()) {
    // the shared pass does not apply: forward sweep, metric, pull-back, adjoint sweep
    void* out = u_out ? u_out : du;
    FO_TRY(fo_chain_forward_from(chain, u_in, out, mods_fwd, direction, stream));
    FO_TRY(fo_sfd_forward(sfd, out, v, c, stream));
    FO_TRY(fo_sfd_backward(sfd, out, v, dc, du, stream));
    return fo_chain_backward_ex(chain, du, mods_bwd, direction, nullptr, nullptr, flags, stream);
  }
  float2* d = reinterpret_cast<float2*>(du);
  float2* w = chain->scratch ? chain->scratch : d;
  cudaStream_t st = S(stream);
  return run_withgradient(chain->props, w, reinterpret_cast<const float2*>(u_in), d, mf.data(), mb.data(), direction,
                          st, (flags & FO_BWD_DISCARD_INPUT_GRAD) != 0, [&](const Layout& L, const float2* tw) {
                            return row_pass_sfd_seed(L, w, reinterpret_cast<float2*>(u_out), sfd,
                                                     reinterpret_cast<const float2*>(v), dc, c, tw, st);
                          });
}

FO_API int fo_chain_backward(fo_chain chain, void* du, const fo_mod* mods, int direction, fo_sid sid,
                             const void* u_out, void* stream) {
  return fo_chain_backward_ex(chain, du, mods, direction, sid, u_out, 0, stream);
}

FO_API int fo_chain_backward_ex(fo_chain chain, void* du, const fo_mod* mods, int direction, fo_sid sid,
                                const void* u_out, int flags, void* stream) {
  if (!chain || !du || !mods) return fail(FO_ERR_ARG, "chain, du and mods must not be NULL");
  FO_TRY(check_dir(direction));
  const int K = (int)chain->props.size();
  std::vector<Mod> m(K + 1);
  for (int k = 0; k <= K; ++k) {
    m[k] = mod_from(&mods[k]);
    FO_TRY(validate_mod(m[k], true));
  }
  float2* d = reinterpret_cast<float2*>(du);
  float2* buf = chain->scratch ? chain->scratch : d;
  SeedArgs seed;
  const float2* src0 = d;
  if (sid) {
    const Layout L = layout_of(chain->props[0]);
    if (!u_out) return fail(FO_ERR_ARG, "a seeded sweep needs u_out");
    if (sid->nx != L.nx || sid->ny != L.ny || sid->batch != L.batch)
      return fail(FO_ERR_SHAPE, "metric and chain shapes differ");
    seed.resid = sid->resid;
    seed.tidx = sid->tidx;
    seed.dc = sid->ones;
    src0 = reinterpret_cast<const float2*>(u_out);
  }
  return run_backward(chain->props, buf, d, src0, m.data(), direction, sid ? &seed : nullptr, S(stream),
                      (flags & FO_BWD_DISCARD_INPUT_GRAD) != 0);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// AS_BPM
// ---------------------------------------------------------------------------
struct fo_bpm_s {
  fo_prop_plan full = nullptr, half = nullptr;
  int nx = 0, ny = 0, batch = 0, n_slices = 0, every = 1, n_ckpt = 0;
  double kdz = 0;
  float2* ckpt = nullptr;  // n_ckpt x batch x ny x nx
  float2* seg = nullptr;   // 2 x every x batch x ny x nx (slot 0 of each half unused): segments alternate halves
  float2* rbuf = nullptr;  // recompute field
  cudaStream_t aux = nullptr;  // recomputes the next segment while the adjoint sweeps the current one
  cudaEvent_t ev_fork = nullptr, ev_rec[2] = {nullptr, nullptr}, ev_use[2] = {nullptr, nullptr};
  size_t ws_bytes = 0;
};

namespace {

// AS_BPM with a scalar cos correction (opt == NULL) or with the options' tilts, whose
// per-field cos correction cos(theta_x) cos(theta_y) is folded into the plans' per-field
// inverse wavelengths (the dn phase of field b is kdz * dn / (lambda_b cos_b), with
// kdz = 2 pi dz).
int bpm_create(fo_bpm* bpm, int nx, int ny, int batch, double dx, double dy, const double* lambdas, int n_lambdas,
               double thickness, double n0, int n_slices, int checkpoint_every, double cos_correction,
               const fo_as_options* opt, int flags) {
  if (!bpm) return fail(FO_ERR_ARG, "bpm output pointer is NULL");
  *bpm = nullptr;
  if (n_slices < 2) return fail(FO_ERR_SHAPE, "AS_BPM needs at least 2 slices");
  if (!(thickness > 0) || !(cos_correction > 0)) return fail(FO_ERR_ARG, "thickness and cos_correction must be positive");
  if (checkpoint_every < 0) return fail(FO_ERR_ARG, "checkpoint_every must be >= 0");
  if (opt && opt->filter) return fail(FO_ERR_ARG, "AS_BPM takes no frequency filter");
  if (opt && opt->tilts && opt->n_tilts != 1 && opt->n_tilts != batch)
    return fail(FO_ERR_ARG, "tilts must hold 1 or batch pairs");
  const double dz = thickness / n_slices;
  fo_bpm b = new fo_bpm_s();
  int rc = make_plan(&b->full, 0, nx, ny, batch, dx, dy, lambdas, n_lambdas, dz, n0, flags, opt);
  if (rc == FO_OK) rc = make_plan(&b->half, 0, nx, ny, batch, dx, dy, lambdas, n_lambdas, dz / 2, n0, flags, opt);
  if (rc == FO_OK && opt && opt->tilts) {
    std::vector<float> il(batch);
    for (int i = 0; i < batch; ++i) {
      const double* th = opt->tilts + 2 * (opt->n_tilts == 1 ? 0 : i);
      const double c = cos(th[0]) * cos(th[1]);
      if (!(c > 0)) {
        rc = fail(FO_ERR_ARG, "tilts must be below pi/2");
        break;
      }
      il[i] = (float)(1.0 / (lambdas[n_lambdas == 1 ? 0 : i] * c));
    }
    for (fo_prop_plan q : {b->full, b->half}) {
      if (rc != FO_OK) break;
      cudaError_t e = cudaMemcpy(q->inv_lambda, il.data(), sizeof(float) * batch, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy BPM phase factors");
    }
  }
  if (rc != FO_OK) {
    plan_free(b->full);
    plan_free(b->half);
    delete b;
    return rc;
  }
  b->nx = nx;
  b->ny = ny;
  b->batch = batch;
  b->n_slices = n_slices;
  int every = checkpoint_every == 0 ? (int)lround(sqrt((double)n_slices)) : checkpoint_every;
  every = std::max(1, std::min(every, n_slices));
  b->every = every;
  b->n_ckpt = (n_slices + every - 1) / every;
  b->kdz = 2.0 * M_PI * dz / cos_correction;
  const size_t field = (size_t)batch * ny * nx;
  if ((rc = dalloc(&b->ckpt, field * b->n_ckpt, "BPM checkpoints")) != FO_OK ||
      (every > 1 && (rc = dalloc(&b->seg, 2 * field * every, "BPM segments")) != FO_OK) ||
      (every > 1 && (rc = dalloc(&b->rbuf, field, "BPM recompute field")) != FO_OK)) {
    cudaFree(b->ckpt);
    cudaFree(b->seg);
    plan_free(b->full);
    plan_free(b->half);
    delete b;
    return rc;
  }
  if (every > 1) {
    cudaError_t e = cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
      e = cudaEventCreateWithFlags(&b->ev_rec[i], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_use[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      fo_bpm_destroy(b);
      return cuda_fail(e, "BPM helper stream");
    }
  }
  b->ws_bytes = sizeof(float2) * field * (b->n_ckpt + (every > 1 ? 2 * every + 1 : 0)) + b->full->ws_bytes +
                b->half->ws_bytes;
  *bpm = b;
  return FO_OK;
}

}  // namespace

extern "C" {

FO_API int fo_bpm_create(fo_bpm* bpm, int nx, int ny, int batch, double dx, double dy,
                         const double* lambdas, int n_lambdas, double thickness, double n0,
                         int n_slices, int checkpoint_every, double cos_correction, int flags) {
  return bpm_create(bpm, nx, ny, batch, dx, dy, lambdas, n_lambdas, thickness, n0, n_slices, checkpoint_every,
                    cos_correction, nullptr, flags);
}

FO_API int fo_bpm_create_ex(fo_bpm* bpm, int nx, int ny, int batch, double dx, double dy,
                            const double* lambdas, int n_lambdas, double thickness, double n0,
                            int n_slices, int checkpoint_every, const fo_as_options* options, int flags) {
  return bpm_create(bpm, nx, ny, batch, dx, dy, lambdas, n_lambdas, thickness, n0, n_slices, checkpoint_every,
                    1.0, options, flags);
}

FO_API int fo_bpm_destroy(fo_bpm b) {
  if (!b) return FO_OK;
  if (b->aux) cudaStreamDestroy(b->aux);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  for (int i = 0; i < 2; ++i) {
    if (b->ev_rec[i]) cudaEventDestroy(b->ev_rec[i]);
    if (b->ev_use[i]) cudaEventDestroy(b->ev_use[i]);
  }
  cudaFree(b->ckpt);
  cudaFree(b->seg);
  cudaFree(b->rbuf);
  plan_free(b->full);
  plan_free(b->half);
  delete b;
  return FO_OK;
}

FO_API int fo_bpm_info(fo_bpm b, int* checkpoint_every, size_t* workspace_bytes) {
  if (!b) return fail(FO_ERR_ARG, "bpm is NULL");
  if (checkpoint_every) *checkpoint_every = b->every;
  if (workspace_bytes) *workspace_bytes = b->ws_bytes;
  return FO_OK;
}

}  // extern "C"

namespace {

float2* bpm_slot(fo_bpm b, int k) {
  const size_t field = (size_t)b->batch * b->ny * b->nx;
  if (k % b->every == 0) return b->ckpt + field * (k / b->every);
  const int half = (k / b->every) & 1;  // consecutive segments use alternate halves
  return b->seg + field * ((size_t)half * b->every + k % b->every);
}

Mod dn_mod(fo_bpm b, const float* dn, int k, void* saved, void* grad) {
  Mod m;
  m.kind = MOD_DN;
  m.param = dn + (size_t)k * b->ny * b->nx;
  m.saved = saved;
  m.grad = grad;
  m.scale = (float)b->kdz;
  return m;
}

// Recompute the slice inputs of the segment that starts at checkpoint g.
int bpm_recompute(fo_bpm b, const float* dn, int g, int s, cudaStream_t st) {
  const int a = g * b->every;
  const int e = std::min(b->n_slices, a + b->every);
  const int K = e - a - 1;  // full steps between the first and the last slice of the segment
  if (K <= 0) return FO_OK;
  const size_t field = (size_t)b->batch * b->ny * b->nx;
  FO_LAUNCH(cudaMemcpyAsync(b->rbuf, b->ckpt + field * g, sizeof(float2) * field, cudaMemcpyDeviceToDevice, st));
  std::vector<fo_prop_plan> props(K, b->full);
  std::vector<Mod> mods(K + 1);
  mods[0] = dn_mod(b, dn, a, nullptr, nullptr);
  for (int k = 1; k <= K; ++k) mods[k] = dn_mod(b, dn, a + k, bpm_slot(b, a + k), nullptr);
  return run_forward(props, b->rbuf, b->rbuf, mods.data(), s, st);
}

}  // namespace

extern "C" {

FO_API int fo_bpm_forward(fo_bpm b, void* u, const float* dn, int direction, int save, void* stream) {
  if (!b || !u || !dn) return fail(FO_ERR_ARG, "bpm, u and dn must not be NULL");
  FO_TRY(check_dir(direction));
  cudaStream_t st = S(stream);
  const int n = b->n_slices;
  // props: half, full x (n-1), half; mods: none, dn_0 .. dn_{n-1}, none
  std::vector<fo_prop_plan> props;
  props.reserve(n + 1);
  props.push_back(b->half);
  for (int k = 0; k < n - 1; ++k) props.push_back(b->full);
  props.push_back(b->half);
  std::vector<Mod> mods(n + 2);
  for (int k = 0; k < n; ++k) {
    void* sv = (save && k % b->every == 0) ? (void*)bpm_slot(b, k) : nullptr;
    mods[k + 1] = dn_mod(b, dn, k, sv, nullptr);
  }
  float2* uu = reinterpret_cast<float2*>(u);
  return run_forward(props, uu, uu, mods.data(), direction, st);
}

FO_API int fo_bpm_backward(fo_bpm b, void* du, const float* dn, float* ddn, int direction, void* stream) {
  if (!b || !du || !dn) return fail(FO_ERR_ARG, "bpm, du and dn must not be NULL");
  FO_TRY(check_dir(direction));
  cudaStream_t st = S(stream);
  const int n = b->n_slices;
  const int s = direction;
  const float sf = (float)s;
  float2* d = reinterpret_cast<float2*>(du);
  const Layout L = layout_of(b->full);
  const float* il = b->full->inv_lambda;
  const float2* tw = b->full->tw_x;
  const int every = b->every;
  const int top = (n - 1) / every;
  bool use_recorded[2] = {false, false};
  // Segment g is recomputed on the helper stream (into half g%2 of the segment
  // buffer) while the adjoint sweeps segment g+1 on the caller's stream.
  auto launch_recompute = [&](int g) -> int {
    if (use_recorded[g & 1]) FO_LAUNCH(cudaStreamWaitEvent(b->aux, b->ev_use[g & 1], 0));
    FO_TRY(bpm_recompute(b, dn, g, s, b->aux));
    FO_LAUNCH(cudaEventRecord(b->ev_rec[g & 1], b->aux));
    return FO_OK;
  };
  if (every > 1) {
    FO_LAUNCH(cudaEventRecord(b->ev_fork, st));  // dn and the checkpoints are ready on st
    FO_LAUNCH(cudaStreamWaitEvent(b->aux, b->ev_fork, 0));
    FO_TRY(launch_recompute(top));
  }
  Mod none;
  FO_TRY(row_pass(L, d, d, false, true, none, true, sf, il, nullptr, tw, st));
  FO_TRY(col_pass(b->half, d, s > 0, st));
  for (int g = top; g >= 0; --g) {
    if (every > 1) {
      FO_LAUNCH(cudaStreamWaitEvent(st, b->ev_rec[g & 1], 0));
      if (g > 0) FO_TRY(launch_recompute(g - 1));
    }
    const int k_hi = std::min(n - 1, (g + 1) * every - 1);
    for (int k = k_hi; k >= g * every; --k) {
      Mod m = dn_mod(b, dn, k, bpm_slot(b, k), ddn ? (void*)(ddn + (size_t)k * b->ny * b->nx) : nullptr);
      FO_TRY(row_pass(L, d, d, true, true, m, true, sf, il, nullptr, tw, st));
      FO_TRY(col_pass(k > 0 ? b->full : b->half, d, s > 0, st));
    }
    if (every > 1) {
      FO_LAUNCH(cudaEventRecord(b->ev_use[g & 1], st));
      use_recorded[g & 1] = true;
    }
  }
  return row_pass(L, d, d, true, false, none, true, sf, il, nullptr, tw, st);
}

// ---------------------------------------------------------------------------
// SquaredIntensityDifference
// ---------------------------------------------------------------------------

FO_API int fo_sid_create(fo_sid* sid, int nx, int ny, int batch, int n_targets, const int* target_index) {
  if (!sid) return fail(FO_ERR_ARG, "sid output pointer is NULL");
  *sid = nullptr;
  if (nx <= 0 || ny <= 0 || batch <= 0 || n_targets <= 0) return fail(FO_ERR_SHAPE, "sizes must be positive");
  std::vector<int> tidx(batch);
  for (int b = 0; b < batch; ++b) {
    tidx[b] = target_index ? target_index[b] : b % n_targets;
    if (tidx[b] < 0 || tidx[b] >= n_targets) return fail(FO_ERR_ARG, "target_index out of range");
  }
  std::vector<int> order, offsets(n_targets + 1, 0);
  for (int t = 0; t < n_targets; ++t) {
    offsets[t] = (int)order.size();
    for (int b = 0; b < batch; ++b)
      if (tidx[b] == t) order.push_back(b);
  }
  offsets[n_targets] = (int)order.size();
  fo_sid m = new fo_sid_s();
  m->group = offsets[1];
  for (int t = 0; t < n_targets; ++t)
    if (offsets[t + 1] - offsets[t] != m->group) m->group = 0;
  m->nx = nx;
  m->ny = ny;
  m->batch = batch;
  m->T = n_targets;
  const long long npix = (long long)nx * ny;
  int rc;
  std::vector<float> ones(n_targets, 1.f);
  if ((rc = dalloc(&m->tidx, batch, "metric index")) != FO_OK ||
      (rc = dalloc(&m->order, batch, "metric order")) != FO_OK ||
      (rc = dalloc(&m->offsets, n_targets + 1, "metric offsets")) != FO_OK ||
      (rc = dalloc(&m->resid, (size_t)n_targets * npix, "metric residuals")) != FO_OK ||
      (rc = dalloc(&m->partials, (size_t)std::max(sid_partial_blocks(npix), ny) * n_targets,
                   "metric partial sums")) != FO_OK ||
      (rc = dalloc(&m->ones, n_targets, "metric ones")) != FO_OK) {
    fo_sid_destroy(m);
    return rc;
  }
  cudaError_t e = cudaMemcpy(m->tidx, tidx.data(), sizeof(int) * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->order, order.data(), sizeof(int) * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(m->offsets, offsets.data(), sizeof(int) * (n_targets + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->ones, ones.data(), sizeof(float) * n_targets, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    fo_sid_destroy(m);
    return cuda_fail(e, "cudaMemcpy metric tables");
  }
  *sid = m;
  return FO_OK;
}

FO_API int fo_sid_destroy(fo_sid m) {
  if (!m) return FO_OK;
  cudaFree(m->tidx);
  cudaFree(m->order);
  cudaFree(m->offsets);
  cudaFree(m->resid);
  cudaFree(m->partials);
  cudaFree(m->ones);
  delete m;
  return FO_OK;
}

FO_API int fo_sid_forward(fo_sid m, const void* u, const float* target, float* loss, void* stream) {
  if (!m || !u || !target || !loss) return fail(FO_ERR_ARG, "sid, u, target and loss must not be NULL");
  FO_LAUNCH(launch_sid_fwd(reinterpret_cast<const float2*>(u), target, m->order, m->offsets, m->T,
                           (long long)m->nx * m->ny, m->resid, m->partials, loss, S(stream)));
  return FO_OK;
}

FO_API int fo_sid_backward(fo_sid m, const void* u, const float* dc, void* du, void* stream) {
  if (!m || !u || !du) return fail(FO_ERR_ARG, "sid, u and du must not be NULL");
  FO_LAUNCH(launch_sid_bwd(reinterpret_cast<const float2*>(u), m->resid, m->tidx, dc ? dc : m->ones,
                           (long long)m->nx * m->ny, m->batch, reinterpret_cast<float2*>(du), S(stream)));
  return FO_OK;
}

// ---------------------------------------------------------------------------
// Optimiser / prox
// ---------------------------------------------------------------------------

FO_API int fo_fista_step(float* x, float* xk, float* newdx, const float* dx, long long n, double eta,
                         double* t_state, void* stream) {
  if (!x || !xk || !dx || !t_state) return fail(FO_ERR_ARG, "x, xk, dx and t_state must not be NULL");
  if (n <= 0) return fail(FO_ERR_SHAPE, "n must be positive");
  FO_LAUNCH(launch_fista(x, xk, newdx, dx, n, (float)(eta * eta), t_state, S(stream)));
  return FO_OK;
}

FO_API int fo_fista_clamp_step(float* x, float* xk, float* newdx, const float* dx, long long n, double eta,
                               double* t_state, double lo, double hi, void* stream) {
  if (!x || !xk || !dx || !t_state) return fail(FO_ERR_ARG, "x, xk, dx and t_state must not be NULL");
  if (n <= 0) return fail(FO_ERR_SHAPE, "n must be positive");
  if (!(lo <= hi)) return fail(FO_ERR_ARG, "lo must not exceed hi");
  FO_LAUNCH(launch_fista(x, xk, newdx, dx, n, (float)(eta * eta), t_state, S(stream), 1, (float)lo, (float)hi));
  return FO_OK;
}

FO_API int fo_clamp(float* x, long long n, double lo, double hi, void* stream) {
  if (!x) return fail(FO_ERR_ARG, "x must not be NULL");
  if (n <= 0) return fail(FO_ERR_SHAPE, "n must be positive");
  if (!(lo <= hi)) return fail(FO_ERR_ARG, "lo must not exceed hi");
  FO_LAUNCH(launch_clamp(x, n, (float)lo, (float)hi, S(stream)));
  return FO_OK;
}

}  // extern "C"

struct fo_tv_s {
  int nd = 2, dims[3] = {1, 1, 1}, n_iter = 0, isotropic = 1;
  double lambda = 0, eta = 0, tol = 0;
  float *p = nullptr, *xk = nullptr, *y = nullptr, *partials = nullptr;
  float *yprev = nullptr, *maxima = nullptr;  // with a tolerance
  void* state = nullptr;
};

extern "C" {

FO_API int fo_tv_create_nd(fo_tv* tv, int ndims, const int* dims, double lambda, int n_iter, int isotropic,
                           double eta, double tol) {
  if (!tv) return fail(FO_ERR_ARG, "tv output pointer is NULL");
  *tv = nullptr;
  if (ndims < 1 || ndims > 3 || !dims) return fail(FO_ERR_SHAPE, "TVProx takes 1-, 2- or 3-D arrays");
  size_t n = 1;
  for (int i = 0; i < ndims; ++i) {
    if (dims[i] < 2) return fail(FO_ERR_SHAPE, "TVProx needs at least 2 samples along every dimension");
    n *= (size_t)dims[i];
  }
  if (n_iter < 0) return fail(FO_ERR_ARG, "n_iter must be >= 0");
  if (!(tol >= 0)) return fail(FO_ERR_ARG, "tol must be >= 0 (0: none)");
  fo_tv t = new fo_tv_s();
  t->nd = ndims;
  for (int i = 0; i < ndims; ++i) t->dims[i] = dims[i];
  t->n_iter = n_iter;
  t->isotropic = isotropic ? 1 : 0;
  t->lambda = lambda;
  t->eta = eta;
  t->tol = tol;
  const size_t blocks = (size_t)tv_partial_blocks((long long)n);
  int rc;
  if ((rc = dalloc(&t->p, ndims * n, "TV dual")) != FO_OK || (rc = dalloc(&t->xk, ndims * n, "TV state")) != FO_OK ||
      (rc = dalloc(&t->y, n, "TV primal")) != FO_OK ||
      (rc = dalloc(&t->partials, blocks * 3, "TV partials")) != FO_OK ||
      (tol > 0 && (rc = dalloc(&t->yprev, n, "TV previous primal")) != FO_OK) ||
      (tol > 0 && (rc = dalloc(&t->maxima, blocks, "TV block maxima")) != FO_OK) ||
      (rc = dalloc(reinterpret_cast<char**>(&t->state), tv_state_bytes(), "TV scalars")) != FO_OK) {
    fo_tv_destroy(t);
    return rc;
  }
  *tv = t;
  return FO_OK;
}

FO_API int fo_tv_create_ex(fo_tv* tv, int nx, int ny, double lambda, int n_iter, int isotropic, double eta,
                           double tol) {
  const int dims[2] = {nx, ny};
  return fo_tv_create_nd(tv, 2, dims, lambda, n_iter, isotropic, eta, tol);
}

FO_API int fo_tv_create(fo_tv* tv, int nx, int ny, double lambda, int n_iter, int isotropic, double eta) {
  return fo_tv_create_ex(tv, nx, ny, lambda, n_iter, isotropic, eta, 0.0);
}

FO_API int fo_tv_destroy(fo_tv t) {
  if (!t) return FO_OK;
  cudaFree(t->p);
  cudaFree(t->xk);
  cudaFree(t->y);
  cudaFree(t->partials);
  cudaFree(t->yprev);
  cudaFree(t->maxima);
  cudaFree(t->state);
  delete t;
  return FO_OK;
}

FO_API int fo_tv_apply(fo_tv t, float* x, void* stream) {
  if (!t || !x) return fail(FO_ERR_ARG, "tv and x must not be NULL");
  const double lam = t->isotropic ? t->lambda : t->lambda / 100.0;
  FO_LAUNCH(launch_tv(x, t->p, t->xk, t->y, t->partials, t->state, t->nd, t->dims, (float)lam, t->n_iter,
                      t->isotropic, (float)(t->eta * t->eta), S(stream), t->tol, t->yprev, t->maxima));
  return FO_OK;
}

// ---------------------------------------------------------------------------
// CUDA graphs
// ---------------------------------------------------------------------------

}  // extern "C"

struct fo_graph_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

FO_API int fo_copy(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes == 0) return FO_OK;
  if (!dst || !src) return fail(FO_ERR_ARG, "dst and src must not be NULL");
  FO_LAUNCH(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, S(stream)));
  return FO_OK;
}

FO_API int fo_graph_begin(void* stream) {
  if (!stream) return fail(FO_ERR_ARG, "graph capture needs a non-default stream");
  FO_LAUNCH(cudaStreamBeginCapture(S(stream), cudaStreamCaptureModeThreadLocal));
  return FO_OK;
}

FO_API int fo_graph_end(void* stream, fo_graph* graph) {
  if (!stream || !graph) return fail(FO_ERR_ARG, "stream and graph must not be NULL");
  *graph = nullptr;
  fo_graph g = new fo_graph_s();
  cudaError_t e = cudaStreamEndCapture(S(stream), &g->graph);
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  *graph = g;
  return FO_OK;
}

FO_API int fo_graph_info(fo_graph g, int* kernel_nodes) {
  if (!g || !kernel_nodes) return fail(FO_ERR_ARG, "graph and kernel_nodes must not be NULL");
  size_t n = 0;
  FO_LAUNCH(cudaGraphGetNodes(g->graph, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  FO_LAUNCH(cudaGraphGetNodes(g->graph, nodes.data(), &n));
  int k = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    FO_LAUNCH(cudaGraphNodeGetType(nd, &t));
    if (t == cudaGraphNodeTypeKernel) ++k;
  }
  *kernel_nodes = k;
  return FO_OK;
}

FO_API int fo_graph_launch(fo_graph g, void* stream) {
  if (!g) return fail(FO_ERR_ARG, "graph is NULL");
  FO_LAUNCH(cudaGraphLaunch(g->exec, S(stream)));
  return FO_OK;
}

FO_API int fo_graph_destroy(fo_graph g) {
  if (!g) return FO_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return FO_OK;
}

}  // extern "C"
