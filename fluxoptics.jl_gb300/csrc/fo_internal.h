// Internal declarations shared by the CUDA translation units of libfluxoptics_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

// SquaredFieldDifference handle (fo_sfd_*): fixed-order per-field sums in `partial`
// (batch x kSfdBlocks) for the standalone metric, and per-row sums in `rows`
// (ny x batch) for the metric fused into a chain's last pass.
struct fo_sfd_s {
  int nx = 0, ny = 0, batch = 0;
  double* partial = nullptr;
  float* rows = nullptr;
};

namespace fo {

// ---------------------------------------------------------------------------
// Errors: every C-ABI entry point returns one of the FO_* status codes from
// include/fluxoptics_gb300.h and leaves a message in a thread-local string.
// ---------------------------------------------------------------------------
void set_error(int code, const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define FO_CUDA_CHECK(expr)                         \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return fo::cuda_fail(_e, #expr); \
  } while (0)

// Modulation kinds applied in real space inside the row passes.
enum ModKind : int { MOD_NONE = 0, MOD_PHASE = 1, MOD_MASK = 2, MOD_DN = 3, MOD_TEA = 4 };

// One row pass over `batch` fields: for every row y < nrows of every field,
// load -> [inverse FFT along x] -> [seed] -> [modulation] -> [forward FFT along x] -> store.
struct RowPassArgs {
  const float2* src;
  float2* dst;
  long long src_bstride, dst_bstride;  // elements between consecutive fields
  int src_ld, dst_ld;                  // elements between consecutive rows
  int nrows;                           // rows processed per field
  int n_valid;                         // real-space x extent (N for AS; n < N for padded RS)
  int batch;                           // fields processed by the launch
  int fields_per_cta;                  // fields looped over inside one CTA
  const int* field_list;               // optional device list of field ids (null: identity)
  int inv_first;                       // row holds a spectrum: inverse-transform it first
  int fwd_after;                       // forward-transform the row before storing
  // modulation
  int mod_kind;
  int mod_bwd;            // 0: forward modulation (+ optional save); 1: adjoint + gradient
  float mod_sign;         // direction sign s
  const void* mod_param;  // phase / dn: float; mask: float2; row stride param_ld
  int param_ld;
  float mod_scale;            // MOD_DN: kdz; the phase factor of field b is mod_scale * inv_lambda[b]
  const float* inv_lambda;    // MOD_DN: per field id, 1 / lambda
  const float4* field_coef;   // MOD_TEA: per field id {2 pi dn(lambda) / lambda, Re r, Im r, 0}
  float2* save;               // forward: modulation input written here (nullable)
  long long save_bstride;
  int save_ld;
  const float2* saved;        // adjoint: saved modulation input
  long long saved_bstride;
  int saved_ld;
  void* grad;                 // adjoint: gradient (float or float2), row stride param_ld (nullable)
  // seed of the adjoint sweep: du = 4 * dc[t] * resid_t * u, t = tidx[field]
  int seed;
  const float* resid;
  long long resid_tstride;
  int resid_ld;
  const int* tidx;
  const float* dc;
  // SquaredIntensityDifference evaluated on the pass output (row kernel GK = 3):
  // each CTA visits one target slice's fields (field_list grouped by slice,
  // fields_per_cta fields per slice), sums their intensities, and writes
  // sid_resid = I - sid_target (layout of resid_tstride / resid_ld) and the row's
  // sum of squares to sid_partials[row * sid_T + slice]; tidx gives the slice.
  const float* sid_target;
  float* sid_resid;
  float* sid_partials;
  int sid_T;
  // field probes of a forward pass (real-space layout of `save`): a copy of the field
  // before (probe_pre) and after (probe_post) the modulation; either may be NULL
  float2* probe_pre;
  float2* probe_post;
  // With sid_partials: the adjoint sweep's first pass in the same launch (row kernel
  // GK = 4), in place on the spectrum: seed_dst must equal src.  The seed
  // 4 dc_t (I_t - target_t) u of every field, forward-transformed along x, replaces the
  // spectrum; `dst` (nullable) receives the output field.  No modulation.
  float2* seed_dst;
  long long seed_bstride;
  int seed_ld;
  // With sfd_rows (row kernel GK = 5): the chain's last forward pass, SquaredFieldDifference
  // against sfd_v (real-space layout of dst) and the adjoint sweep's first pass, in place on
  // the spectrum (seed_dst == src): per field, the output row u (to dst when set), the
  // row's sum |u - v|^2 to sfd_rows[row * batch + field], and the seed 2 dc_b (u - v)
  // (sfd_dc: per field, NULL: ones) forward-transformed along x over the spectrum row.
  const float2* sfd_v;
  float* sfd_rows;
  const float* sfd_dc;
};

// One column pass: forward FFT along y, multiply by the transfer function of the
// field's wavelength (conjugated for the adjoint direction), inverse FFT along y.
struct ColPassArgs {
  float2* buf;
  long long bstride;
  int ld;                // row stride (elements)
  int ncols;             // columns to process
  int y_in, y_out;       // rows read (zero beyond) / rows written
  const float2* H;       // transfer functions, one table of N x ncols per wavelength
  long long h_stride;
  const int* h_index;    // per field id: table index
  int conj_h;
  int fft_only;          // 1: store the forward transform along y (no H, no inverse)
  int batch;
  const int* field_list;  // fields ordered so that each work item shares one table
  const int* item_start;  // n_items+1 offsets into field_list (null: one field per item)
  int n_items;
  // TMA variants: optional 1-D list of work units {first, end (positions in
  // field_list), strip, 0}; the grid is then (n_units, 1)
  const int4* units;
  int n_units;
  int persistent;         // with units: launch this many CTAs, each taking every persistent-th unit (0: one per unit)
  int* occupancy_out;     // when set, the launcher stores the variant's CTAs per SM and launches nothing
  // TMA variants: host addresses of the tensor maps (CUtensorMap) of the buffer,
  // viewed as fields x rows x ncols, and of the transfer functions, viewed as
  // (tables * N) x ncols; the device error word and the wait limit.
  const void* tmap_buf;
  const void* tmap_h;
  unsigned int* err_word;
  unsigned long long wait_ns;
  int test_skip_copy;  // test knob: arm the barrier but issue no copy (the wait must time out)
  // 1: tmap_buf is the 4-D view (columns, row within a 256-row block, row block,
  // field) and tmap_h the 4-D view (columns, row within block, row block, table),
  // so one TMA instruction moves a whole tile (rows a multiple of 256)
  int tile4d;
};

// Device error word of the current device (allocated once, zero).  Bit 0: a bounded
// wait in a kernel gave up.
unsigned int* device_error_word(int* err);
// Host helpers for the TMA variants: encode a 2-D tiled tensor map over a
// float2 array of `rows` x `cols` (row stride `ld` elements) with boxes of
// box_cols x box_rows.  Returns FO_OK or an FO_ERR_* code.
int encode_tmap_2d(void* tmap, const void* base, long long rows, int cols, int ld, int box_cols, int box_rows);
// The same over `fields` consecutive rows x cols slabs (row stride ld, slab stride
// rows * ld elements), boxes of box_cols x box_rows x 1: a box is clipped at the
// last row of its slab.
int encode_tmap_3d(void* tmap, const void* base, int fields, int rows, int cols, int ld, int box_cols, int box_rows);
// 4-D view of `fields` slabs of rows x cols (rows a multiple of 256, at most
// 65536): (column, row within a 256-row block, row block, slab), boxes of
// box_cols x 256 x rows/256 x 1, i.e. a whole column strip of one slab.
int encode_tmap_4d(void* tmap, const void* base, int fields, int rows, int cols, int ld, int box_cols);

// Launch-shape variants (fo_variants.h): E elements per thread, `lanes` rows or
// columns per CTA.  N is the FFT length along the transformed axis; supported:
// powers of two from 16 to 4096.  `pf` selects the cp.async-staged kernels.
struct PassVariant {
  int E;
  int lanes;
  int P;  // transforms per thread (column pass: 2 = paired columns)
};
bool fft_size_supported(int n);
int row_variant_count(int N);
int col_variant_count(int N);
PassVariant row_variant(int N, int v);
PassVariant col_variant(int N, int v);
size_t row_smem_bytes(int N, int v, bool pf);
size_t col_smem_bytes(int N, int v, bool pf);
bool row_prefetch_fits(int N, int v);
bool col_prefetch_fits(int N, int v);
bool col_variant_uses_tma(int N, int v);
// staging of the row passes: 0 none, 1 cp.async staging in shared memory, 2 register
// prefetch of the next field's row (passes without a gradient)
cudaError_t launch_row_pass(int N, int v, int staging, const RowPassArgs& a, const float2* tw, cudaStream_t s);
cudaError_t launch_col_pass(int N, int v, bool pf, const ColPassArgs& a, const float2* tw, cudaStream_t s);

// Stage-major twiddle tables of the (N, E) schedule for the current device (cached).
const float2* twiddles(int N, int E, int* err);

}  // namespace fo
