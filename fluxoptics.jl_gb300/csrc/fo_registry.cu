// Dispatch of the row / column passes to their per-size launch-shape variants.
#include "fo_fft.cuh"
#include "fo_internal.h"
#include "fo_variants.h"

#include <cstdlib>

namespace fo {

#define FO_DECL(NN)                                                                                  \
  cudaError_t row_launch_##NN(int v, const RowPassArgs& a, const float2* tw, cudaStream_t s, int pf); \
  cudaError_t col_launch_##NN(int v, const ColPassArgs& a, const float2* tw, cudaStream_t s, bool pf);
FO_FOR_EACH_N(FO_DECL)
#undef FO_DECL

namespace {

struct Table {
  int n = 0;
  PassVariant v[12];
};

template <int N>
Table row_table();
template <int N>
Table col_table();

#define FO_TABLES(NN)                                             \
  template <>                                                     \
  Table row_table<NN>() {                                         \
    Table t;                                                      \
    FO_ROW_VARIANTS_##NN(FO_ADD) return t;                        \
  }                                                               \
  template <>                                                     \
  Table col_table<NN>() {                                         \
    Table t;                                                      \
    FO_COL_VARIANTS_##NN(FO_ADDC) return t;                       \
  }
#define FO_ADD(I, E, L) t.v[t.n++] = PassVariant{E, L, 1};
#define FO_ADDC(I, E, L, P) t.v[t.n++] = PassVariant{E, L, P};
FO_FOR_EACH_N(FO_TABLES)
#undef FO_ADD
#undef FO_ADDC
#undef FO_TABLES

Table table_for(int N, bool row) {
  switch (N) {
#define FO_CASE(NN) \
  case NN:          \
    return row ? row_table<NN>() : col_table<NN>();
    FO_FOR_EACH_N(FO_CASE)
#undef FO_CASE
    default:
      return Table{};
  }
}

constexpr size_t kMaxSmem = 227 * 1024;

}  // namespace

bool fft_size_supported(int n) { return table_for(n, true).n > 0; }

// Programmatic dependent launch lets a pass start while the previous one drains; every
// pass kernel waits for its predecessor (griddepcontrol.wait) before touching memory.
// It pays for small passes, whose launch latency it hides (a 512^2 RSProp chain on
// 1024^2 grids: 62.1 vs 58.5 k propagations/s), and costs large ones (2048^2 x 48
// fields: 12.17 vs 10.52 ms per iteration).  So it is used for passes over at most
// kPdlMaxBytes of fields; FO_PDL=1 / FO_PDL=0 force it on / off for every pass.
constexpr long long kPdlMaxBytes = 32LL << 20;

bool pdl_for(long long field_bytes) {
  static const int mode = [] {
    const char* v = getenv("FO_PDL");
    return !v || !*v ? -1 : (v[0] == '1' ? 1 : 0);
  }();
  return mode < 0 ? field_bytes <= kPdlMaxBytes : mode == 1;
}

int row_variant_count(int N) { return table_for(N, true).n; }
int col_variant_count(int N) { return table_for(N, false).n; }
PassVariant row_variant(int N, int v) { return table_for(N, true).v[v]; }
PassVariant col_variant(int N, int v) { return table_for(N, false).v[v]; }

size_t row_smem_bytes(int N, int v, bool pf) {
  const PassVariant pv = row_variant(N, v);
  // the gradient passes add a modulation cache of N float2 per row
  return sizeof(float2) * ((size_t)(pf ? 2 : 1) * pv.lanes * (size_t)(N + N / 16) + (size_t)pv.lanes * N);
}
size_t col_smem_bytes(int N, int v, bool pf) {
  const PassVariant pv = col_variant(N, v);
  if (pv.P == 0) return sizeof(float2) * 2 * pv.lanes * (size_t)(N + N / 16 + 4);  // always staged
  if (pv.P == 4 || pv.P == 6) return sizeof(float2) * pv.lanes * (size_t)(2 * N + N + N / 16);  // TMA staging
  return sizeof(float2) * (size_t)(pf ? 2 : 1) * pv.lanes * (size_t)(N + N / 16);  // staging only
}
bool row_prefetch_fits(int N, int v) { return row_smem_bytes(N, v, true) <= kMaxSmem; }
bool col_prefetch_fits(int N, int v) { return col_smem_bytes(N, v, true) <= kMaxSmem; }
bool col_variant_uses_tma(int N, int v) { return col_variant(N, v).P == 4 || col_variant(N, v).P == 6; }

cudaError_t launch_row_pass(int N, int v, int staging, const RowPassArgs& a, const float2* tw, cudaStream_t s) {
  switch (N) {
#define FO_CASE(NN) \
  case NN:          \
    return row_launch_##NN(v, a, tw, s, staging);
    FO_FOR_EACH_N(FO_CASE)
#undef FO_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_col_pass(int N, int v, bool pf, const ColPassArgs& a, const float2* tw, cudaStream_t s) {
  switch (N) {
#define FO_CASE(NN) \
  case NN:          \
    return col_launch_##NN(v, a, tw, s, pf);
    FO_FOR_EACH_N(FO_CASE)
#undef FO_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace fo
