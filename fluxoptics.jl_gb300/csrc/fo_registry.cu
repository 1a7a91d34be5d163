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

// Off by default: with the whole iteration captured as one graph, programmatic
// edges between the passes measured slower (16.8 vs 15.4 ms for 2048^2 x 48 fields,
// three propagations forward and back) and only the launch-bound BPM march
// gained (about 2 %).  FO_PDL=1 turns it on.
bool pdl_enabled() {
  static const bool on = [] {
    const char* v = getenv("FO_PDL");
    return v && v[0] == '1';
  }();
  return on;
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
