// Instantiations of the row / column passes for transform length 2048.
#include "fo_passes.cuh"
#include "fo_variants.h"

namespace fo {

cudaError_t row_launch_2048(int v, const RowPassArgs& a, const float2* tw, cudaStream_t s, int pf) {
  switch (v) {
#define X(I, E, L) \
  case I:          \
    return row_launch_shape<2048, E, L>(a, tw, s, pf);
    FO_ROW_VARIANTS_2048(X)
#undef X
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t col_launch_2048(int v, const ColPassArgs& a, const float2* tw, cudaStream_t s, bool pf) {
  switch (v) {
#define X(I, E, W, P) \
  case I:             \
    return col_launch_shape<2048, E, W, P>(a, tw, s, pf);
    FO_COL_VARIANTS_2048(X)
#undef X
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace fo
