// pn_traverse_mixed_lists.cu -- the precomputed search's list build for a search with
// Float64 coordinates and a Float32 search radius (PN_FLAG_FLOAT32_SEARCH).
#include "pn_traverse_impl.cuh"

namespace pn {

int lists_count_mixed(pn_search* s, const double* x, int64_t n_x, const double* y, int64_t n_y,
                      int32_t* len, int32_t* by_slot, int64_t* n_rows, cudaStream_t st) {
  return lists_count_t<double, float>(s, x, n_x, y, n_y, len, by_slot, n_rows, st);
}

int lists_emit_mixed(pn_search* s, const double* x, int64_t n_x, const double* y, int64_t n_y,
                     int32_t* nb, const int64_t* grp, int32_t cap, int32_t* len,
                     cudaStream_t st) {
  return lists_emit_t<double, float>(s, x, n_x, y, n_y, nb, grp, cap, len, st);
}

}  // namespace pn
