// pn_traverse_mixed.cu -- foreach_point_neighbor kernels for a search with Float64
// coordinates and a Float32 search radius (PN_FLAG_FLOAT32_SEARCH): Float64 traversal,
// Float32 pair functions behind Mixed<D, F>.
#include "pn_traverse_impl.cuh"

namespace pn {

int foreach_mixed(pn_search* s, int32_t functor, const double* x, int64_t n_x, const double* y,
                  int64_t n_y, const int32_t* points, int64_t n_points, const void* params,
                  cudaStream_t st, const ListsRef* lists) {
  return foreach_t<double, float>(s, functor, x, n_x, y, n_y, points, n_points, params, st,
                                  lists);
}

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
