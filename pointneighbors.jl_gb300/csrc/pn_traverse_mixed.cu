// pn_traverse_mixed.cu -- foreach_point_neighbor kernels for a search with Float64
// coordinates and a Float32 search radius (PN_FLAG_FLOAT32_SEARCH): the Float32 traversal
// of the cell-sorted queries (MixedFast<D, F>) and the Float64 one of the others
// (Mixed<D, F>), with Float32 pair functions; the WCSPH and adjoint functions are in
// pn_traverse_mixed_sph.cu, the precomputed search's list build in
// pn_traverse_mixed_lists.cu.
#include "pn_traverse_impl.cuh"

namespace pn {

int foreach_mixed(pn_search* s, int32_t functor, const double* x, int64_t n_x, const double* y,
                  int64_t n_y, const int32_t* points, int64_t n_points, const void* params,
                  cudaStream_t st, const ListsRef* lists) {
  return foreach_t<double, float>(s, functor, x, n_x, y, n_y, points, n_points, params, st,
                                  lists);
}

}  // namespace pn
