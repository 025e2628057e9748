// pn_traverse_f64.cu -- foreach_point_neighbor kernels for Float64 searches.
#include "pn_traverse_impl.cuh"

namespace pn {
template int foreach<double>(pn_search*, int32_t, const double*, int64_t, const double*, int64_t,
                             const int32_t*, int64_t, const void*, cudaStream_t,
                             const ListsRef*);
template int lists_count<double>(pn_search*, const double*, int64_t, const double*, int64_t,
                                 int32_t*, int32_t*, int64_t*, cudaStream_t);
template int lists_emit<double>(pn_search*, const double*, int64_t, const double*, int64_t,
                               int32_t*, const int64_t*, int32_t, int32_t*, cudaStream_t);
}  // namespace pn
