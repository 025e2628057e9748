// pn_traverse_f32.cu -- foreach_point_neighbor kernels for Float32 searches.
#include "pn_traverse_impl.cuh"

namespace pn {
template int foreach<float>(pn_search*, int32_t, const float*, int64_t, const float*, int64_t,
                            const int32_t*, int64_t, const void*, cudaStream_t,
                            const ListsRef*);
template int lists_count<float>(pn_search*, const float*, int64_t, const float*, int64_t,
                                int32_t*, int32_t*, int64_t*, cudaStream_t);
template int lists_emit<float>(pn_search*, const float*, int64_t, const float*, int64_t,
                               int32_t*, const int64_t*, int32_t, int32_t*, cudaStream_t);
}  // namespace pn
