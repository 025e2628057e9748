// pn_traverse_f32_sph.cu -- the WCSPH and adjoint traversals for Float32 searches.
#include "pn_traverse_sph.cuh"

namespace pn {
template int foreach_sph<float, float>(pn_search*, int32_t, int64_t, const void*, TravCall<float>&,
                                   cudaStream_t);
}  // namespace pn
