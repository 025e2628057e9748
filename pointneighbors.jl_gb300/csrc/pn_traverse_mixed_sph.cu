// pn_traverse_mixed_sph.cu -- the WCSPH and adjoint traversals for searches with Float64
// coordinates and a Float32 search radius.
#include "pn_traverse_sph.cuh"

namespace pn {
template int foreach_sph<double, float>(pn_search*, int32_t, int64_t, const void*,
                                        TravCall<double>&, cudaStream_t);
}  // namespace pn
