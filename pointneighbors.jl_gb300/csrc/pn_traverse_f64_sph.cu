// pn_traverse_f64_sph.cu -- the WCSPH and adjoint traversals for Float64 searches.
#include "pn_traverse_sph.cuh"

namespace pn {
template int foreach_sph<double, double>(pn_search*, int32_t, int64_t, const void*, TravCall<double>&,
                                   cudaStream_t);
}  // namespace pn
