// pn_precomputed.cu -- PrecomputedNeighborhoodSearch (nhs_precomputed.jl): neighbour lists
// computed by an internal GridNeighborhoodSearch at initialize!/update!, then every
// foreach_point_neighbor walks the lists instead of the cell stencil.
//
// Lists.  A row holds the neighbours of one query as slots of the internal search's
// cell-sorted arrays (rows are slots too when x is y, so a warp's 32 consecutive queries are
// spatial neighbours).  Rows are grouped by 32 and each group is stored transposed with the
// group's longest row as width: entry t of row r at grp[r / 32] + 32 t + r % 32, the
// transposed backend the reference recommends for GPUs (transpose_backend = true), with the
// padding of a fixed max_neighbors column height replaced by per-group widths.  A row is
// in ascending slot order, i.e. spatial order; pn_pre_neighbor_lists returns point indices
// sorted ascending like the reference's sorteach!.
//
// max_neighbors (> 0) keeps the reference's capacity check: a point with more neighbours
// is its "cell list is full" error.
#include <algorithm>
#include <new>

#include "pn_internal.cuh"

struct pn_precomputed {
  pn_search* grid = nullptr;
  int32_t max_neighbors = 0;
  int32_t dtype = 0;
  int32_t ndims = 0;
  bool built = false;
  pn::ListsRef ref{};
  int32_t* d_len = nullptr;    // [rows]
  int64_t len_cap = 0;
  int32_t* d_width = nullptr;  // [groups] 32 x (longest row of the group)
  int64_t width_cap = 0;
  int64_t* d_grp = nullptr;    // [groups + 1]
  int64_t grp_cap = 0;
  int32_t* d_nb = nullptr;     // [total]
  int64_t nb_cap = 0;
  int32_t* d_row_of = nullptr;  // [points] slot of each point (rows by slot)
  int64_t row_of_cap = 0;
  int64_t* h_total = nullptr;   // pinned
  cudaStream_t last_stream = nullptr;
  int32_t host_error = 0;
};

namespace pn {
namespace {

__global__ void __launch_bounds__(256)
k_group_width(const int32_t* __restrict__ len, int64_t n_rows, int32_t max_nb,
              int32_t* __restrict__ width, int32_t* __restrict__ err) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t v = r < n_rows ? len[r] : 0;
  if (max_nb > 0 && v > max_nb) set_error(err, PN_ERR_CELL_FULL);
  int32_t m = v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && r < n_rows) width[r >> 5] = 32 * ((m + 3) & ~3);  // quads
}

__global__ void __launch_bounds__(256)
k_row_of(const int32_t* __restrict__ perm, const int32_t* __restrict__ n_slots_ptr,
         int64_t n_slots_max, int32_t* __restrict__ row_of) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_slots_max || k >= *n_slots_ptr) return;
  const int32_t i = perm[k];
  if (i >= 0) row_of[i] = (int32_t)k;
}

// Row lengths and point indices of the lists in point order (for the export).
__global__ void __launch_bounds__(256)
k_export_len(const int32_t* __restrict__ len, const int32_t* __restrict__ row_of, int64_t n,
             int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = len[row_of ? row_of[i] : i];
}

__global__ void __launch_bounds__(256)
k_export_rows(const int32_t* __restrict__ len, const int32_t* __restrict__ row_of,
              const int32_t* __restrict__ nb, const int64_t* __restrict__ grp,
              const int32_t* __restrict__ perm, int64_t n, const int64_t* __restrict__ off,
              int64_t capacity, int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || off[n] > capacity) return;  // nothing is written when the lists do not fit
  const int32_t r = row_of ? row_of[i] : (int32_t)i;
  const int32_t* row = nb + grp[r >> 5] + 4 * (r & 31);  // quads of 4 entries, 128 apart
  const int64_t o = off[i];
  for (int32_t t = 0; t < len[r]; ++t) out[o + t] = perm[row[128 * (t >> 2) + (t & 3)]];
}

__global__ void k_check_export(const int64_t* total, int64_t capacity, int32_t* err) {
  if (*total > capacity) set_error(err, PN_ERR_CAPACITY);
}

template <typename P>
int grow(P** p, int64_t* cap, int64_t need) {
  if (need <= *cap) return PN_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const int64_t n = std::max<int64_t>(need + need / 4, 64);
  if (cudaMalloc(p, sizeof(P) * n) != cudaSuccess) {
    cudaGetLastError();
    return PN_ERR_OUT_OF_MEMORY;
  }
  *cap = n;
  return PN_OK;
}

__global__ void k_fixed_groups(int64_t n_groups, int64_t group_size, int64_t* __restrict__ grp) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g <= n_groups) grp[g] = g * group_size;
}

void make_row_of(pn_precomputed* s, int64_t n_rows, cudaStream_t st) {
  pn_search* g = s->grid;
  const int32_t* n_slots = g->ovf_active ? g->d_ovf_start + g->n_total : g->d_start + g->n_total;
  k_row_of<<<div_up(n_rows, 256), 256, 0, st>>>(g->d_perm, n_slots, n_rows, s->d_row_of); count_launch();
}

// max_neighbors > 0: the reference's fixed capacity per point (its DynamicVectorOfVectors
// with max_neighbors rows, transposed), so one traversal writes the lists and their
// lengths, with no counting pass and no host synchronisation; a longer row is the
// "cell list is full" error, reported by the next synchronisation.
template <typename T>
int build_fixed(pn_precomputed* s, const T* x, int64_t n_x, const T* y, int64_t n_y,
                cudaStream_t st) {
  pn_search* g = s->grid;
  if (!g->initialized || g->is_template) return PN_ERR_NOT_INITIALIZED;
  const bool sorted = (const void*)x == (const void*)y && n_x == n_y && g->full_binned;
  const int64_t n_rows = sorted ? g->n_binned + (g->ovf_active ? g->cap : 0) : n_x;
  const int64_t n_groups = (n_rows + 31) / 32;
  const int64_t group_size = 32 * (int64_t)((s->max_neighbors + 3) & ~3);  // whole quads
  int rc = grow(&s->d_grp, &s->grp_cap, n_groups + 1);
  if (rc == PN_OK) rc = grow(&s->d_nb, &s->nb_cap, n_groups * group_size + 1);
  if (rc == PN_OK && sorted) rc = grow(&s->d_row_of, &s->row_of_cap, n_x + 1);
  if (rc != PN_OK) return rc;
  k_fixed_groups<<<div_up(n_groups + 1, 256), 256, 0, st>>>(n_groups, group_size, s->d_grp); count_launch();
  rc = lists_emit<T>(g, x, n_x, y, n_y, s->d_nb, s->d_grp, s->max_neighbors, s->d_len, st);
  if (rc != PN_OK) return rc;
  if (sorted) make_row_of(s, n_rows, st);
  s->ref = ListsRef{s->d_nb, s->d_grp, s->d_len, sorted ? s->d_row_of : nullptr,
                    sorted ? 1 : 0, n_rows};
  s->built = true;
  return cuda_status(cudaGetLastError());
}

// The lists of x against y (the internal search holds y).  Without a capacity, one host
// synchronisation: the total length decides the allocation, as the reference's resize! of
// the lists does.
template <typename T>
int build_lists(pn_precomputed* s, const T* x, int64_t n_x, const T* y, int64_t n_y,
                cudaStream_t st) {
  pn_search* g = s->grid;
  s->built = false;
  int rc = ensure_capacity(g, std::max(n_x, n_y));
  if (rc != PN_OK) return rc;
  const int64_t rows_max = std::max<int64_t>(n_x, g->n_binned + (g->ovf_active ? g->cap : 0));
  rc = grow(&s->d_len, &s->len_cap, rows_max + 1);
  if (rc == PN_OK) rc = grow(&s->d_grp, &s->grp_cap, rows_max / 32 + 2);
  if (rc == PN_OK) rc = grow(&s->d_width, &s->width_cap, rows_max / 32 + 2);
  if (rc != PN_OK) return rc;
  if (s->max_neighbors > 0) return build_fixed<T>(s, x, n_x, y, n_y, st);
  int32_t by_slot = 0;
  int64_t n_rows = 0;
  rc = lists_count<T>(g, x, n_x, y, n_y, s->d_len, &by_slot, &n_rows, st);
  if (rc != PN_OK) return rc;
  const int64_t n_groups = (n_rows + 31) / 32;
  if (n_rows > 0) {
    k_group_width<<<div_up(n_groups * 32, 256), 256, 0, st>>>(s->d_len, n_rows, s->max_neighbors,
                                                              s->d_width, g->d_err); count_launch();
  }
  rc = scan64(g, s->d_width, n_groups, s->d_grp, st);
  if (rc != PN_OK) return rc;
  if (cudaMemcpyAsync(s->h_total, s->d_grp + n_groups, sizeof(int64_t), cudaMemcpyDeviceToHost,
                      st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return PN_ERR_CUDA;
  const int rc_dev = pn_get_error(g, 0);
  if (rc_dev != PN_OK) return rc_dev;
  rc = grow(&s->d_nb, &s->nb_cap, *s->h_total + 1);
  if (rc != PN_OK) return rc;
  rc = lists_emit<T>(g, x, n_x, y, n_y, s->d_nb, s->d_grp, 0, nullptr, st);
  if (rc != PN_OK) return rc;
  if (by_slot) {
    rc = grow(&s->d_row_of, &s->row_of_cap, n_x + 1);
    if (rc != PN_OK) return rc;
    make_row_of(s, n_rows, st);
  }
  s->ref = ListsRef{s->d_nb, s->d_grp, s->d_len, by_slot ? s->d_row_of : nullptr, by_slot, n_rows};
  s->built = true;
  return cuda_status(cudaGetLastError());
}

int record(pn_precomputed* s, int rc, cudaStream_t st) {
  s->last_stream = st;
  if (s->grid) s->grid->last_stream = st;
  if (rc != PN_OK && s->host_error == 0) s->host_error = rc;
  return rc;
}

}  // namespace
}  // namespace pn

using namespace pn;

extern "C" {

static int pre_create(const pn_config* cfg, int64_t list_size, int32_t max_neighbors,
                      pn_precomputed** out) {
  if (!cfg || !out || max_neighbors < 0) return PN_ERR_INVALID_ARG;
  *out = nullptr;
  pn_precomputed* s = new (std::nothrow) pn_precomputed();
  if (!s) return PN_ERR_OUT_OF_MEMORY;
  int rc = list_size > 0 ? pn_create_spatial_hashing(cfg, list_size, &s->grid)
                         : pn_create(cfg, &s->grid);
  if (rc == PN_OK && cudaMallocHost(&s->h_total, sizeof(int64_t)) != cudaSuccess) {
    cudaGetLastError();
    rc = PN_ERR_OUT_OF_MEMORY;
  }
  if (rc != PN_OK) {
    if (s->grid) pn_destroy(s->grid);
    delete s;
    return rc;
  }
  s->max_neighbors = max_neighbors;
  s->dtype = cfg->dtype;
  s->ndims = cfg->ndims;
  *out = s;
  return PN_OK;
}

int pn_pre_create(const pn_config* cfg, int32_t max_neighbors, pn_precomputed** out) {
  PN_NVTX_RANGE("pn_pre_create");
  return pre_create(cfg, 0, max_neighbors, out);
}

int pn_pre_create_spatial_hashing(const pn_config* cfg, int64_t list_size,
                                  int32_t max_neighbors, pn_precomputed** out) {
  PN_NVTX_RANGE("pn_pre_create_spatial_hashing");
  if (list_size < 1) return PN_ERR_INVALID_ARG;
  return pre_create(cfg, list_size, max_neighbors, out);
}

int pn_pre_destroy(pn_precomputed* s) {
  if (!s) return PN_OK;
  void* ptrs[] = {s->d_len, s->d_width, s->d_grp, s->d_nb, s->d_row_of};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->h_total) cudaFreeHost(s->h_total);
  if (s->grid) pn_destroy(s->grid);
  delete s;
  return PN_OK;
}

int pn_pre_initialize(pn_precomputed* s, const void* x, int64_t n_x, const void* y,
                      int64_t n_y, const int32_t* eachindex_y, int64_t n_eachindex_y,
                      pn_stream_t stream) {
  PN_NVTX_RANGE("pn_pre_initialize");
  if (!s) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  // "this neighborhood search does not support inactive points" (nhs_precomputed.jl:136)
  if (eachindex_y != nullptr && n_eachindex_y != n_y) return record(s, PN_ERR_INVALID_ARG, st);
  int rc = pn_initialize(s->grid, y, n_y, nullptr, 0, stream);
  if (rc == PN_OK)
    rc = s->dtype == PN_FLOAT64
             ? build_lists<double>(s, (const double*)x, n_x, (const double*)y, n_y, st)
             : build_lists<float>(s, (const float*)x, n_x, (const float*)y, n_y, st);
  return record(s, rc, st);
}

int pn_pre_update(pn_precomputed* s, const void* x, int64_t n_x, const void* y, int64_t n_y,
                  const int32_t* eachindex_y, int64_t n_eachindex_y, int32_t points_moving_x,
                  int32_t points_moving_y, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_pre_update");
  if (!s) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (eachindex_y != nullptr && n_eachindex_y != n_y) return record(s, PN_ERR_INVALID_ARG, st);
  if (!s->built) return record(s, PN_ERR_NOT_INITIALIZED, st);
  int rc = pn_update(s->grid, y, n_y, nullptr, 0, points_moving_y, stream);
  // nhs_precomputed.jl:160-164: the lists are rebuilt unless both point sets are static
  if (rc == PN_OK && (points_moving_x || points_moving_y))
    rc = s->dtype == PN_FLOAT64
             ? build_lists<double>(s, (const double*)x, n_x, (const double*)y, n_y, st)
             : build_lists<float>(s, (const float*)x, n_x, (const float*)y, n_y, st);
  return record(s, rc, st);
}

int pn_pre_foreach_point_neighbor(pn_precomputed* s, int32_t functor, const void* x,
                                  int64_t n_x, const void* y, int64_t n_y,
                                  const int32_t* points, int64_t n_points, const void* params,
                                  pn_stream_t stream) {
  PN_NVTX_RANGE("pn_pre_foreach_point_neighbor");
  if (!s) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (!s->built) return record(s, PN_ERR_NOT_INITIALIZED, st);
  const int rc = s->dtype == PN_FLOAT64
                     ? pn::foreach<double>(s->grid, functor, (const double*)x, n_x,
                                           (const double*)y, n_y, points, n_points, params, st,
                                           &s->ref)
                     : pn::foreach<float>(s->grid, functor, (const float*)x, n_x,
                                          (const float*)y, n_y, points, n_points, params, st,
                                          &s->ref);
  return record(s, rc, st);
}

int pn_pre_neighbor_lists(pn_precomputed* s, int32_t sort, int64_t* offsets, int32_t* neighbors,
                          int64_t capacity, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_pre_neighbor_lists");
  if (!s || !offsets) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (!s->built) return record(s, PN_ERR_NOT_INITIALIZED, st);
  pn_search* g = s->grid;
  const int64_t n = s->ref.by_slot ? g->n_y : s->ref.n_rows;
  int rc = ensure_qcount(g, n);
  if (rc != PN_OK) return record(s, rc, st);
  const int b = div_up(n, 256);
  if (b > 0) {
    k_export_len<<<b, 256, 0, st>>>(s->d_len, s->ref.row_of, n, g->d_qcount); count_launch();
  }
  rc = scan64(g, g->d_qcount, n, offsets, st);
  if (rc == PN_OK && neighbors && capacity > 0 && b > 0) {
    k_check_export<<<1, 1, 0, st>>>(offsets + n, capacity, g->d_err); count_launch();
    k_export_rows<<<b, 256, 0, st>>>(s->d_len, s->ref.row_of, s->d_nb, s->d_grp, g->d_perm, n,
                                     offsets, capacity, neighbors); count_launch();
    if (sort) rc = sort_rows(g, offsets, n, neighbors, capacity, st);
  }
  return record(s, rc != PN_OK ? rc : cuda_status(cudaGetLastError()), st);
}

int pn_pre_sync(pn_precomputed* s) {
  if (!s) return PN_ERR_INVALID_ARG;
  const int rc = pn_sync(s->grid);
  const int h = s->host_error;
  s->host_error = 0;
  return h ? h : rc;
}

int pn_pre_requires_update(const pn_precomputed* s, int32_t out[2]) {
  if (!s || !out) return PN_ERR_INVALID_ARG;
  out[0] = 1;  // requires_update(::PrecomputedNeighborhoodSearch) = (true, true)
  out[1] = 1;
  return PN_OK;
}

}  // extern "C"
