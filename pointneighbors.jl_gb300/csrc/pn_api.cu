// pn_api.cu -- the C ABI of libpn_gb300 (include/pn_gb300.h): construction of a
// GridNeighborhoodSearch over a FullGridCellList, its device scratch, and dispatch by dtype.
//
// Geometry follows the reference constructors exactly, in the element type T:
//   FullGridCellList (full_grid.jl:48-82): corners padded by T(1001)/T(1000) * r,
//     n = ceil(Int, (max - min) / r) cells per dimension, column-major linear indices;
//   GridNeighborhoodSearch (nhs_grid.jl:77-129): with a PeriodicBox,
//     n_cells = floor(Int, (size + 10 eps()) / r) in Float64, cell_size = size / n_cells in T,
//     at least 3 cells per dimension.
// With PN_FLAG_FLOAT32_SEARCH (Float64 coordinates, Float32 search radius) the corners are
// Float64 padded by the Float32 value Float32(1001 // 1000) * r, the cell count divides the
// Float64 extent by the widened radius, and the PeriodicBox is Float32 like the radius
// (nhs_grid.jl:107-110): its size and cell size are Float32 values.
// This file is compiled with -ffp-contract=off for the host compiler as well, so these T
// expressions are rounded exactly like Julia's.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "pn_internal.cuh"

namespace pn {

int cuda_status(cudaError_t e) { return e == cudaSuccess ? PN_OK : PN_ERR_CUDA; }

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static void free_points(pn_search* s) {
  void* ptrs[] = {s->d_cell_of, s->d_slot_of, s->d_tmp_perm, s->d_perm, s->d_cell_of_slot,
                  s->d_pos,     s->d_pa,      s->d_pb,       s->d_main_perm, s->d_ovf_list,
                  s->d_ovf_cell, s->d_ovf_slot, s->d_pos32, s->d_pos32lo, s->d_xkey,
                  s->d_pos32lo2, s->d_sdf};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  s->d_xkey = s->d_pos32lo2 = s->d_sdf = nullptr;
  s->d_cell_of = s->d_slot_of = s->d_tmp_perm = s->d_perm = s->d_cell_of_slot = nullptr;
  s->d_main_perm = s->d_ovf_list = s->d_ovf_cell = s->d_ovf_slot = nullptr;
  s->d_pos = s->d_pa = s->d_pb = nullptr;
  s->d_pos32 = s->d_pos32lo = nullptr;
  s->cap = 0;
}

// Grow the point arrays to hold n points (2n slots).  Growing discards the cell list, so
// it only happens at the start of a build.
int ensure_capacity(pn_search* s, int64_t n) {
  if (n <= s->cap) return PN_OK;
  if (n > (int64_t)INT32_MAX / 2) return PN_ERR_INVALID_ARG;  // Int32 point indices
  free_points(s);
  const int64_t cap = n + n / 8 + 1024;
  const size_t tb = s->dtype == PN_FLOAT64 ? 8 : 4;
  const size_t i4 = sizeof(int32_t);
  bool ok = true;
  auto alloc = [&](void** p, size_t bytes) {
    if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false;
  };
  alloc((void**)&s->d_cell_of, i4 * cap);
  alloc((void**)&s->d_slot_of, i4 * cap);
  // Slot arrays: main and overflow slots, plus SLOT_PAD slots that a candidate scan may
  // read past the end of a run (those reads are masked off).
  const int64_t slots = 2 * cap + SLOT_PAD;
  alloc((void**)&s->d_tmp_perm, i4 * slots);
  alloc((void**)&s->d_perm, i4 * slots);
  alloc((void**)&s->d_cell_of_slot, i4 * slots);
  alloc(&s->d_pos, tb * 4 * slots);
  alloc(&s->d_pa, tb * 4 * slots);
  alloc(&s->d_pb, tb * 4 * slots);
  const bool split3 = s->dtype == PN_FLOAT64 && !s->hashed && !s->mixed;
  if (s->mixed || split3) alloc((void**)&s->d_pos32, sizeof(float) * 4 * slots);
  if (s->mixed || split3) alloc((void**)&s->d_pos32lo, sizeof(float) * 4 * slots);
  if (split3 && s->ndims == 3) {
    alloc((void**)&s->d_pos32lo2, sizeof(float) * 4 * slots);
    alloc((void**)&s->d_sdf, sizeof(float) * 12 * slots);
  }
  if (s->dtype == PN_FLOAT32 && !s->mixed && !s->hashed &&
      s->cfg.update_strategy == PN_PARALLEL_INCREMENTAL_UPDATE)
    alloc((void**)&s->d_xkey, sizeof(float) * slots);
  alloc((void**)&s->d_main_perm, i4 * cap);
  alloc((void**)&s->d_ovf_list, i4 * cap);
  alloc((void**)&s->d_ovf_cell, i4 * cap);
  alloc((void**)&s->d_ovf_slot, i4 * cap);
  if (!ok) {
    free_points(s);
    cudaGetLastError();
    return PN_ERR_OUT_OF_MEMORY;
  }
  s->cap = cap;
  s->initialized = false;
  s->ovf_active = false;
  s->main_perm_valid = false;
  return PN_OK;
}

int ensure_sum_part(pn_search* s) {
  if (s->d_sum_part) return PN_OK;
  if (cudaMalloc(&s->d_sum_part, sizeof(double) * SUM_BLOCKS) != cudaSuccess) {
    cudaGetLastError();
    s->d_sum_part = nullptr;
    return PN_ERR_OUT_OF_MEMORY;
  }
  return PN_OK;
}

int ensure_qcount(pn_search* s, int64_t n) {
  if (n <= s->qcount_cap) return PN_OK;
  if (s->d_qcount) cudaFree(s->d_qcount);
  s->d_qcount = nullptr;
  s->qcount_cap = 0;
  if (cudaMalloc(&s->d_qcount, sizeof(int32_t) * (n + 1)) != cudaSuccess) {
    cudaGetLastError();
    return PN_ERR_OUT_OF_MEMORY;
  }
  s->qcount_cap = n;
  return PN_OK;
}

// T: the coordinates' type (corners, cells); R: the search radius's (and PeriodicBox's) type.
template <typename T, typename R>
static int geometry(pn_search* s) {
  pn_config& c = s->cfg;
  const int d = c.ndims;
  const R r = (R)c.search_radius;
  const R pad = (R)((R)1001 / (R)1000) * r;  // `1001 // 1000 * search_radius`
  s->radius = (double)r;
  s->is_template = (double)r < 2.220446049250313e-16 ? 1 : 0;  // search_radius < eps()
  int64_t total = 1;
  for (int k = 0; k < 3; ++k) {
    s->grid_size[k] = 1;
    s->n_cells[k] = -1;
    s->min_pad[k] = s->max_pad[k] = 0.0;
    s->cell_size[k] = 1.0;
    s->box_size[k] = 0.0;
  }
  for (int k = 0; k < d; ++k) {
    const T mn = (T)c.min_corner[k], mx = (T)c.max_corner[k];
    // from a cell list's stored state: the corners are padded already
    const T mnp = s->from_grid ? mn : (T)(mn - (T)pad);
    const T mxp = s->from_grid ? mx : (T)(mx + (T)pad);
    s->min_pad[k] = (double)mnp;
    s->max_pad[k] = (double)mxp;
    s->cell_size[k] = (double)r;
    if (s->from_grid) {
      // size(linear_indices): zero for a template, else at least one cell
      const int64_t gk = s->given_grid[k];
      if (s->is_template ? gk != 0 : (gk < 1 || gk > (int64_t)INT32_MAX - 1))
        return PN_ERR_INVALID_ARG;
      if (!s->is_template) {
        s->grid_size[k] = gk;
        total *= gk;
        if (total > (int64_t)INT32_MAX - 1) return PN_ERR_INVALID_ARG;
      }
    } else if (!s->is_template) {
      const T q = (T)((T)(mxp - mnp) / (T)r);
      if (!(q >= (T)1) || !(q < (T)2147483647.0)) return PN_ERR_INVALID_ARG;
      s->grid_size[k] = (int64_t)std::ceil((double)q);
      total *= s->grid_size[k];
      if (total > (int64_t)INT32_MAX - 1) return PN_ERR_INVALID_ARG;
    }
  }
  s->n_total = s->is_template ? 0 : (int32_t)total;
  s->periodic = 0;
  if (c.periodic && !s->is_template) {
    s->periodic = 1;
    for (int k = 0; k < d; ++k) {
      c.periodic_min[k] = (double)(R)c.periodic_min[k];  // the box is in R
      c.periodic_max[k] = (double)(R)c.periodic_max[k];
      const R size = (R)((R)c.periodic_max[k] - (R)c.periodic_min[k]);
      s->box_size[k] = (double)size;
      const double nc = std::floor(((double)size + 10.0 * 2.220446049250313e-16) / (double)r);
      if (!(nc >= 3.0)) return PN_ERR_INVALID_ARG;  // "needs at least 3 cells"
      if (nc > 1e9) return PN_ERR_INVALID_ARG;
      s->n_cells[k] = (int64_t)nc;
      s->cell_size[k] = (double)(R)(size / (R)s->n_cells[k]);
      // The periodic cells 2..n_cells+1 (and the stencil's wrap-around neighbours) must be
      // cells of the padded grid; the reference's tests always build the cell list over the
      // periodic box, which gives n_cells + 3 <= grid_size.
      if (s->n_cells[k] + 2 > s->grid_size[k]) return PN_ERR_INVALID_ARG;
    }
  }
  return PN_OK;
}

// GridNeighborhoodSearch over a SpatialHashingCellList: no corners; the cell size is r, or
// the periodic one as above (nhs_grid.jl:102-124); n_total = list_size hash lists.
template <typename R>
static int geometry_hash(pn_search* s) {
  pn_config& c = s->cfg;
  const int d = c.ndims;
  const R r = (R)c.search_radius;
  s->radius = (double)r;
  s->is_template = (double)r < 2.220446049250313e-16 ? 1 : 0;
  if (s->list_size < 1 || s->list_size > (int64_t)INT32_MAX - 1) return PN_ERR_INVALID_ARG;
  for (int k = 0; k < 3; ++k) {
    s->grid_size[k] = 1;
    s->n_cells[k] = -1;
    s->min_pad[k] = s->max_pad[k] = 0.0;
    s->cell_size[k] = k < d ? (double)r : 1.0;
    s->box_size[k] = 0.0;
  }
  s->n_total = s->is_template ? 0 : (int32_t)s->list_size;
  s->periodic = 0;
  if (c.periodic && !s->is_template) {
    s->periodic = 1;
    for (int k = 0; k < d; ++k) {
      c.periodic_min[k] = (double)(R)c.periodic_min[k];
      c.periodic_max[k] = (double)(R)c.periodic_max[k];
      const R size = (R)((R)c.periodic_max[k] - (R)c.periodic_min[k]);
      s->box_size[k] = (double)size;
      const double nc = std::floor(((double)size + 10.0 * 2.220446049250313e-16) / (double)r);
      if (!(nc >= 3.0)) return PN_ERR_INVALID_ARG;  // "needs at least 3 cells"
      if (nc > 1e9) return PN_ERR_INVALID_ARG;
      s->n_cells[k] = (int64_t)nc;
      s->cell_size[k] = (double)(R)(size / (R)s->n_cells[k]);
    }
  }
  return PN_OK;
}

static int geometry_for(pn_search* s) {
  if (s->cfg.flags & ~PN_FLAG_FLOAT32_SEARCH) return PN_ERR_INVALID_ARG;
  s->mixed = (s->cfg.flags & PN_FLAG_FLOAT32_SEARCH) ? 1 : 0;
  if (s->mixed && s->dtype != PN_FLOAT64) return PN_ERR_INVALID_ARG;
  if (s->hashed) {
    if (s->cfg.update_strategy != PN_PARALLEL_UPDATE) return PN_ERR_INVALID_ARG;
    return (s->mixed || s->dtype == PN_FLOAT32) ? geometry_hash<float>(s)
                                                : geometry_hash<double>(s);
  }
  if (s->mixed) return geometry<double, float>(s);
  return s->dtype == PN_FLOAT64 ? geometry<double, double>(s) : geometry<float, float>(s);
}

// list_size > 0: a SpatialHashingCellList with that many lists, else a FullGridCellList;
// grid (FullGridCellList only): the cell list's own state (padded corners in cfg, cells per
// dimension here) instead of the constructor's arguments.
static int create(const pn_config* cfg, int64_t list_size, pn_search** out,
                  const int64_t* grid = nullptr) {
  if (!cfg || !out) return PN_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->ndims < 1 || cfg->ndims > 3) return PN_ERR_INVALID_ARG;
  if (cfg->dtype != PN_FLOAT32 && cfg->dtype != PN_FLOAT64) return PN_ERR_INVALID_ARG;
  if (cfg->update_strategy != PN_PARALLEL_UPDATE &&
      cfg->update_strategy != PN_PARALLEL_INCREMENTAL_UPDATE)
    return PN_ERR_INVALID_ARG;
  if (!(cfg->search_radius >= 0.0) || cfg->max_points_per_cell < 0 || cfg->n_points < 0)
    return PN_ERR_INVALID_ARG;
  pn_search* s = new (std::nothrow) pn_search();
  if (!s) return PN_ERR_OUT_OF_MEMORY;
  s->cfg = *cfg;
  s->ndims = cfg->ndims;
  s->dtype = cfg->dtype;
  s->hashed = list_size > 0 ? 1 : 0;
  s->list_size = list_size > 0 ? list_size : 0;
  if (grid != nullptr) {
    s->from_grid = 1;
    for (int k = 0; k < 3; ++k) s->given_grid[k] = k < cfg->ndims ? grid[k] : 0;
  }
  int rc = geometry_for(s);
  if (rc != PN_OK) {
    delete s;
    return rc;
  }
  // d_err: [0] sticky error, [1] a point outside the periodic box, [2] incremental-update
  // decision, [3] cells not sorted by x, [4] some query needs the pair cache's fallback,
  // [5] largest cell of the last build, [6] max_points_per_cell exceeded, [8] [9] site and
  // index of the first bounds failure (bounds-checked build)
  bool ok = cudaMalloc(&s->d_err, sizeof(int32_t) * pn::ERR_WORDS) == cudaSuccess;
  ok = ok && cudaMemset(s->d_err, 0, sizeof(int32_t) * pn::ERR_WORDS) == cudaSuccess;
  ok = ok && cudaMallocHost(&s->h_ovf_n, sizeof(int32_t)) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&s->ev_ovf, cudaEventDisableTiming) == cudaSuccess;
  if (ok && !s->is_template) {
    const int64_t nt = s->n_total;
    s->scan_tiles = div_up(nt, 2048);
    ok = cudaMalloc(&s->d_counts, sizeof(int32_t) * nt) == cudaSuccess &&
         cudaMalloc(&s->d_start, sizeof(int32_t) * (nt + 1)) == cudaSuccess &&
         cudaMalloc(&s->d_ovf_counts, sizeof(int32_t) * nt) == cudaSuccess &&
         cudaMalloc(&s->d_ovf_start, sizeof(int32_t) * (nt + 1)) == cudaSuccess &&
         cudaMalloc(&s->d_ovf_n, sizeof(int32_t) * 4) == cudaSuccess &&
         cudaMalloc(&s->d_scan_state, sizeof(unsigned long long) * (s->scan_tiles + 1)) == cudaSuccess;
    if (ok && !s->hashed && !s->mixed && s->dtype == PN_FLOAT32 &&
        s->cfg.update_strategy == PN_PARALLEL_INCREMENTAL_UPDATE) {
      ok = cudaMalloc(&s->d_cell_delta, sizeof(float) * nt) == cudaSuccess &&
           cudaMemset(s->d_cell_delta, 0, sizeof(float) * nt) == cudaSuccess;
    }
    if (ok && s->hashed)
      ok = cudaMalloc(&s->d_hbucket, sizeof(int32_t) * (nt + 1)) == cudaSuccess &&
           cudaMalloc(&s->d_hbbox, sizeof(int32_t) * 6) == cudaSuccess &&
           cudaMallocHost(&s->h_hbbox, sizeof(int32_t) * 6) == cudaSuccess;
    if (ok && cfg->n_points > 0) ok = ensure_capacity(s, cfg->n_points) == PN_OK;
  }
  if (!ok) {
    cudaGetLastError();
    pn_destroy(s);
    return PN_ERR_OUT_OF_MEMORY;
  }
  *out = s;
  return PN_OK;
}

// 8 independent FMA chains per thread (enough to cover the FMA latency with 8 resident
// blocks of 256 threads per SM); the multipliers stay near 1 so the values stay finite.
static __global__ void __launch_bounds__(256) k_fma_probe(float* __restrict__ out, int32_t iters) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) v[c] = 1.0f + 1e-7f * (float)(t + c);
  const float m = 0.9999999f, a = 1e-8f;
  for (int32_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = fmaf(v[c], m, a);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += v[c];
  out[t] = s;
}

static int record(pn_search* s, int rc, cudaStream_t st) {
  s->last_stream = st;
  if (rc != PN_OK && s->host_error == 0) s->host_error = rc;
  return rc;
}

}  // namespace pn

using namespace pn;

extern "C" {

int pn_abi_version(void) { return PN_ABI_VERSION; }

unsigned long long pn_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int pn_fma_probe(float* out, int32_t iters, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_fma_probe");
  if (!out || iters <= 0) return PN_ERR_INVALID_ARG;
  k_fma_probe<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(out, iters);
  count_launch();
  return cuda_status(cudaGetLastError());
}

int pn_selftest_bounded_wait(pn_stream_t stream) {
  PN_NVTX_RANGE("pn_selftest_bounded_wait");
  return selftest_bounded_wait((cudaStream_t)stream);
}

int pn_create(const pn_config* cfg, pn_search** out) {
  PN_NVTX_RANGE("pn_create");
  return create(cfg, 0, out);
}

int pn_create_spatial_hashing(const pn_config* cfg, int64_t list_size, pn_search** out) {
  PN_NVTX_RANGE("pn_create_spatial_hashing");
  if (list_size < 1) return PN_ERR_INVALID_ARG;
  return create(cfg, list_size, out);
}

int pn_create_from_grid(const pn_config* cfg, const int64_t* grid_size, pn_search** out) {
  PN_NVTX_RANGE("pn_create_from_grid");
  if (!grid_size) return PN_ERR_INVALID_ARG;
  return create(cfg, 0, out, grid_size);
}

int pn_copy_search(const pn_search* tmpl, double search_radius, int64_t n_points,
                   pn_search** out) {
  PN_NVTX_RANGE("pn_copy_search");
  if (!tmpl) return PN_ERR_INVALID_ARG;
  pn_config c = tmpl->cfg;
  c.search_radius = search_radius;
  c.n_points = n_points;
  // copy_cell_list (full_grid.jl:179-185) hands the template's stored corners -- padded by
  // the template's radius, i.e. not at all for a template -- to the constructor, which pads
  // them by the new radius
  if (!tmpl->hashed) {
    for (int k = 0; k < tmpl->ndims; ++k) {
      c.min_corner[k] = tmpl->min_pad[k];
      c.max_corner[k] = tmpl->max_pad[k];
    }
  }
  const int rc = create(&c, tmpl->list_size, out);
  if (rc == PN_OK) (*out)->rebuild_fraction = tmpl->rebuild_fraction;
  return rc;
}

int pn_set_pair_cache(pn_search* s, int32_t max_neighbors) {
  if (!s || max_neighbors < 0) return PN_ERR_INVALID_ARG;
  s->pc_cap = max_neighbors;
  s->pc_valid = false;
  return PN_OK;
}

int pn_set_rebuild_fraction(pn_search* s, double fraction) {
  if (!s || !(fraction >= 0.0)) return PN_ERR_INVALID_ARG;
  s->rebuild_fraction = fraction;
  return PN_OK;
}

int pn_destroy(pn_search* s) {
  if (!s) return PN_OK;
  free_points(s);
  void* ptrs[] = {s->d_err,       s->d_counts,     s->d_start,     s->d_scan_state,
                  s->d_cell_delta,
                  s->d_ovf_counts, s->d_ovf_start,  s->d_ovf_n,     s->d_qcount,
                  s->d_part,       s->d_sort_tmp,   s->d_sum_part,  s->d_pc_b0,
                  s->d_pc_mask,    s->d_pc_ob0,     s->d_pc_omask,  s->d_hkey_t,
                  s->d_hkey_tmp,   s->d_hkey,
                  s->d_hcellidx,   s->d_hcell,      s->d_hbucket,   s->d_hscan_state,
                  s->d_hbbox};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->h_ovf_n) cudaFreeHost(s->h_ovf_n);
  if (s->h_hbbox) cudaFreeHost(s->h_hbbox);
  if (s->ev_ovf) cudaEventDestroy(s->ev_ovf);
  delete s;
  return PN_OK;
}

int pn_initialize(pn_search* s, const void* y, int64_t n_y, const int32_t* eachindex_y,
                  int64_t n_eachindex_y, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_initialize");
  if (!s || n_y < 0 || (n_y > 0 && !y) || (eachindex_y && n_eachindex_y < 0))
    return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (s->is_template) {
    // initialize_grid! returns early for search_radius < eps() (nhs_grid.jl:263-267).
    s->initialized = false;
    return record(s, PN_OK, st);
  }
  int rc;
  if (s->hashed)
    rc = s->dtype == PN_FLOAT64
             ? build_hash<double>(s, (const double*)y, n_y, eachindex_y, n_eachindex_y, st)
             : build_hash<float>(s, (const float*)y, n_y, eachindex_y, n_eachindex_y, st);
  else
    rc = s->dtype == PN_FLOAT64
             ? build<double>(s, (const double*)y, n_y, eachindex_y, n_eachindex_y, st)
             : build<float>(s, (const float*)y, n_y, eachindex_y, n_eachindex_y, st);
  if (rc == PN_OK) {
    s->initialized = true;
    s->full_binned = eachindex_y == nullptr;
    s->n_y = n_y;
    s->y_ptr = y;
  }
  return record(s, rc, st);
}

int pn_update(pn_search* s, const void* y, int64_t n_y, const int32_t* eachindex_y,
              int64_t n_eachindex_y, int32_t points_moving_y, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_update");
  if (!s) return PN_ERR_INVALID_ARG;
  // update! is a no-op when the neighbour points do not move (nhs_grid.jl:289).
  if (!points_moving_y) return PN_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (s->cfg.update_strategy == PN_PARALLEL_UPDATE || s->is_template)
    return pn_initialize(s, y, n_y, eachindex_y, n_eachindex_y, stream);
  // ParallelIncrementalUpdate: no inactive points (nhs_grid.jl:414-417).
  if (eachindex_y != nullptr) return record(s, PN_ERR_INVALID_ARG, st);
  if (!s->initialized) return record(s, PN_ERR_NOT_INITIALIZED, st);
  if (n_y != s->n_y || !s->full_binned) return record(s, PN_ERR_INVALID_ARG, st);
  // The choice between overflow lists and a full rebuild is made on the device, after the
  // movers are counted (update_incremental); the host only refreshes its statistics.
  if (s->ovf_pending && cudaEventQuery(s->ev_ovf) == cudaSuccess) {
    s->n_ovf = *s->h_ovf_n;
    s->ovf_pending = false;
  }
  int rc = s->dtype == PN_FLOAT64 ? update_incremental<double>(s, (const double*)y, n_y, st)
                                  : update_incremental<float>(s, (const float*)y, n_y, st);
  if (rc == PN_OK) s->y_ptr = y;
  return record(s, rc, st);
}

int pn_foreach_point_neighbor(pn_search* s, int32_t functor, const void* x, int64_t n_x,
                              const void* y, int64_t n_y, const int32_t* points,
                              int64_t n_points, const void* params, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_foreach_point_neighbor");
  if (!s) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = s->dtype == PN_FLOAT64
               ? pn::foreach<double>(s, functor, (const double*)x, n_x, (const double*)y, n_y,
                                     points, n_points, params, st)
               : pn::foreach<float>(s, functor, (const float*)x, n_x, (const float*)y, n_y,
                                    points, n_points, params, st);
  return record(s, rc, st);
}

int32_t pn_build_flags(void) {
#ifdef PN_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

int pn_bounds_failure(pn_search* s, int32_t* site, int32_t* index) {
  if (!s || !site || !index) return PN_ERR_INVALID_ARG;
  int32_t w[2] = {0, 0};
  if (cudaMemcpy(w, s->d_err + pn::ERR_BC_SITE, sizeof(w), cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return PN_ERR_CUDA;
  *site = w[0];
  *index = w[1];
  return PN_OK;
}

int pn_get_error(pn_search* s, int32_t clear) {
  if (!s) return PN_ERR_INVALID_ARG;
  int32_t e = 0;
  if (cudaMemcpy(&e, s->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PN_ERR_CUDA;
  int rc = s->host_error ? s->host_error : e;
  if (clear) {
    s->host_error = 0;
    if (e) cudaMemset(s->d_err, 0, sizeof(int32_t));
  }
  return rc;
}

int pn_sync(pn_search* s) {
  if (!s) return PN_ERR_INVALID_ARG;
  cudaError_t ce = cudaStreamSynchronize(s->last_stream);
  if (ce != cudaSuccess) return PN_ERR_CUDA;
  return pn_get_error(s, 1);
}

const char* pn_status_string(int32_t status) {
  switch (status) {
    case PN_OK: return "ok";
    case PN_ERR_OUT_OF_DOMAIN:
      return "particle coordinates are NaN or outside the domain bounds of the cell list";
    case PN_ERR_INVALID_ARG: return "invalid argument";
    case PN_ERR_CUDA: return "CUDA error";
    case PN_ERR_TIMEOUT: return "a device-side wait timed out";
    case PN_ERR_UNSUPPORTED_FUNCTOR: return "unsupported pair function";
    case PN_ERR_CELL_FULL: return "cell list is full. Use a larger `max_points_per_cell`.";
    case PN_ERR_NOT_INITIALIZED: return "`search_radius` is not defined or the search is not initialized";
    case PN_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PN_ERR_BOUNDS: return "BoundsError: a query point's neighbouring cells are outside the grid";
    case PN_ERR_CAPACITY: return "neighbour-list buffer too small";
    case PN_ERR_SCRATCH_LIMIT:
      return "the problem needs more than the 4 MiB fixed scratch of the no-allocation entry "
             "point (4 bytes per grid cell + 12 bytes per point + 20 bytes)";
    case PN_ERR_INDEX: return "a device index out of range (bounds-checked build)";
    default: return "unknown status";
  }
}

int pn_requires_update(const pn_search* s, int32_t out[2]) {
  if (!s || !out) return PN_ERR_INVALID_ARG;
  out[0] = 0;
  out[1] = 1;
  return PN_OK;
}

int pn_get_grid_info(const pn_search* s, pn_grid_info* out) {
  if (!s || !out) return PN_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  out->ndims = s->ndims;
  out->dtype = s->dtype;
  out->periodic = s->periodic;
  out->is_template = s->is_template;
  for (int k = 0; k < 3; ++k) {
    out->grid_size[k] = k < s->ndims ? s->grid_size[k] : 0;
    out->n_cells[k] = k < s->ndims ? s->n_cells[k] : 0;
    out->min_corner[k] = s->min_pad[k];
    out->max_corner[k] = s->max_pad[k];
    out->cell_size[k] = s->cell_size[k];
  }
  out->search_radius = s->radius;
  out->list_size = s->list_size;
  out->n_binned = s->n_binned;
  // the mover count of the last update, once its asynchronous read-back has landed
  out->n_overflow = (s->ovf_pending && cudaEventQuery(s->ev_ovf) == cudaSuccess)
                        ? (int64_t)*s->h_ovf_n : s->n_ovf;
  return PN_OK;
}

static int compute_geometry(const pn_config* cfg, const int64_t* grid, pn_grid_info* out) {
  if (!cfg || !out || cfg->ndims < 1 || cfg->ndims > 3) return PN_ERR_INVALID_ARG;
  if (cfg->dtype != PN_FLOAT32 && cfg->dtype != PN_FLOAT64) return PN_ERR_INVALID_ARG;
  pn_search tmp;
  tmp.cfg = *cfg;
  tmp.ndims = cfg->ndims;
  tmp.dtype = cfg->dtype;
  tmp.hashed = 0;
  tmp.list_size = 0;
  if (grid != nullptr) {
    tmp.from_grid = 1;
    for (int k = 0; k < 3; ++k) tmp.given_grid[k] = k < cfg->ndims ? grid[k] : 0;
  }
  int rc = geometry_for(&tmp);
  if (rc != PN_OK) return rc;
  return pn_get_grid_info(&tmp, out);
}

int pn_compute_geometry(const pn_config* cfg, pn_grid_info* out) {
  return compute_geometry(cfg, nullptr, out);
}

int pn_compute_geometry_from_grid(const pn_config* cfg, const int64_t* grid_size,
                                  pn_grid_info* out) {
  if (!grid_size) return PN_ERR_INVALID_ARG;
  return compute_geometry(cfg, grid_size, out);
}

int pn_cell_coords(pn_search* s, const void* x, int64_t n, int64_t* out, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_cell_coords");
  if (!s || n < 0 || (n > 0 && (!x || !out))) return PN_ERR_INVALID_ARG;
  if (s->is_template) return PN_ERR_NOT_INITIALIZED;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = s->dtype == PN_FLOAT64 ? cell_coords<double>(s, (const double*)x, n, out, st)
                                  : cell_coords<float>(s, (const float*)x, n, out, st);
  return record(s, rc, st);
}

int pn_export_cells(pn_search* s, int32_t* counts, int32_t* points, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_export_cells");
  if (!s || !counts) return PN_ERR_INVALID_ARG;
  if (!s->initialized) return PN_ERR_NOT_INITIALIZED;
  cudaStream_t st = (cudaStream_t)stream;
  if (s->hashed) return record(s, export_hash_lists(s, counts, points, st), st);
  return record(s, export_cells(s, counts, points, st), st);
}

}  // extern "C"
