/*
 * pn_gb300.h -- C ABI of libpn_gb300.so: PointNeighbors.jl's GridNeighborhoodSearch over a
 * FullGridCellList, implemented as CUDA kernels for GB300 (sm_103a).
 *
 * The entry points are what a Julia `ccall` binding of the reference's API for this path
 * needs.  Each declaration cites the reference function it replaces (paths inside
 * PointNeighbors.jl v0.6.7).
 *
 * Conventions
 *  - Coordinates use the reference's memory layout: a Julia `T[d, N]` column-major matrix,
 *    i.e. point-major (x1 y1 z1 x2 y2 z2 ...).  T is Float32 or Float64 and equals the
 *    eltype of the search radius and of the corners (pn_config.dtype).
 *  - All array arguments are DEVICE pointers owned by the caller.  Point indices are
 *    0-based at this interface (the Julia binding subtracts 1).
 *  - Calls are asynchronous on the given stream (a cudaStream_t; NULL = default stream).
 *    Kernel-side errors (a point outside the grid, a full cell, ...) are recorded in a
 *    sticky per-search error word: pn_sync() waits for the stream and returns it.
 *  - A search is not thread-safe: one host thread at a time per handle.
 *  - Scratch memory (cell arrays, the cell-sorted copy of the points) is owned by the
 *    handle and allocated by pn_create / grown on demand.
 *  - The pair function is a compile-time functor picked by `functor` (pn_functor); an
 *    arbitrary Julia closure cannot be compiled into the library, and there is no CPU
 *    fallback: unknown functors return PN_ERR_UNSUPPORTED_FUNCTOR.
 *  - Float64 searches decide every neighbour by the reference's Float64 test.  For the 3D
 *    WCSPH density and force of a Float64 search without a periodic box, the pair
 *    arithmetic itself runs in double-float (pairs of Float32 numbers, about 48 significant
 *    bits; GB300's Float64 units are slow): the sums agree with Float64 sums to about 1e-14
 *    of the sum of their terms' magnitudes.  The other Float64 pair functions and periodic
 *    or 2D searches compute in Float64.
 */
#ifndef PN_GB300_H
#define PN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PN_ABI_VERSION 1

typedef struct pn_search pn_search; /* one GridNeighborhoodSearch{NDIMS} */
typedef void* pn_stream_t;          /* cudaStream_t */

typedef enum {
  PN_OK = 0,
  PN_ERR_OUT_OF_DOMAIN = 1,  /* "particle coordinates are NaN or outside the domain bounds
                                of the cell list" (full_grid.jl:205-212)                   */
  PN_ERR_INVALID_ARG = 2,    /* ArgumentError / bad sizes / eachindex_y out of bounds       */
  PN_ERR_CUDA = 3,           /* a CUDA runtime error                                        */
  PN_ERR_TIMEOUT = 4,        /* a bounded device-side wait gave up                          */
  PN_ERR_UNSUPPORTED_FUNCTOR = 5,
  PN_ERR_CELL_FULL = 6,      /* "cell list is full. Use a larger `max_points_per_cell`."
                                (vector_of_vectors.jl:114-121), only when the limit is set  */
  PN_ERR_NOT_INITIALIZED = 7,/* traversal before initialize, or on an empty template        */
  PN_ERR_OUT_OF_MEMORY = 8,
  PN_ERR_BOUNDS = 9,         /* a query point whose neighbouring cells are outside the grid
                                (the reference's BoundsError in points_in_cell)             */
  PN_ERR_CAPACITY = 10,      /* neighbour-list output buffer too small                      */
  PN_ERR_SCRATCH_LIMIT = 11, /* problem larger than pn_count_neighbors_noalloc's fixed
                                scratch (PN_NOALLOC_SCRATCH_BYTES)                          */
  PN_ERR_INDEX = 12          /* a device index out of range (bounds-checked library only,
                                see pn_bounds_failure)                                      */
} pn_status;

typedef enum { PN_FLOAT32 = 0, PN_FLOAT64 = 1 } pn_dtype;

/* pn_config.flags.  PN_FLAG_FLOAT32_SEARCH: Float64 coordinates (dtype PN_FLOAT64) with a
 * Float32 search radius and PeriodicBox -- the reference's mixed precision
 * (docs/literate/src/tut_gpu_usage.jl:38-50): cells are computed in Float64, but pos_diff is
 * the Float64 difference converted to Float32, and d^2, the periodic correction and the test
 * d^2 <= r^2 are Float32 (neighborhood_search.jl:402-410).  The pair functions' arrays
 * (masses, density, pressure, velocity, accel, energy, ...) are then Float32, the type of
 * pos_diff and distance.  Neighbour sets are the reference's exactly; for x is y the pair
 * functions receive pos_diff within about 2^-22 of the reference's Float32 value away from
 * the radius (the exact value near it).  Not taken by pn_count_neighbors_noalloc or
 * pn_batch_create. */
#define PN_FLAG_FLOAT32_SEARCH 1

/* nhs_grid.jl:135-192 update strategies available for a FullGridCellList. */
typedef enum {
  PN_PARALLEL_UPDATE = 0,             /* full rebuild (the FullGridCellList default)       */
  PN_PARALLEL_INCREMENTAL_UPDATE = 1  /* re-bin only points whose cell changed            */
} pn_update_strategy;

/* Pair functions (the `f` of foreach_point_neighbor), with their parameter structs. */
typedef enum {
  PN_F_COUNT = 0,          /* pn_count_params                                             */
  PN_F_NEIGHBOR_LIST = 1,  /* pn_neighbor_list_params                                     */
  PN_F_NBODY_ACCEL = 2,    /* pn_nbody_params    (benchmarks/n_body.jl:16-55)             */
  PN_F_POTENTIAL = 3,      /* pn_potential_params                                         */
  PN_F_WCSPH_DENSITY = 4,  /* pn_wcsph_params                                             */
  PN_F_WCSPH_FORCE = 5,    /* pn_wcsph_params                                             */
  PN_F_WCSPH_STEP = 6,     /* pn_wcsph_params: density + EOS, then force, one call        */
  PN_F_INDEX_SUM = 7,      /* pn_index_sum_params: mapreduce_neighbor(+) of j (1-based)   */
  PN_F_ADJOINT_FORWARD = 8,  /* pn_adjoint_params: density, loss terms, loss              */
  PN_F_ADJOINT_BACKWARD = 9  /* pn_adjoint_params: dL/dx with the neighbour set fixed     */
} pn_functor;

/* GridNeighborhoodSearch{NDIMS}(; search_radius, n_points, periodic_box,
 *   cell_list = FullGridCellList(; min_corner, max_corner, search_radius,
 *                                  max_points_per_cell), update_strategy)
 * (nhs_grid.jl:77-129, full_grid.jl:48-82, neighborhood_search.jl:129-141). */
typedef struct {
  int32_t ndims;               /* 1, 2 or 3                                                 */
  int32_t dtype;               /* pn_dtype                                                  */
  double search_radius;        /* value in T (exactly representable)                        */
  double min_corner[3];        /* FullGridCellList corners, unpadded, values in T           */
  double max_corner[3];
  int32_t periodic;            /* 1 if a PeriodicBox is given                               */
  int32_t update_strategy;     /* pn_update_strategy                                        */
  double periodic_min[3];      /* PeriodicBox corners, values in T                          */
  double periodic_max[3];
  int64_t n_points;            /* expected number of points in y (pre-sizes scratch)       */
  int32_t max_points_per_cell; /* > 0: error like the reference when a cell exceeds it;
                                  0: no limit (the CSR cell list has no fixed capacity)     */
  int32_t flags;               /* 0 or PN_FLAG_FLOAT32_SEARCH                               */
} pn_config;

/* Geometry as computed by the constructors (for tests and for the Julia binding's
 * `cell_list.min_corner`, `nhs.n_cells`, `nhs.cell_size`). */
typedef struct {
  int32_t ndims, dtype, periodic, is_template;
  int64_t grid_size[3];        /* padded FullGridCellList size per dimension               */
  int64_t n_cells[3];          /* periodic cells per dimension, -1 when not periodic       */
  double min_corner[3];        /* padded corners (min_corner - 1.001 r)                     */
  double max_corner[3];
  double cell_size[3];
  double search_radius;
  int64_t n_binned;            /* points in the cell list after the last initialize/update */
  int64_t n_overflow;          /* points held in the incremental-update overflow lists     */
  int64_t list_size;           /* SpatialHashingCellList lists (0: FullGridCellList)       */
} pn_grid_info;

typedef struct { int32_t* counts; } pn_count_params;       /* out int32[n_queries]         */
typedef struct { int64_t* sums; } pn_index_sum_params;     /* out int64[n_queries]         */

/* Neighbour lists in CSR form: row q holds the neighbour indices j of query q.
 * The call counts, writes offsets (exclusive scan, offsets[n_queries] = total), and if
 * total <= capacity writes the rows (else sets PN_ERR_CAPACITY); sort_rows sorts each row
 * ascending (the reference's test compares sorted lists). */
typedef struct {
  int32_t* counts;      /* out int32[n_queries] (may be NULL)                               */
  int64_t* offsets;     /* out int64[n_queries + 1]                                         */
  int32_t* neighbors;   /* out int32[capacity]                                              */
  int64_t capacity;
  int32_t sort_rows;
  int32_t pad_;
} pn_neighbor_list_params;

/* benchmarks/n_body.jl:41-56: dv_i += -G m_j pos_diff / d^3 for d >= sqrt(eps(T)). */
typedef struct {
  const void* masses;   /* T[n_y]                                                           */
  double G;
  void* accel;          /* out T[n_queries * d]                                             */
} pn_nbody_params;

/* Truncated pair potential e_i = sum_j m_i m_j (1/d - 1/R) for 0 < d < R. */
typedef struct {
  const void* masses;   /* T[n]  (x == y)                                                   */
  double cutoff;        /* R                                                                */
  void* energy;         /* out T[n_queries]                                                 */
} pn_potential_params;

/* Weakly compressible SPH: Wendland C2 kernel (support 2h), Tait equation of state
 * p = c0^2 rho0 / gamma ((rho/rho0)^gamma - 1), momentum equation with Monaghan artificial
 * viscosity (alpha, beta = 0, mu = h v.x / (d^2 + eps_visc h^2)).
 * DENSITY: density[i] = sum_j m W(d_ij) (self included), pressure[i] = EOS(density[i]);
 *          when x is y and velocity is given, it also keeps a cell-sorted copy of
 *          (x, p/rho^2) and (v, rho) in the search for a following FORCE call.
 * FORCE:   accel[i] = -sum_{j, d>r_min} m (p_i/rho_i^2 + p_j/rho_j^2 + Pi_ij) grad W_ij,
 *          reading density, pressure, velocity (x == y required).
 * STEP:    DENSITY then FORCE in one call. */
typedef struct {
  double mass, h, c0, rho0, gamma_exp, alpha, eps_visc;
  double r_min;          /* pairs closer than this are skipped by FORCE (self pair)        */
  void* density;         /* T[n]: out for DENSITY/STEP, in for FORCE                       */
  void* pressure;        /* T[n]: out for DENSITY/STEP, in for FORCE                       */
  const void* velocity;  /* T[n * d]: in for FORCE/STEP                                    */
  void* accel;           /* T[n * d]: out for FORCE/STEP                                   */
  int32_t reuse_state;   /* FORCE: 1 = the previous call on this search was a DENSITY
                            call (x is y, same velocity) whose cell-sorted copy of
                            density, pressure and velocity is still valid; 0 = gather
                            them from the arrays above                                 */
  int32_t pad_;
} pn_wcsph_params;

/* Differentiable form (no counterpart in the reference, which has no adjoint): the loss
 *   L = sum_i (rho_i - 1)^2 + lambda * E,   rho_i = sum_j m W(d_ij) (Wendland C2 as for
 *   WCSPH, self included),   E = 1/2 sum_i sum_{j != i, 0 < d_ij < cutoff} m^2 (1/d_ij - 1/cutoff)
 * over the neighbour pairs of the search (x == y), and its gradient
 *   dL/dx_k = sum_j [(g_k + g_j) m W'(d_kj) + lambda phi'(d_kj)] (x_k - x_j) / d_kj,
 *   g = 2 (rho - 1), phi(d) = m^2 (1/d - 1/cutoff),
 * with the neighbour set held fixed (the search is piecewise constant in x).  Both sweeps
 * re-traverse the cell list; no pair list is stored.
 * FORWARD writes density[i], terms[i] = (rho_i - 1)^2 + lambda/2 * e_i, loss[0] = sum of
 *   the terms in FP64 (fixed summation order), and keeps (x, g) in slot order for BACKWARD.
 * BACKWARD writes grad[i * d + k] = scale * dL/dx_ik, scale = *grad_scale (device
 *   pointer; NULL = 1); reuse_state = 1 uses the state of the preceding FORWARD call on
 *   this search, 0 rebuilds it from `density`. */
typedef struct {
  double mass, h, cutoff, lambda_pot;  /* lambda_pot: the weight lambda of E */
  void* density;            /* T[n]: out (FORWARD), in (BACKWARD without reuse_state)      */
  void* terms;              /* T[n]: out (FORWARD)                                          */
  double* loss;             /* double[1]: out (FORWARD)                                     */
  void* grad;               /* T[n * d]: out (BACKWARD)                                     */
  const double* grad_scale; /* double[1] or NULL (BACKWARD)                                 */
  int32_t reuse_state;
  int32_t pad_;
} pn_adjoint_params;

/* ----------------------------------------------------------------- lifetime */

/* GridNeighborhoodSearch{NDIMS}(...) with a FullGridCellList (nhs_grid.jl:77-129,
 * full_grid.jl:48-82).  ArgumentError cases of the reference return PN_ERR_INVALID_ARG:
 * integer-like radius is not representable here; periodic boxes with < 3 cells. */
int pn_create(const pn_config* cfg, pn_search** out);

/* The same search from a FullGridCellList's own state, for a binding that holds a search
 * the reference's constructors built (full_grid.jl:30-35,66-79): cfg->min_corner and
 * max_corner are the corners the cell list stores (`cell_list.min_corner`, `max_corner`,
 * already padded by 1001//1000 * search_radius), grid_size[k] = size(cell_list.linear_indices,
 * k) for k < ndims (all zero for a template), and cfg->max_points_per_cell =
 * size(cell_list.cells.backend, 1), the DynamicVectorOfVectors capacity
 * (vector_of_vectors.jl:3-31).  The stored values are taken as they are, so the cells equal
 * the reference's bit for bit; subtracting the padding from the stored corners and padding
 * again does not round-trip in floating point.  Everything else as pn_create. */
int pn_create_from_grid(const pn_config* cfg, const int64_t* grid_size, pn_search** out);

/* GridNeighborhoodSearch{NDIMS}(; search_radius, n_points, periodic_box,
 *   cell_list = SpatialHashingCellList{NDIMS}(; list_size, max_points_per_cell))
 * (spatial_hashing.jl:79-89, nhs_grid.jl:77-129): an unbounded domain whose cells
 * floor.(x ./ cell_size) (nhs_grid.jl:636-638; wrapped to 2:n_cells+1 with a periodic box)
 * are hashed into list_size lists (spatial_hash, spatial_hashing.jl:142-156).  cfg's corners
 * are not used; update_strategy must be PN_PARALLEL_UPDATE (update! rebuilds);
 * max_points_per_cell > 0 limits each hash list ("cell list is full").  A cell coordinate
 * must leave its neighbours inside Int32 (the reference's InexactError), and NaN
 * coordinates are rejected: both PN_ERR_OUT_OF_DOMAIN.  The lists hold each cell's points
 * as a separate run, so the traversal visits exactly the points of the 3^d cells -- the
 * result of the reference's collision checks (nhs_grid.jl:479-513). */
int pn_create_spatial_hashing(const pn_config* cfg, int64_t list_size, pn_search** out);

/* copy_neighborhood_search(nhs, search_radius, n_points) (nhs_grid.jl:640-649,
 * full_grid.jl:179-185, spatial_hashing.jl:133-141): same list size, periodic box, strategy
 * and cell capacity; a FullGridCellList's stored corners (unpadded for a template, whose
 * radius is zero) are the new cell list's corners, padded by the new radius, like
 * copy_cell_list passes them to the constructor. */
int pn_copy_search(const pn_search* tmpl, double search_radius, int64_t n_points,
                   pn_search** out);

int pn_destroy(pn_search* s);

/* ----------------------------------------------------------------- cell list */

/* initialize!(nhs, x, y; eachindex_y) -> initialize_grid! (nhs_grid.jl:220-281):
 * bins the points y[:, eachindex_y] (all points when eachindex_y == NULL). */
int pn_initialize(pn_search* s, const void* y, int64_t n_y, const int32_t* eachindex_y,
                  int64_t n_eachindex_y, pn_stream_t stream);

/* update!(nhs, x, y; points_moving, eachindex_y) (nhs_grid.jl:283-292, 408-477):
 * a no-op when points_moving_y == 0; PN_PARALLEL_UPDATE rebuilds, the incremental
 * strategy re-bins only points whose cell changed (it rejects eachindex_y subsets, like
 * nhs_grid.jl:414-417). */
int pn_update(pn_search* s, const void* y, int64_t n_y, const int32_t* eachindex_y,
              int64_t n_eachindex_y, int32_t points_moving_y, pn_stream_t stream);

/* ParallelIncrementalUpdate's policy (no counterpart in the reference, whose incremental
 * update always moves only the changed points): each pn_update counts the points outside
 * the cell they had at the last full build and, on the device, keeps them in overflow
 * lists when they are at most `fraction` of the points, else rebuilds the cell list
 * (empty overflow).  Results are identical either way; the overflow lists make each
 * traversal slower in proportion to their length, a rebuild costs about as much as the
 * mover count.  Default 0.01; 0 rebuilds whenever a point changed cell, a value >= 1
 * never rebuilds. */
int pn_set_rebuild_fraction(pn_search* s, double fraction);

/* Pair cache (no counterpart in the reference; what its PrecomputedNeighborhoodSearch does,
 * inside a GridNeighborhoodSearch): with `enable` > 0 the first WCSPH-density (or
 * adjoint-forward) sweep with x is y after initialize/update also records, for every query
 * and stencil row, where the row's clipped run starts and which of its (at most 128)
 * candidates are neighbours; the sweeps that follow, until the next initialize/update,
 * visit exactly those.  Queries whose rows are not single clipped runs (periodic faces,
 * incremental overflow lists, runs over 128 slots) keep the stencil, so results never depend
 * on the cache.  Memory: 20 bytes x 3^(d-1) per slot.  0 (the default) turns it off. */
int pn_set_pair_cache(pn_search* s, int32_t enable);

/* ----------------------------------------------------------------- traversal */

/* foreach_point_neighbor(f, x, y, nhs; points) (neighborhood_search.jl:183-234,
 * nhs_grid.jl:519-575).  Loops over the query points x[:, points] (all of x when
 * points == NULL) and, for every neighbour j in y with d^2 <= r^2 (periodic images
 * included, the point itself included), applies the functor.  The search must have been
 * initialized/updated with this y.  Outputs are indexed like `points` (query order). */
int pn_foreach_point_neighbor(pn_search* s, int32_t functor, const void* x, int64_t n_x,
                              const void* y, int64_t n_y, const int32_t* points,
                              int64_t n_points, const void* params, pn_stream_t stream);

/* ----------------------------------------------------------------- status / tests */

/* Wait for the stream of the last call and return (and clear) the sticky error. */
int pn_sync(pn_search* s);
/* Return the sticky error without waiting for queued kernels; clear it if `clear`. */
int pn_get_error(pn_search* s, int32_t clear);
const char* pn_status_string(int32_t status);

/* requires_update(nhs) == (false, true) (nhs_grid.jl:133). */
int pn_requires_update(const pn_search* s, int32_t out[2]);

int pn_get_grid_info(const pn_search* s, pn_grid_info* out);

/* The geometry pn_create would compute for `cfg` (FullGridCellList padding and cell
 * counts, periodic n_cells and cell_size), on the host only: no device is touched. */
int pn_compute_geometry(const pn_config* cfg, pn_grid_info* out);
/* The same for pn_create_from_grid's arguments. */
int pn_compute_geometry_from_grid(const pn_config* cfg, const int64_t* grid_size,
                                  pn_grid_info* out);

/* cell_coords(x, nhs) (nhs_grid.jl:622-638, util.jl:19-34) for n points:
 * out int64[n * ndims], the reference's 1-based (periodic) cell coordinates. */
int pn_cell_coords(pn_search* s, const void* x, int64_t n, int64_t* out, pn_stream_t stream);

/* The contents of the cell list (`cell_list[cell]` for every cell, full_grid.jl:165-169):
 * counts int32[prod(grid_size)] per linear cell index, points int32[n_binned] with each
 * cell's points ascending. */
int pn_export_cells(pn_search* s, int32_t* counts, int32_t* points, pn_stream_t stream);

/* ----------------------------------------------------------------- precomputed lists */

/* PrecomputedNeighborhoodSearch{NDIMS}(; search_radius, n_points, periodic_box,
 *   update_strategy, max_neighbors, sort_neighbor_lists) (nhs_precomputed.jl:67-124) with
 * a FullGridCellList grid search (cfg) computing the lists (update_neighborhood_search).
 * max_neighbors > 0 keeps the reference's capacity error (PN_ERR_CELL_FULL when a point has
 * more neighbours); 0 = no limit.  The lists are stored per query as slots of the grid
 * search's cell-sorted arrays, in groups of 32 rows transposed (the reference's
 * transpose_backend layout for GPUs, without a fixed column height). */
typedef struct pn_precomputed pn_precomputed;
int pn_pre_create(const pn_config* cfg, int32_t max_neighbors, pn_precomputed** out);
/* The same with a SpatialHashingCellList grid search (pn_create_spatial_hashing). */
int pn_pre_create_spatial_hashing(const pn_config* cfg, int64_t list_size,
                                  int32_t max_neighbors, pn_precomputed** out);
int pn_pre_destroy(pn_precomputed* s);
/* initialize!(search, x, y) (nhs_precomputed.jl:130-147): the grid search bins y, then the
 * neighbour lists of every point of x are built (one host synchronisation to size them).
 * eachindex_y other than all points is the reference's "does not support inactive points"
 * error (PN_ERR_INVALID_ARG). */
int pn_pre_initialize(pn_precomputed* s, const void* x, int64_t n_x, const void* y,
                      int64_t n_y, const int32_t* eachindex_y, int64_t n_eachindex_y,
                      pn_stream_t stream);
/* update!(search, x, y; points_moving) (nhs_precomputed.jl:149-167). */
int pn_pre_update(pn_precomputed* s, const void* x, int64_t n_x, const void* y, int64_t n_y,
                  const int32_t* eachindex_y, int64_t n_eachindex_y, int32_t points_moving_x,
                  int32_t points_moving_y, pn_stream_t stream);
/* foreach_point_neighbor over the stored lists (nhs_precomputed.jl:206-247): pos_diff and
 * distance recomputed (periodic image when d^2 > r^2), no distance check; any functor of
 * pn_foreach_point_neighbor.  x and y must be the arrays of the last initialize!/update!
 * (requires_update is (true, true)). */
int pn_pre_foreach_point_neighbor(pn_precomputed* s, int32_t functor, const void* x,
                                  int64_t n_x, const void* y, int64_t n_y,
                                  const int32_t* points, int64_t n_points, const void* params,
                                  pn_stream_t stream);
/* The lists as CSR over the points of x: offsets int64[n_x + 1] (always written), neighbour
 * point indices int32[capacity] (written when they fit, else PN_ERR_CAPACITY), each row
 * sorted ascending when `sort` (the reference's sorteach!, sort_neighbor_lists). */
int pn_pre_neighbor_lists(pn_precomputed* s, int32_t sort, int64_t* offsets, int32_t* neighbors,
                          int64_t capacity, pn_stream_t stream);
int pn_pre_sync(pn_precomputed* s);
/* requires_update(::PrecomputedNeighborhoodSearch) == (true, true) (nhs_precomputed.jl:128). */
int pn_pre_requires_update(const pn_precomputed* s, int32_t out[2]);

/* ----------------------------------------------------------------- batched form */

/* Many independent clouds, each its own GridNeighborhoodSearch (own corners, radius and
 * size), built and traversed together: no counterpart in the reference, where each cloud
 * is a separate search (copy_neighborhood_search, nhs_grid.jl:640-649) with its own
 * launches.  Here the clouds' cell lists are concatenated in one set of arrays, one build
 * bins all points, and one persistent traversal kernel takes (cloud, tile of slots) work
 * items from a device queue, so a batch step is a handful of launches whatever the number
 * of clouds; the whole update! + WCSPH step can be captured in a CUDA graph.
 * Scope: 3D, Float32, non-periodic clouds; update! re-bins every point (the rebuild of
 * ParallelUpdate).  Coordinates: one T[3, N] array (N = sum of n_points), clouds
 * concatenated in order; outputs are indexed by the same global point index. */
typedef struct pn_batch pn_batch;

/* Tile schedule of one batched traversal: block size (64, 128 or 256 threads), tile order
 * (0: cloud order, 1: costliest clouds first, by radius^3), persistent (1: one wave of
 * blocks pulling tiles from a device queue; 0: one block per tile), and points per thread
 * (1 or 2; 0 reads as 1): a tile holds block x points_per_thread consecutive query slots,
 * which the block walks in rounds of `block`.  (No staging depth: the traversal reads its
 * candidates through L1 and stages nothing in shared memory.) */
typedef struct { int32_t block, order, persistent, points_per_thread; } pn_batch_schedule;

int pn_batch_create(const pn_config* cfgs, const int64_t* n_points, int32_t n_clouds,
                    pn_batch** out);
int pn_batch_destroy(pn_batch* b);
/* initialize! / update! of every cloud (a full re-bin of all points). */
int pn_batch_initialize(pn_batch* b, const void* y, pn_stream_t stream);
int pn_batch_update(pn_batch* b, const void* y, pn_stream_t stream);
/* foreach_point_neighbor over every cloud (x is y): functor PN_F_COUNT (params: one
 * pn_count_params per cloud) or PN_F_WCSPH_DENSITY / PN_F_WCSPH_FORCE (reuse_state = 1
 * required) / PN_F_WCSPH_STEP (one pn_wcsph_params per cloud: the constants may differ per
 * cloud, the array pointers must be the same global arrays for all clouds). */
int pn_batch_foreach_point_neighbor(pn_batch* b, int32_t functor, const void* y,
                                    const void* params, pn_stream_t stream);
/* Time every schedule (3 blocks x 2 orders x 2 persistence x 2 points per thread) on this
 * batch (reps launches each, CUDA events) and keep the fastest for `functor` (PN_F_COUNT,
 * PN_F_WCSPH_DENSITY or PN_F_WCSPH_FORCE); results do not depend on the schedule. */
int pn_batch_autotune(pn_batch* b, int32_t functor, const void* y, const void* params,
                      int32_t reps, pn_stream_t stream);
/* The same with a schedule cache file: when `cache_path` holds this batch's key
 * (pn_batch_tune_key) the cached schedule is taken untimed, else the batch is autotuned and
 * the winner stored under the key.  The file is text, one line per key:
 * "<key> <block> <order> <persistent> <points_per_thread> <ms>". */
int pn_batch_autotune_cached(pn_batch* b, int32_t functor, const void* y, const void* params,
                             int32_t reps, const char* cache_path, pn_stream_t stream);
/* The cache key of this batch and pair function: element type and dimension, the clouds'
 * median radius (steps of 0.25), log2 of the points and of the clouds.  PN_ERR_CAPACITY when
 * key_size bytes do not hold it. */
int pn_batch_tune_key(const pn_batch* b, int32_t functor, char* key, int32_t key_size);
/* Host-only access to a schedule cache file (no device is touched): look a key up
 * (*found = 1 and *out when present), or store a schedule under it, replacing an older
 * entry (the file is rewritten through a temporary file and a rename). */
int pn_tune_cache_lookup(const char* path, const char* key, pn_batch_schedule* out,
                         int32_t* found);
int pn_tune_cache_store(const char* path, const char* key, const pn_batch_schedule* sched,
                        double ms);
int pn_batch_get_schedule(const pn_batch* b, int32_t functor, pn_batch_schedule* out);
int pn_batch_set_schedule(pn_batch* b, int32_t functor, const pn_batch_schedule* sched);
/* Capture update!(y) + WCSPH density + force of every cloud into a CUDA graph (the
 * library's own stream; no launch happens), replayed by pn_batch_launch_step on any
 * stream.  The graph reads y and writes the arrays of `params` at the captured addresses. */
int pn_batch_capture_step(pn_batch* b, const void* y, const pn_wcsph_params* params);
int pn_batch_launch_step(pn_batch* b, pn_stream_t stream);
/* Wait for the stream of the last call; return (and clear) the sticky error. */
int pn_batch_sync(pn_batch* b);

/* ----------------------------------------------------------------- no-allocation entry */

/* Size of the fixed device scratch that pn_count_neighbors_noalloc works in. */
#define PN_NOALLOC_SCRATCH_BYTES (4 * 1024 * 1024)

/* No counterpart in the reference: an entry point for callers that cannot allocate device
 * memory (a host whose own memory pool owns the device, or a multi-stream time loop that
 * cudaMalloc/cudaFree would synchronise).  It computes what pn_initialize(y = x) followed by
 * pn_foreach_point_neighbor(PN_F_COUNT, x, x) computes -- counts[i] = number of points of x
 * within cfg->search_radius of point i, itself included -- for the geometry `cfg`
 * describes (FullGridCellList corners, optional periodic box, dtype, max_points_per_cell),
 * without a pn_search handle and without allocating: it works in a file-scope device array
 * of PN_NOALLOC_SCRATCH_BYTES that is part of the library image.
 *  - Limit: 4 bytes per cell of the padded grid + 12 bytes per point + 20 bytes must fit
 *    PN_NOALLOC_SCRATCH_BYTES, else PN_ERR_SCRATCH_LIMIT (nothing is launched).
 *  - The first call on a device (the current one) looks up the scratch's address there,
 *    which can load the library's module: make that first call before any stream capture
 *    (and again after a cudaDeviceReset).  Every call looks the address up anew, so a
 *    module loaded elsewhere after a reset is found.
 *  - Every call shares the scratch, which keeps the last call's contents (each call clears
 *    what must start at zero); calls that overlap on the GPU race, so serialise calls made
 *    from several host threads or streams.
 *  - x and counts are device pointers.  The call is synchronous on `stream`: it reads the
 *    kernel's status back and waits for the stream before it returns that status
 *    (PN_ERR_OUT_OF_DOMAIN, PN_ERR_CELL_FULL) as its result, so the host blocks until
 *    the work queued on `stream` before it has finished as well. */
int pn_count_neighbors_noalloc(const pn_config* cfg, const void* x, int64_t n, int32_t* counts,
                               pn_stream_t stream);

int pn_abi_version(void);

/* Number of CUDA kernels the library has launched in this process (all searches). */
unsigned long long pn_launch_count(void);

/* Bounds-checked build (libpn_gb300_bc.so, compiled with -DPN_BOUNDS_CHECK): every device
 * index of the cell-list build and of the traversals is checked before it reaches memory
 * (cell indices, slots, candidate runs, point indices read from the permutation, pair-cache
 * entries); the first index out of range sets PN_ERR_INDEX and the access goes to element 0
 * instead.  pn_build_flags() has bit 0 set in that build.  pn_bounds_failure reports the
 * first failure of a search: site (1 query slot, 2 cell, 3 candidate run, 4 point index,
 * 5 pair-cache entry, 6 slot written by the build, 7 neighbour slot of the pair cache; 0
 * none) and the index, truncated to 32 bits. */
int32_t pn_build_flags(void);
int pn_bounds_failure(pn_search* s, int32_t* site, int32_t* index);

/* Measurement aid (no counterpart in the reference): one launch of a kernel whose every
 * thread runs `iters` rounds of 8 independent Float32 FMA chains (152 x 8 blocks of 256
 * threads), writing one value per thread to out[152 * 8 * 256] so nothing is elided.  It
 * performs 2 * 8 * iters * 311,296 Float32 operations; timing it gives the GPU's Float32
 * issue peak, the roofline of the traversal's arithmetic. */
#define PN_FMA_PROBE_THREADS (152 * 8 * 256)
int pn_fma_probe(float* out, int32_t iters, pn_stream_t stream);

/* Self-test of the device-side wait bound (no counterpart in the reference).  The one
 * device-side wait of the library is the cell-list scan's look-back on its predecessor
 * tiles, bounded by an iteration limit after which it records PN_ERR_TIMEOUT and returns.
 * This runs that scan on a small private array whose first tile never publishes, so the
 * wait must give up (after about a second), and returns the status the scan recorded:
 * PN_ERR_TIMEOUT when the bound works.  Synchronous on `stream`; the context stays usable. */
int pn_selftest_bounded_wait(pn_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
