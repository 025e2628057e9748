// pn_host.h -- the search handle and the host-side launchers shared by the translation
// units of libpn_gb300 (build/update kernels, traversal kernels, C ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "../../include/pn_gb300.h"

// One GridNeighborhoodSearch over a FullGridCellList.
//
// Device layout of the cell list (a CSR counting-sort structure instead of the
// reference's fixed-capacity DynamicVectorOfVectors columns):
//   start[c] .. start[c+1]   slots of cell c (c = 0-based column-major linear index)
//   perm[slot]               point index of the slot (inside a cell: ascending first
//                            coordinate, ties by point index)
//   cell_of_slot[slot]       linear cell index of the slot
//   pos[slot * PS]           the point's coordinates, cell-sorted (3D padded to 4 values)
// Incremental update! keeps this "main" structure from the last full build and holds the
// points that have left their main cell in a second CSR over the same cells (the overflow
// lists): ovf_start[c] .. ovf_start[c+1] are slots after the main ones, in the same
// perm / cell_of_slot / pos arrays (which therefore hold up to 2 * cap slots).  A main slot
// whose point left is vacated: perm = -1 and NaN coordinates, which no distance test
// accepts.
struct pn_search {
  pn_config cfg;
  // geometry (values exact in T, stored as double)
  int32_t ndims, dtype, periodic, is_template;
  int32_t mixed;        // PN_FLAG_FLOAT32_SEARCH: Float64 coordinates, Float32 pair arithmetic
  // pn_create_from_grid: cfg.min_corner / max_corner are the cell list's stored (padded)
  // corners and the grid has given_grid cells per dimension, both taken as they are
  int32_t from_grid = 0;
  int64_t given_grid[3] = {0, 0, 0};
  int32_t hashed;       // SpatialHashingCellList (n_total = list_size hash lists)
  int64_t list_size;
  int64_t grid_size[3], n_cells[3];
  double min_pad[3], max_pad[3], cell_size[3], box_size[3];
  double radius;
  int32_t n_total;      // number of cells, prod(grid_size)
  int32_t scan_tiles;   // tiles of the cell-start scan

  // device scratch owned by the handle
  int32_t* d_err = nullptr;        // sticky error word
  int32_t* d_counts = nullptr;     // [n_total] histogram
  int32_t* d_start = nullptr;      // [n_total + 1]
  unsigned long long* d_scan_state = nullptr;  // [scan_tiles + 1] look-back state + counter
  int64_t cap = 0;                 // point capacity; slot arrays hold 2 * cap slots
  int32_t* d_cell_of = nullptr;    // [cap] cell of the t-th binned input point
  int32_t* d_slot_of = nullptr;    // [cap] its rank inside the cell (atomic order)
  int32_t* d_tmp_perm = nullptr;   // [2 cap] scatter target before the in-cell sort
  int32_t* d_perm = nullptr;       // [2 cap]
  int32_t* d_cell_of_slot = nullptr;  // [2 cap]
  void* d_pos = nullptr;           // [2 cap * 4] T
  void* d_pa = nullptr;            // [2 cap * 4] T  WCSPH neighbour state (x, y, z, p/rho^2)
  void* d_pb = nullptr;            // [2 cap * 4] T  WCSPH neighbour state (vx, vy, vz, rho)
  float* d_pos32 = nullptr;        // [2 cap * 4] pos rounded to Float32 (mixed precision, and
                                   // a Float64 FullGridCellList search's Float32 traversal)
  float* d_pos32lo = nullptr;      // [2 cap * 4] and the rest, pos - pos32, rounded to Float32
  int32_t* d_qcount = nullptr;     // [qcount_cap] per-query counts (neighbour lists)
  int64_t qcount_cap = 0;
  int64_t* d_part = nullptr;       // partial sums of the 64-bit scan
  int64_t part_cap = 0;
  int32_t* d_sort_tmp = nullptr;   // row-sort scratch of the neighbour lists
  int64_t sort_tmp_cap = 0;
  double* d_sum_part = nullptr;    // [SUM_BLOCKS] partial sums of the adjoint loss

  // incremental update (overflow lists relative to the main structure)
  int32_t* d_main_perm = nullptr;      // [cap] perm of the last full build
  int32_t* d_ovf_counts = nullptr;     // [n_total]
  int32_t* d_ovf_start = nullptr;      // [n_total + 1] absolute slots
  int32_t* d_ovf_n = nullptr;          // [1] number of movers
  int32_t* d_ovf_list = nullptr;       // [cap] point index of each mover
  int32_t* d_ovf_cell = nullptr;       // [cap] its new cell
  int32_t* d_ovf_slot = nullptr;       // [cap] rank in the new cell (atomic order)
  int32_t* h_ovf_n = nullptr;          // pinned copy of the mover count
  cudaEvent_t ev_ovf = nullptr;        // recorded after the copy
  bool ovf_pending = false;
  int64_t n_ovf = 0;                   // movers after the last update (host view)
  bool ovf_active = false;             // overflow lists in use
  // Float32 incremental searches: each slot's first coordinate when its cell was last
  // sorted (main slots: the last full build; overflow slots: the last update), the key the
  // rows are clipped by while the positions of the main slots move in place; the largest
  // distance of a main slot's x from its key is err word ERR_DELTA
  float* d_xkey = nullptr;             // [slots]
  float* d_cell_delta = nullptr;       // [n_total] the largest |x - xkey| per cell
  // Float64 searches (not hashed): the third part of the coordinates' Float32 split
  // (x = pos32 + pos32lo + pos32lo2 exactly) and the double-float WCSPH state, for the
  // double-float sums of the 3D WCSPH sweeps
  float* d_pos32lo2 = nullptr;         // [slots][4]
  float* d_sdf = nullptr;              // [slots][12]
  bool main_perm_valid = false;
  double rebuild_fraction = 0.01;      // full rebuild when movers exceed this fraction
  int32_t updates_since_build = 0;

  // pair cache (opt-in, pn_set_pair_cache): per cell-sorted query and stencil row, the start
  // of the clipped run and a 128-bit mask of its neighbours, written by the first density
  // sweep after a build and walked by the sweeps after it
  int32_t pc_cap = 0;                   // > 0: on
  bool pc_valid = false;
  int32_t* d_pc_b0 = nullptr;           // [rows of 3^(d-1)][slots]; row 0 < 0: stencil fallback
  int64_t pc_b0_cap = 0;
  unsigned long long* d_pc_mask = nullptr;  // [rows][slots] x 2 words
  int64_t pc_mask_cap = 0;
  // while overflow lists are in use: per row the start of the clipped overflow run (-1: no
  // neighbour in it) and a 64-bit mask of its neighbours
  int32_t* d_pc_ob0 = nullptr;              // [rows][slots]
  int64_t pc_ob0_cap = 0;
  unsigned long long* d_pc_omask = nullptr;  // [rows][slots]
  int64_t pc_omask_cap = 0;
  bool pc_ovf = false;                      // the last recording wrote the overflow masks
  int64_t pc_rows = 0;

  // SpatialHashingCellList: the slots of a hash list are sorted by cell, then by first
  // coordinate; every distinct cell is an entry (x, y, z, first slot) of hcell, and the
  // entries of list h are hcell[hbucket[h] .. hbucket[h + 1]) (a sentinel entry closes the
  // last run)
  int4* d_hkey_t = nullptr;         // [cap] cell of the t-th binned point (w unused)
  int4* d_hkey_tmp = nullptr;       // [cap] cells in scatter order
  int4* d_hkey = nullptr;           // [cap] cell of each slot
  int32_t* d_hcellidx = nullptr;    // [cap + 1] scan of the cell heads
  int4* d_hcell = nullptr;          // [cap + 1] cell entries
  int32_t* d_hbucket = nullptr;     // [list_size + 1]
  unsigned long long* d_hscan_state = nullptr;
  int64_t hash_cap = 0;
  // When the bounding box of the occupied cells (padded by two cells) has at most list_size
  // cells, the points are stored in a dense grid over that box instead (space order, the
  // full grid's traversal); hash_off maps a cell coordinate to its 1-based grid index.
  bool hash_dense = false;
  int32_t hash_off[3] = {0, 0, 0};
  int32_t* d_hbbox = nullptr;       // [6] min and max cell coordinate per dimension
  int32_t* h_hbbox = nullptr;       // pinned copy

  // state
  bool initialized = false;
  bool full_binned = false;   // every point of y is binned (no eachindex_y subset)
  int64_t n_binned = 0;
  int64_t n_y = 0;            // size of y at the last build
  const void* y_ptr = nullptr;
  cudaStream_t last_stream = nullptr;
  int32_t host_error = 0;     // errors detected on the host before launching
};

namespace pn {

// An NVTX range around each entry point that queues device work, named after the entry
// point, so that a profiler's timeline shows the library's calls (header-only NVTX: without
// a profiler attached a range costs a call through a no-op pointer).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define PN_NVTX_RANGE(name) ::pn::NvtxRange pn_nvtx_range_(name)

// Spare slots at the end of the slot arrays (candidate scans read up to 7 past a run).
constexpr int64_t SLOT_PAD = 64;

// Slots allocated in the slot arrays (main, overflow and the spare slots).
inline int64_t slot_capacity(const pn_search* s) { return 2 * s->cap + SLOT_PAD; }

// Host-side count of kernel launches made by the library (pn_launch_count()).
void count_launch();

int ensure_capacity(pn_search* s, int64_t n);
int ensure_qcount(pn_search* s, int64_t n);
constexpr int SUM_BLOCKS = 256;
int ensure_sum_part(pn_search* s);
int cuda_status(cudaError_t e);

// pn_build.cu
template <typename T>
int build(pn_search* s, const T* y, int64_t n_y, const int32_t* idx, int64_t n_idx,
          cudaStream_t st);
template <typename T>
int build_hash(pn_search* s, const T* y, int64_t n_y, const int32_t* idx, int64_t n_idx,
               cudaStream_t st);
template <typename T>
int update_incremental(pn_search* s, const T* y, int64_t n_y, cudaStream_t st);
template <typename T>
int cell_coords(pn_search* s, const T* x, int64_t n, int64_t* out, cudaStream_t st);
int export_cells(pn_search* s, int32_t* counts, int32_t* points, cudaStream_t st);
// The Float32 copy of the cell-sorted coordinates of a mixed-precision or Float64 search
// (d_pos32, and d_pos32lo for mixed precision).
void refresh_pos32(pn_search* s, cudaStream_t st);
int export_hash_lists(pn_search* s, int32_t* counts, int32_t* points, cudaStream_t st);
int scan64(pn_search* s, const int32_t* in, int64_t n, int64_t* out, cudaStream_t st);
// generic pieces of the build, reused by the batched build (pn_batch.cu)
// stats (or null): receives the largest count and the limit flag (see k_scan_cells)
void scan_counts(const int32_t* counts, int32_t n, int32_t* start, unsigned long long* state,
                 int32_t tiles, int32_t* err, cudaStream_t st, int32_t* stats = nullptr);
int32_t scan_tile_count(int64_t n);
int selftest_bounded_wait(cudaStream_t st);
void scatter_slots(const int32_t* cell_of, const int32_t* slot_of, int32_t m,
                   const int32_t* start, int32_t* tmp_perm, int32_t* cell_of_slot,
                   cudaStream_t st);
template <typename T>
void finalize_slots(int ndims, const int32_t* tmp_perm, const int32_t* cell_of_slot,
                    const int32_t* start, int32_t n_total, const T* y, int32_t m, int32_t* perm,
                    T* pos, cudaStream_t st);
int sort_rows(pn_search* s, const int64_t* offsets, int64_t n_rows, int32_t* vals,
              int64_t total, cudaStream_t st);

// Precomputed neighbour lists handed to a traversal: row r's t-th neighbour slot is
// nb[grp[r / 32] + 32 t + r % 32], len[r] of them; rows are slots (by_slot) or queries.
struct ListsRef {
  const int32_t* nb;
  const int64_t* grp;
  const int32_t* len;
  const int32_t* row_of;  // point -> slot row (by_slot lists)
  int32_t by_slot;
  int64_t n_rows;
};

// pn_traverse_f32.cu / pn_traverse_f64.cu
template <typename T>
int foreach(pn_search* s, int32_t functor, const T* x, int64_t n_x, const T* y, int64_t n_y,
            const int32_t* points, int64_t n_points, const void* params, cudaStream_t st,
            const ListsRef* lists = nullptr);
// The precomputed search's list build over the grid search `s` (x against y): row lengths
// into `len` (slot rows when x is y, else query rows), then the slots into the lists.
template <typename T>
int lists_count(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y, int32_t* len,
                int32_t* by_slot, int64_t* n_rows, cudaStream_t st);
// cap > 0 with len: fixed capacity per row, lengths written by the same pass.
template <typename T>
int lists_emit(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y, int32_t* nb,
               const int64_t* grp, int32_t cap, int32_t* len, cudaStream_t st);

// pn_traverse_mixed.cu: the same three for a search with PN_FLAG_FLOAT32_SEARCH (Float64
// coordinates, Float32 pair functions); foreach<double> and friends forward to them.
int foreach_mixed(pn_search* s, int32_t functor, const double* x, int64_t n_x, const double* y,
                  int64_t n_y, const int32_t* points, int64_t n_points, const void* params,
                  cudaStream_t st, const ListsRef* lists);
int lists_count_mixed(pn_search* s, const double* x, int64_t n_x, const double* y, int64_t n_y,
                      int32_t* len, int32_t* by_slot, int64_t* n_rows, cudaStream_t st);
int lists_emit_mixed(pn_search* s, const double* x, int64_t n_x, const double* y, int64_t n_y,
                     int32_t* nb, const int64_t* grp, int32_t cap, int32_t* len,
                     cudaStream_t st);

}  // namespace pn
