// pn_noalloc.cu -- pn_count_neighbors_noalloc: neighbour counts of one point set without
// any device allocation.
//
// Who needs this.  Every other entry point works on a pn_search handle whose cell arrays
// pn_create / pn_initialize obtain with cudaMalloc.  Some callers cannot allow that:
//  - hosts whose own memory manager owns the device, e.g. a simulation that reserves
//    nearly all HBM for its particle arrays at start-up, or a Julia program whose memory
//    pool has a hard limit: an allocation behind the pool's back fails or evicts its cache;
//  - time-stepping loops that run several systems on several streams: cudaFree (and
//    cudaMalloc, when the driver must grow its heap) synchronises the whole device and so
//    stalls the other streams' work;
//  - code that must not allocate after its set-up phase at all (fixed memory budget).
// For them this entry point counts, for each point of x, the points of x within the search
// radius (the point itself included) -- the result of initialize!(nhs, x, x) followed by
// foreach_point_neighbor with a counting pair function -- using only a fixed scratch array
// that is part of the library's device image.
//
// The scratch.  `pn_noalloc_scratch` below is a file-scope __device__ array of
// PN_NOALLOC_SCRATCH_BYTES (4 MiB).  The CUDA driver reserves it on a device when it loads
// this file's module there; no call here allocates anything (no cudaMalloc, cudaFree or any
// allocating library routine).  A call needs 4 bytes per grid cell of the padded
// FullGridCellList plus 12 bytes per point plus 20 bytes; larger problems are rejected with
// PN_ERR_SCRATCH_LIMIT before any device work.
//
// Set-up.  The first call on a device (the device current on the calling thread) looks up
// the array's device address with cudaGetSymbolAddress, which can load the module; that
// first call should therefore come before any stream capture on that device.  Later calls
// look the address up again, which allocates nothing.
//
// Sharing.  Every call on a device uses the same array and the array keeps the contents of
// the last call; the kernel clears what must start at zero (the error word and the per-cell
// counters) itself.  Calls whose kernels overlap on the GPU race on the array: from several
// host threads or streams, serialise them.
//
// The kernel is one thread block of 1024 threads (the cell-list build needs block-wide
// barriers between its phases and no block waits on another).  It is meant for the point
// sets that fit the scratch (up to about 340,000 points), not as the fast path: the
// pn_search traversal is.

#include "pn_traverse.cuh"

// The shared scratch of pn_count_neighbors_noalloc (zero when the module is loaded).
static __device__ __align__(256) int32_t pn_noalloc_scratch[PN_NOALLOC_SCRATCH_BYTES / 4];

namespace pn {
namespace {

constexpr int NA_THREADS = 1024;
constexpr int64_t NA_HEADER_WORDS = 4;  // word 0: error code; words 1-3 unused

// Exclusive prefix sum of one value per thread over the block; `total` gets the sum.
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* sm, int32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t w = sm[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sm[lane] = w;
  }
  __syncthreads();
  const int32_t base = warp ? sm[warp - 1] : 0;
  total = sm[31];
  __syncthreads();
  return base + x - v;
}

// Scratch layout (int32 words): [header 4][cell start, n_total + 1][cell of point, n]
// [rank of the point in its cell, n][cell-ordered point indices, n].
template <typename T, int D, bool PER>
__global__ void __launch_bounds__(NA_THREADS, 1)
k_count_noalloc(GridDev<T> g, const T* __restrict__ x, int32_t n, int32_t max_ppc,
                int32_t* __restrict__ counts, int32_t* __restrict__ ws) {
  __shared__ int32_t sm[32];
  int32_t* err = ws;
  int32_t* start = ws + NA_HEADER_WORDS;
  const int32_t n_cells1 = g.n_total + 1;
  int32_t* cell_of = start + n_cells1;
  int32_t* rank = cell_of + n;
  int32_t* perm = rank + n;
  const int tid = threadIdx.x;

  // 1. what must start at zero: the error word and the per-cell counters
  if (tid == 0) *err = 0;
  for (int32_t c = tid; c < n_cells1; c += NA_THREADS) start[c] = 0;
  __syncthreads();

  // 2. each point's cell (the reference's cell coordinates, full_grid.jl:205-212 bounds)
  for (int32_t i = tid; i < n; i += NA_THREADS) {
    int32_t lin = 0, stride = 1;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      int32_t ck;
      ok &= cell_coord_1d(g, PER, k, x[(int64_t)i * D + k], ck);
      lin += (ck - 1) * stride;
      stride *= g.n[k];
    }
    if (!ok) {
      set_error(err, PN_ERR_OUT_OF_DOMAIN);
      cell_of[i] = -1;
      continue;
    }
    cell_of[i] = lin;
    rank[i] = atomicAdd(&start[lin], 1);
  }
  __syncthreads();

  // 3. cell counts -> cell starts (exclusive scan, one contiguous run of cells per thread)
  const int32_t seg = (n_cells1 + NA_THREADS - 1) / NA_THREADS;
  const int32_t b = min(tid * seg, n_cells1), e = min(b + seg, n_cells1);
  int32_t local = 0;
  for (int32_t c = b; c < e; ++c) {
    const int32_t v = start[c];
    if (max_ppc > 0 && v > max_ppc) set_error(err, PN_ERR_CELL_FULL);
    local += v;
  }
  int32_t total;
  int32_t run = block_exclusive_scan(local, sm, total);
  for (int32_t c = b; c < e; ++c) {
    const int32_t v = start[c];
    start[c] = run;
    run += v;
  }
  __syncthreads();
  if (*(volatile int32_t*)err != 0) return;  // every thread reads the same word

  // 4. points in cell order
  for (int32_t i = tid; i < n; i += NA_THREADS) perm[start[cell_of[i]] + rank[i]] = i;
  __syncthreads();

  // 5. count each point's neighbours over the 3^D cells around its cell, with the
  //    reference's pair geometry (pos_diff, d2, and the periodic image when d2 > r^2)
  for (int32_t s = tid; s < n; s += NA_THREADS) {
    const int32_t i = perm[s];
    T xi[D];
    int32_t ci[D];
    int32_t lin = cell_of[i];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      xi[k] = x[(int64_t)i * D + k];
      ci[k] = lin % g.n[k] + 1;
      lin /= g.n[k];
    }
    int32_t cnt = 0;
    constexpr int NSTENCIL = D == 1 ? 3 : (D == 2 ? 9 : 27);
    for (int o = 0; o < NSTENCIL; ++o) {
      int32_t cell = 0, stride = 1, oo = o;
#pragma unroll
      for (int k = 0; k < D; ++k) {
        int32_t ck = ci[k] + oo % 3 - 1;
        oo /= 3;
        if (PER) ck = pwrap(ck, g.ncell[k]);
        cell += (ck - 1) * stride;
        stride *= g.n[k];
      }
      const int32_t t1 = start[cell + 1];
      for (int32_t t = start[cell]; t < t1; ++t) {
        const int32_t j = perm[t];
        T yj[D], pd[D];
#pragma unroll
        for (int k = 0; k < D; ++k) yj[k] = x[(int64_t)j * D + k];
        cnt += pair_geom<T, D, PER>(g, xi, yj, pd) <= g.r2 ? 1 : 0;
      }
    }
    counts[i] = cnt;
  }
}

// The scratch array's address on the current device.  It is looked up on every call (after
// the module is loaded the lookup allocates nothing), so that it stays right when the device
// was reset and the module loaded anew elsewhere.
int scratch_on_current_device(int32_t** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, pn_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) {
    cudaGetLastError();
    return PN_ERR_CUDA;
  }
  *out = (int32_t*)p;
  return PN_OK;
}

template <typename T>
GridDev<T> grid_from_info(const pn_grid_info& gi, const pn_config& cfg) {
  GridDev<T> g{};
  int64_t total = 1;
  for (int k = 0; k < 3; ++k) {
    const bool used = k < gi.ndims;
    g.n[k] = used ? (int32_t)gi.grid_size[k] : 1;
    g.ncell[k] = used && gi.periodic ? (int32_t)gi.n_cells[k] : 0;
    g.min_pad[k] = used ? (T)gi.min_corner[k] : (T)0;
    g.cell_size[k] = used ? (T)gi.cell_size[k] : (T)1;
    if (used && gi.periodic) {
      g.box_min[k] = (T)cfg.periodic_min[k];
      g.box_max[k] = (T)cfg.periodic_max[k];
      g.box_size[k] = (T)(g.box_max[k] - g.box_min[k]);
    }
    g.half_box[k] = g.box_size[k] / (T)2;
    total *= g.n[k];
  }
  g.n_total = (int32_t)total;
  g.r = (T)gi.search_radius;
  g.r2 = g.r * g.r;
  return g;
}

template <typename T, int D>
void launch_count_noalloc(const GridDev<T>& g, bool periodic, const T* x, int32_t n,
                          int32_t max_ppc, int32_t* counts, int32_t* ws, cudaStream_t st) {
  if (periodic)
    k_count_noalloc<T, D, true><<<1, NA_THREADS, 0, st>>>(g, x, n, max_ppc, counts, ws);
  else
    k_count_noalloc<T, D, false><<<1, NA_THREADS, 0, st>>>(g, x, n, max_ppc, counts, ws);
  count_launch();
}

template <typename T>
int count_noalloc(const pn_grid_info& gi, const pn_config& cfg, const T* x, int32_t n,
                  int32_t* counts, int32_t* ws, cudaStream_t st) {
  const GridDev<T> g = grid_from_info<T>(gi, cfg);
  const bool per = gi.periodic != 0;
  const int32_t mppc = cfg.max_points_per_cell;
  switch (gi.ndims) {
    case 1: launch_count_noalloc<T, 1>(g, per, x, n, mppc, counts, ws, st); break;
    case 2: launch_count_noalloc<T, 2>(g, per, x, n, mppc, counts, ws, st); break;
    default: launch_count_noalloc<T, 3>(g, per, x, n, mppc, counts, ws, st); break;
  }
  return cudaGetLastError() == cudaSuccess ? PN_OK : PN_ERR_CUDA;
}

}  // namespace
}  // namespace pn

extern "C" int pn_count_neighbors_noalloc(const pn_config* cfg, const void* x, int64_t n,
                                          int32_t* counts, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_count_neighbors_noalloc");
  using namespace pn;
  if (!cfg || n < 0 || (n > 0 && (!x || !counts))) return PN_ERR_INVALID_ARG;
  if (!(cfg->search_radius >= 0.0) || cfg->max_points_per_cell < 0) return PN_ERR_INVALID_ARG;
  if (cfg->flags != 0) return PN_ERR_INVALID_ARG;  // one element type only
  pn_grid_info gi;
  int rc = pn_compute_geometry(cfg, &gi);  // host only: the geometry pn_create computes
  if (rc != PN_OK) return rc;
  if (gi.is_template) return PN_ERR_NOT_INITIALIZED;
  int64_t n_total = 1;
  for (int k = 0; k < gi.ndims; ++k) n_total *= gi.grid_size[k];
  const int64_t words = NA_HEADER_WORDS + (n_total + 1) + 3 * n;
  if (words > (int64_t)(PN_NOALLOC_SCRATCH_BYTES / 4)) return PN_ERR_SCRATCH_LIMIT;
  if (n == 0) return PN_OK;
  int32_t* ws = nullptr;
  rc = scratch_on_current_device(&ws);
  if (rc != PN_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  rc = gi.dtype == PN_FLOAT64
           ? count_noalloc<double>(gi, *cfg, (const double*)x, (int32_t)n, counts, ws, st)
           : count_noalloc<float>(gi, *cfg, (const float*)x, (int32_t)n, counts, ws, st);
  if (rc != PN_OK) return rc;
  // the kernel's status: one word read back into this stack variable (no staging buffer of
  // ours), which also makes the call return after the counts are written
  int32_t status = 0;
  if (cudaMemcpyAsync(&status, ws, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return PN_ERR_CUDA;
  return status;
}
