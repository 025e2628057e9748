// pn_batch.cu -- the batched form: many independent 3D Float32 clouds (each with its own
// FullGridCellList corners, search radius and size) in one set of arrays.
//
// Layout.  Points are the clouds' points concatenated (global index = cloud offset +
// local index); cells are the clouds' padded grids concatenated (global cell = cloud's
// cell offset + the reference's linear cell index in that grid).  One counting sort over
// the global cells gives every cloud its cell-sorted slots, contiguous and in cloud order,
// because each cloud's cells are contiguous and every point is binned.
//
// Traversal.  Work items are tiles: (cloud, a run of `block` consecutive slots of that
// cloud).  A block copies its cloud's grid, traversal arguments and pair-function
// constants into shared memory once per tile and runs the per-query traversal of the
// single-cloud path (traverse_query) on it, so results equal the per-cloud searches'.  In
// persistent mode one wave of blocks pulls tiles from a device counter; tiles can be ordered
// costliest first (radius^3) so the long ones start early.  No block waits on another.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <limits>
#include <map>
#include <new>
#include <vector>

#include "pn_traverse.cuh"

namespace pn {

struct BatchTile {
  int32_t cloud, begin, end, cell_base;
};

constexpr int BATCH_MAX_QUEUES = 8;
constexpr int BATCH_KINDS = 3;  // count, density, force

}  // namespace pn

using namespace pn;

struct pn_batch {
  int32_t n_clouds = 0;
  std::vector<pn_config> cfg;
  std::vector<int32_t> pt_off;    // [n + 1] point offsets
  std::vector<int32_t> cell_off;  // [n + 1] cell offsets
  std::vector<double> radius;     // per cloud (tile cost ~ radius^3)
  std::vector<GridDev<float>> grids;
  int32_t n_points = 0, n_cells = 0, scan_tiles = 0;

  GridDev<float>* d_grids = nullptr;
  int32_t* d_pt_off = nullptr;
  int32_t* d_cell_off = nullptr;
  int32_t* d_err = nullptr;
  int32_t* d_counts = nullptr;
  int32_t* d_start = nullptr;
  unsigned long long* d_scan_state = nullptr;
  int32_t *d_cell_of = nullptr, *d_slot_of = nullptr, *d_tmp_perm = nullptr, *d_perm = nullptr,
          *d_cell_of_slot = nullptr;
  float *d_pos = nullptr, *d_pa = nullptr, *d_pb = nullptr;
  TravArgs<float>* d_args = nullptr;
  int32_t* d_queue = nullptr;  // [BATCH_MAX_QUEUES] tile counters
  std::map<int, BatchTile*> d_tiles;
  std::map<int, int32_t> n_tiles;
  void* d_params[BATCH_KINDS] = {};
  std::vector<unsigned char> h_params[BATCH_KINDS];
  pn_batch_schedule sched[BATCH_KINDS];

  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t last_stream = nullptr;
  bool initialized = false;
  int32_t host_error = 0;
};

namespace pn {
namespace {

// ------------------------------------------------------------------ build
// Cell of every point of every cloud (the cloud found by binary search over the point
// offsets), warp-aggregated histogram over the global cells.
__global__ void __launch_bounds__(256)
k_bin_batch(const GridDev<float>* __restrict__ grids, const int32_t* __restrict__ pt_off,
            int32_t n_clouds, const int32_t* __restrict__ cell_off, const float* __restrict__ y,
            int32_t n, int32_t* __restrict__ cell_of, int32_t* __restrict__ slot_of,
            int32_t* __restrict__ counts, int32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int32_t cell = -1;
    if (i < n) {
      int32_t lo = 0, hi = n_clouds;  // pt_off[lo] <= i < pt_off[hi]
      while (hi - lo > 1) {
        const int32_t mid = (lo + hi) >> 1;
        if (pt_off[mid] <= i) lo = mid;
        else hi = mid;
      }
      const GridDev<float>& g = grids[lo];
      bool ok = true;
      int32_t lin = 0, stride = 1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        int32_t c;
        ok &= cell_coord_1d(g, false, k, y[i * 3 + k], c);
        lin += (c - 1) * stride;
        stride *= g.n[k];
      }
      if (ok) cell = cell_off[lo] + lin;
      else set_error(err, PN_ERR_OUT_OF_DOMAIN);
    }
    const unsigned valid = __ballot_sync(0xffffffffu, cell >= 0);
    if (cell >= 0) {
      const unsigned peers = __match_any_sync(valid, cell);
      const int leader = __ffs(peers) - 1;
      int32_t b = 0;
      if (lane == leader) b = atomicAdd(&counts[cell], __popc(peers));
      b = __shfl_sync(peers, b, leader);
      slot_of[i] = b + __popc(peers & lanemask_lt());
    }
    if (i < n) cell_of[i] = cell;
  }
}

// ------------------------------------------------------------------ traversal
template <typename W>
__device__ __forceinline__ void copy_words(W* dst, const W* src, int n_words) {
  for (int w = threadIdx.x; w < n_words; w += blockDim.x) dst[w] = src[w];
}

template <class F, int BS, bool PERSIST>
__global__ void __launch_bounds__(BS, 1024 / BS)
k_trav_batch(const TravArgs<float>* __restrict__ args,
             const typename F::Params* __restrict__ params, const BatchTile* __restrict__ tiles,
             int32_t n_tiles, int32_t* __restrict__ queue, const float* pos_override) {
  static_assert(sizeof(TravArgs<float>) % 4 == 0 && sizeof(typename F::Params) % 4 == 0, "");
  __shared__ TravArgs<float> sa;
  __shared__ typename F::Params sp;
  __shared__ int32_t s_tile;
  int32_t t = blockIdx.x;
  for (;;) {
    if (PERSIST) {
      if (threadIdx.x == 0) s_tile = atomicAdd(queue, 1);
      __syncthreads();
      t = s_tile;
    }
    if (t >= n_tiles) return;  // uniform over the block
    const BatchTile tile = tiles[t];
    copy_words(reinterpret_cast<int32_t*>(&sa),
               reinterpret_cast<const int32_t*>(&args[tile.cloud]),
               (int)(sizeof(TravArgs<float>) / 4));
    copy_words(reinterpret_cast<int32_t*>(&sp),
               reinterpret_cast<const int32_t*>(&params[tile.cloud]),
               (int)(sizeof(typename F::Params) / 4));
    __syncthreads();
    if (threadIdx.x == 0 && pos_override != nullptr) sa.pos = pos_override;
    __syncthreads();

    // a tile holds points_per_thread rounds of BS consecutive slots (the bound is uniform)
    for (int32_t k0 = tile.begin; k0 < tile.end; k0 += BS) {
    const int32_t k = k0 + (int32_t)threadIdx.x;
    Query<float, 3> q;
    bool valid = k < tile.end;
    q.i = valid ? sa.perm[k] : -1;
    valid = valid && q.i >= 0;
    q.q = q.i;
    q.k = k;
    int32_t c[3] = {1, 1, 1};
    if (valid) {
      load_pos<float, 3>(sa.pos, k, q.x);
      const int32_t lin = sa.cell_of_slot[k] - tile.cell_base;
      c[0] = lin % sa.g.n[0] + 1;
      c[1] = (lin / sa.g.n[0]) % sa.g.n[1] + 1;
      c[2] = lin / (sa.g.n[0] * sa.g.n[1]) + 1;
    } else {
      q.x[0] = q.x[1] = q.x[2] = 0.0f;
    }
    traverse_query<float, 3, false, F>(sa, sp, q, c, valid);
    }
    if (!PERSIST) return;
    __syncthreads();  // the shared copies are re-used by the next tile
  }
}

// ------------------------------------------------------------------ host helpers
int kind_of(int32_t functor) {
  switch (functor) {
    case PN_F_COUNT: return 0;
    case PN_F_WCSPH_DENSITY: return 1;
    case PN_F_WCSPH_FORCE: return 2;
    default: return -1;
  }
}

// points_per_thread 0 reads as 1 (the field was padding before it was a dimension)
int ppt_of(const pn_batch_schedule& s) { return s.points_per_thread == 2 ? 2 : 1; }

bool valid_schedule(const pn_batch_schedule& s) {
  return (s.block == 64 || s.block == 128 || s.block == 256) && (s.order == 0 || s.order == 1) &&
         (s.persistent == 0 || s.persistent == 1) &&
         (s.points_per_thread >= 0 && s.points_per_thread <= 2);
}

int tile_key(const pn_batch_schedule& s) { return (s.block * 2 + s.order) * 4 + ppt_of(s); }

// Tiles of block x points_per_thread slots per cloud, in cloud order or costliest first
// (radius^3, stable).
int ensure_tiles(pn_batch* b, const pn_batch_schedule& s) {
  const int key = tile_key(s);
  if (b->d_tiles.count(key)) return PN_OK;
  std::vector<int32_t> order(b->n_clouds);
  for (int32_t c = 0; c < b->n_clouds; ++c) order[c] = c;
  if (s.order == 1)
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t c) {
      return b->radius[a] > b->radius[c];
    });
  std::vector<BatchTile> tiles;
  for (int32_t c : order)
    for (int32_t k = b->pt_off[c]; k < b->pt_off[c + 1]; k += s.block * ppt_of(s))
      tiles.push_back({c, k, std::min(k + s.block * ppt_of(s), b->pt_off[c + 1]),
                       b->cell_off[c]});
  BatchTile* d = nullptr;
  if (!tiles.empty()) {
    if (cudaMalloc(&d, sizeof(BatchTile) * tiles.size()) != cudaSuccess) {
      cudaGetLastError();
      return PN_ERR_OUT_OF_MEMORY;
    }
    if (cudaMemcpy(d, tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice) !=
        cudaSuccess) {
      cudaFree(d);
      return PN_ERR_CUDA;
    }
  }
  b->d_tiles[key] = d;
  b->n_tiles[key] = (int32_t)tiles.size();
  return PN_OK;
}

// Upload the per-cloud pair-function parameters when they changed (synchronous copy; a
// graph capture prepares them before it starts).
template <class P>
int upload_params(pn_batch* b, int kind, const std::vector<P>& h) {
  const size_t bytes = sizeof(P) * h.size();
  std::vector<unsigned char>& cache = b->h_params[kind];
  if (cache.size() == bytes && std::memcmp(cache.data(), h.data(), bytes) == 0) return PN_OK;
  if (b->d_params[kind] == nullptr || cache.size() != bytes) {
    if (b->d_params[kind]) cudaFree(b->d_params[kind]);
    b->d_params[kind] = nullptr;
    if (cudaMalloc(&b->d_params[kind], bytes) != cudaSuccess) {
      cudaGetLastError();
      cache.clear();
      return PN_ERR_OUT_OF_MEMORY;
    }
  }
  if (cudaMemcpy(b->d_params[kind], h.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    return PN_ERR_CUDA;
  cache.assign(reinterpret_cast<const unsigned char*>(h.data()),
               reinterpret_cast<const unsigned char*>(h.data()) + bytes);
  return PN_OK;
}

SphConst<float> batch_sph_const(const pn_wcsph_params& w) {
  SphConst<float> c{};
  const double h = w.h;
  const double sigma = 21.0 / (16.0 * 3.14159265358979323846 * h * h * h);
  c.mass = (float)w.mass;
  c.h = (float)h;
  c.inv_h = (float)(1.0 / h);
  c.sigma = (float)sigma;
  c.dw_coef = (float)(-5.0 * sigma / (h * h));
  c.c0 = (float)w.c0;
  c.rho0 = (float)w.rho0;
  c.inv_rho0 = (float)(1.0 / w.rho0);
  c.gamma = (float)w.gamma_exp;
  c.gamma_int = (w.gamma_exp == std::floor(w.gamma_exp) && w.gamma_exp >= 1.0 &&
                 w.gamma_exp <= 64.0) ? (int32_t)w.gamma_exp : 0;
  c.eos_b = (float)(w.c0 * w.c0 * w.rho0 / w.gamma_exp);
  c.alpha = (float)w.alpha;
  c.eps_h2 = (float)(w.eps_visc * h * h);
  c.r_min2 = (float)(w.r_min * w.r_min);
  return c;
}

// Per-cloud parameters of `kind` from the caller's arrays of structs.
int prepare_params(pn_batch* b, int kind, const void* params) {
  const int32_t n = b->n_clouds;
  if (kind == 0) {
    const auto* u = static_cast<const pn_count_params*>(params);
    std::vector<CountParams<float>> h(n);
    for (int32_t c = 0; c < n; ++c) {
      if (u[c].counts != u[0].counts || u[c].counts == nullptr) return PN_ERR_INVALID_ARG;
      h[c] = CountParams<float>{u[c].counts, 0};
    }
    return upload_params(b, 0, h);
  }
  const auto* u = static_cast<const pn_wcsph_params*>(params);
  for (int32_t c = 0; c < n; ++c)
    if (u[c].density != u[0].density || u[c].pressure != u[0].pressure ||
        u[c].velocity != u[0].velocity || u[c].accel != u[0].accel || !(u[c].h > 0.0))
      return PN_ERR_INVALID_ARG;
  if (kind == 1) {
    if (!u[0].density || !u[0].pressure || !u[0].velocity) return PN_ERR_INVALID_ARG;
    std::vector<DensityParams<float>> h(n);
    for (int32_t c = 0; c < n; ++c)
      h[c] = DensityParams<float>{batch_sph_const(u[c]), static_cast<float*>(u[c].density),
                                  static_cast<float*>(u[c].pressure),
                                  static_cast<const float*>(u[c].velocity), b->d_pa, b->d_pb};
    return upload_params(b, 1, h);
  }
  if (!u[0].accel || !u[0].reuse_state) return PN_ERR_INVALID_ARG;
  std::vector<ForceParams<float>> h(n);
  for (int32_t c = 0; c < n; ++c)
    h[c] = ForceParams<float>{batch_sph_const(u[c]), b->d_pa, b->d_pb,
                              static_cast<float*>(u[c].accel)};
  return upload_params(b, 2, h);
}

template <class F, int BS>
void launch_bs(pn_batch* b, int kind, const pn_batch_schedule& s, int queue_slot,
               const float* pos_override, cudaStream_t st) {
  const int key = tile_key(s);
  const int32_t nt = b->n_tiles[key];
  if (nt == 0) return;
  const auto* params = static_cast<const typename F::Params*>(b->d_params[kind]);
  int32_t* queue = b->d_queue + queue_slot;
  if (s.persistent) {
    cudaMemsetAsync(queue, 0, sizeof(int32_t), st);
    const int blocks = std::min(nt, 152 * (1024 / BS));
    k_trav_batch<F, BS, true><<<blocks, BS, 0, st>>>(b->d_args, params, b->d_tiles[key], nt,
                                                      queue, pos_override);
  } else {
    k_trav_batch<F, BS, false><<<nt, BS, 0, st>>>(b->d_args, params, b->d_tiles[key], nt,
                                                   queue, pos_override);
  }
  count_launch();
}

template <class F>
int launch_traversal(pn_batch* b, int kind, const pn_batch_schedule& s, int queue_slot,
                     const float* pos_override, cudaStream_t st) {
  int rc = ensure_tiles(b, s);
  if (rc != PN_OK) return rc;
  if (b->d_params[kind] == nullptr) return PN_ERR_INVALID_ARG;
  switch (s.block) {
    case 64: launch_bs<F, 64>(b, kind, s, queue_slot, pos_override, st); break;
    case 256: launch_bs<F, 256>(b, kind, s, queue_slot, pos_override, st); break;
    default: launch_bs<F, 128>(b, kind, s, queue_slot, pos_override, st); break;
  }
  return cuda_status(cudaGetLastError());
}

// kind 0: neighbour count, 1: WCSPH density (+ EOS, sorted state), 2: WCSPH force (its
// candidates are read from the sorted state (x, p/rho^2))
int launch_kind(pn_batch* b, int kind, const pn_batch_schedule& s, int queue_slot,
                cudaStream_t st) {
  switch (kind) {
    case 0: return launch_traversal<FCount<float, 3>>(b, 0, s, queue_slot, nullptr, st);
    case 1: return launch_traversal<FDensity<float, 3>>(b, 1, s, queue_slot, nullptr, st);
    default: return launch_traversal<FForce<float, 3>>(b, 2, s, queue_slot, b->d_pa, st);
  }
}

int rebin(pn_batch* b, const float* y, cudaStream_t st) {
  if (!y) return PN_ERR_INVALID_ARG;
  cudaMemsetAsync(b->d_counts, 0, sizeof(int32_t) * b->n_cells, st);
  const int blocks = std::max(1, std::min((b->n_points + 255) / 256, 152 * 8));
  k_bin_batch<<<blocks, 256, 0, st>>>(b->d_grids, b->d_pt_off, b->n_clouds, b->d_cell_off, y,
                                      b->n_points, b->d_cell_of, b->d_slot_of, b->d_counts,
                                      b->d_err); count_launch();
  scan_counts(b->d_counts, b->n_cells, b->d_start, b->d_scan_state, b->scan_tiles, b->d_err, st);
  scatter_slots(b->d_cell_of, b->d_slot_of, b->n_points, b->d_start, b->d_tmp_perm,
                b->d_cell_of_slot, st);
  finalize_slots<float>(3, b->d_tmp_perm, b->d_cell_of_slot, b->d_start, b->n_cells, y,
                        b->n_points, b->d_perm, b->d_pos, st);
  return cuda_status(cudaGetLastError());
}

// One WCSPH step's traversals: density (with EOS and the sorted state), then force.
int wcsph_step(pn_batch* b, cudaStream_t st) {
  int rc = launch_kind(b, 1, b->sched[1], 0, st);
  if (rc != PN_OK) return rc;
  return launch_kind(b, 2, b->sched[2], 1, st);
}

void destroy(pn_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  void* ptrs[] = {b->d_grids, b->d_pt_off, b->d_cell_off, b->d_err, b->d_counts, b->d_start,
                  b->d_scan_state, b->d_cell_of, b->d_slot_of, b->d_tmp_perm, b->d_perm,
                  b->d_cell_of_slot, b->d_pos, b->d_pa, b->d_pb, b->d_args, b->d_queue,
                  b->d_params[0], b->d_params[1], b->d_params[2]};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& kv : b->d_tiles)
    if (kv.second) cudaFree(kv.second);
  delete b;
}

int record(pn_batch* b, int rc, cudaStream_t st) {
  b->last_stream = st;
  if (rc != PN_OK && b->host_error == 0) b->host_error = rc;
  return rc;
}

}  // namespace

// ------------------------------------------------------------------ schedule cache
// The autotuner's winners persist in a text file, one line per key:
//   <key> <block> <order> <persistent> <points_per_thread> <ms>
// The key names what decides the best schedule -- the pair function, element type and
// dimension, the clouds' radius (median, in steps of 0.25) and the sizes (log2 of the points
// and of the clouds) -- so a later batch of the same kind reuses the schedule untimed.
// Unreadable lines are skipped; a store rewrites the file through a temporary and a rename.
struct CacheEntry {
  std::string key;
  pn_batch_schedule s;
  double ms;
};

bool valid_key(const std::string& k) {
  if (k.empty() || k.size() > 200) return false;
  for (char c : k)
    if (c <= ' ' || c > '~') return false;
  return true;
}

std::vector<CacheEntry> read_cache(const char* path) {
  std::vector<CacheEntry> out;
  FILE* f = std::fopen(path, "r");
  if (!f) return out;
  char line[512];
  while (std::fgets(line, sizeof line, f)) {
    char key[256];
    pn_batch_schedule s{};
    double ms = 0.0;
    if (std::sscanf(line, "%255s %d %d %d %d %lf", key, &s.block, &s.order, &s.persistent,
                    &s.points_per_thread, &ms) == 6 &&
        valid_schedule(s) && valid_key(key))
      out.push_back(CacheEntry{key, s, ms});
  }
  std::fclose(f);
  return out;
}

bool write_cache(const char* path, const std::vector<CacheEntry>& es) {
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return false;
  bool ok = true;
  for (const auto& e : es)
    ok = ok && std::fprintf(f, "%s %d %d %d %d %.6f\n", e.key.c_str(), e.s.block, e.s.order,
                            e.s.persistent, ppt_of(e.s), e.ms) > 0;
  ok = (std::fclose(f) == 0) && ok;
  if (ok) ok = std::rename(tmp.c_str(), path) == 0;
  if (!ok) std::remove(tmp.c_str());
  return ok;
}

std::string tune_key(const pn_batch* b, int32_t functor) {
  std::vector<double> r(b->radius.begin(), b->radius.end());
  std::sort(r.begin(), r.end());
  const double med = r.empty() ? 0.0 : r[r.size() / 2];
  const int64_t n_pts = b->pt_off[b->n_clouds];
  const char* f = functor == PN_F_COUNT ? "count" : functor == PN_F_WCSPH_DENSITY ? "density"
                                                                                   : "force";
  char buf[160];
  std::snprintf(buf, sizeof buf, "batch/%s/f32/d3/r%.2f/n2^%d/c2^%d", f,
                std::round(med * 4.0) / 4.0,
                (int)std::lround(std::log2((double)std::max<int64_t>(n_pts, 1))),
                (int)std::lround(std::log2((double)std::max(b->n_clouds, 1))));
  return buf;
}

int autotune(pn_batch* b, int32_t functor, const void* y, const void* params, int32_t reps,
             cudaStream_t st, float* best_ms);

}  // namespace pn

extern "C" {

int pn_batch_create(const pn_config* cfgs, const int64_t* n_points, int32_t n_clouds,
                    pn_batch** out) {
  PN_NVTX_RANGE("pn_batch_create");
  if (!cfgs || !n_points || !out || n_clouds <= 0) return PN_ERR_INVALID_ARG;
  *out = nullptr;
  pn_batch* b = new (std::nothrow) pn_batch();
  if (!b) return PN_ERR_OUT_OF_MEMORY;
  b->n_clouds = n_clouds;
  b->cfg.assign(cfgs, cfgs + n_clouds);
  b->pt_off.assign(1, 0);
  b->cell_off.assign(1, 0);
  int64_t np = 0, nc = 0;
  for (int32_t c = 0; c < n_clouds; ++c) {
    const pn_config& cf = cfgs[c];
    if (cf.ndims != 3 || cf.dtype != PN_FLOAT32 || cf.flags != 0 || cf.periodic ||
        n_points[c] < 0 || !(cf.search_radius > 0.0)) {
      delete b;
      return PN_ERR_INVALID_ARG;
    }
    pn_grid_info gi;
    int rc = pn_compute_geometry(&cf, &gi);
    if (rc != PN_OK || gi.is_template) {
      delete b;
      return rc != PN_OK ? rc : PN_ERR_INVALID_ARG;
    }
    GridDev<float> g{};
    int64_t tot = 1;
    for (int k = 0; k < 3; ++k) {
      g.n[k] = (int32_t)gi.grid_size[k];
      g.min_pad[k] = (float)gi.min_corner[k];
      g.cell_size[k] = (float)gi.cell_size[k];
      tot *= gi.grid_size[k];
    }
    g.n_total = (int32_t)tot;
    g.r = (float)gi.search_radius;
    g.r2 = g.r * g.r;
    b->grids.push_back(g);
    b->radius.push_back(gi.search_radius);
    np += n_points[c];
    nc += tot;
    if (np > INT32_MAX - 2 * SLOT_PAD || nc > INT32_MAX - 1) {
      delete b;
      return PN_ERR_INVALID_ARG;
    }
    b->pt_off.push_back((int32_t)np);
    b->cell_off.push_back((int32_t)nc);
  }
  b->n_points = (int32_t)np;
  b->n_cells = (int32_t)nc;
  b->scan_tiles = scan_tile_count(nc);
  for (int k = 0; k < BATCH_KINDS; ++k) b->sched[k] = pn_batch_schedule{128, 1, 1, 0};

  const int64_t slots = np + SLOT_PAD;
  bool ok = cudaMalloc(&b->d_grids, sizeof(GridDev<float>) * n_clouds) == cudaSuccess &&
            cudaMalloc(&b->d_pt_off, sizeof(int32_t) * (n_clouds + 1)) == cudaSuccess &&
            cudaMalloc(&b->d_cell_off, sizeof(int32_t) * (n_clouds + 1)) == cudaSuccess &&
            cudaMalloc(&b->d_err, sizeof(int32_t) * ERR_WORDS) == cudaSuccess &&
            cudaMalloc(&b->d_counts, sizeof(int32_t) * (nc + 8)) == cudaSuccess &&
            cudaMalloc(&b->d_start, sizeof(int32_t) * (nc + 1)) == cudaSuccess &&
            cudaMalloc(&b->d_scan_state, sizeof(unsigned long long) * (b->scan_tiles + 1)) ==
                cudaSuccess &&
            cudaMalloc(&b->d_cell_of, sizeof(int32_t) * (np + 1)) == cudaSuccess &&
            cudaMalloc(&b->d_slot_of, sizeof(int32_t) * (np + 1)) == cudaSuccess &&
            cudaMalloc(&b->d_tmp_perm, sizeof(int32_t) * slots) == cudaSuccess &&
            cudaMalloc(&b->d_perm, sizeof(int32_t) * slots) == cudaSuccess &&
            cudaMalloc(&b->d_cell_of_slot, sizeof(int32_t) * slots) == cudaSuccess &&
            cudaMalloc(&b->d_pos, sizeof(float) * 4 * slots) == cudaSuccess &&
            cudaMalloc(&b->d_pa, sizeof(float) * 4 * slots) == cudaSuccess &&
            cudaMalloc(&b->d_pb, sizeof(float) * 4 * slots) == cudaSuccess &&
            cudaMalloc(&b->d_args, sizeof(TravArgs<float>) * n_clouds) == cudaSuccess &&
            cudaMalloc(&b->d_queue, sizeof(int32_t) * BATCH_MAX_QUEUES) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) == cudaSuccess;
  if (ok) {
    // spare slots: never a neighbour (NaN coordinates), never a query (perm -1)
    ok = cudaMemset(b->d_err, 0, sizeof(int32_t) * ERR_WORDS) == cudaSuccess &&
         cudaMemset(b->d_perm + np, 0xff, sizeof(int32_t) * SLOT_PAD) == cudaSuccess &&
         cudaMemset(b->d_pos, 0xff, sizeof(float) * 4 * slots) == cudaSuccess &&
         cudaMemset(b->d_pa, 0xff, sizeof(float) * 4 * slots) == cudaSuccess;
    std::vector<TravArgs<float>> args(n_clouds);
    const double u = std::numeric_limits<float>::epsilon() / 2;
    for (int32_t c = 0; c < n_clouds; ++c) {
      TravArgs<float>& a = args[c];
      a = TravArgs<float>{};
      a.g = b->grids[c];
      a.start = b->d_start + b->cell_off[c];
      a.ovf_start = nullptr;
      a.perm = b->d_perm;
      a.cell_of_slot = b->d_cell_of_slot;
      a.pos = b->d_pos;
      a.err = b->d_err;
      a.bc_slots = slots;
      a.bc_points = np;
      a.outside = b->d_err + 1;
      a.unsorted = nullptr;  // the batch always re-bins: every cell sorted by x
      for (int k = 0; k < 3; ++k) {
        const double mn = a.g.min_pad[k], mx = mn + a.g.n[k] * (double)a.g.cell_size[k];
        a.clip_m[k] = (float)(16.0 * (double)std::numeric_limits<float>::epsilon() *
                              (std::fabs(mn) + std::fabs(mx) + a.g.cell_size[k]));
      }
      const double r2 = (double)a.g.r2;
      a.r2_lo = (float)(r2 * (1.0 - 32.0 * u));
      a.r2_hi = (float)(r2 * (1.0 + 32.0 * u));
    }
    ok = ok &&
         cudaMemcpy(b->d_grids, b->grids.data(), sizeof(GridDev<float>) * n_clouds,
                    cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_pt_off, b->pt_off.data(), sizeof(int32_t) * (n_clouds + 1),
                    cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_cell_off, b->cell_off.data(), sizeof(int32_t) * (n_clouds + 1),
                    cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_args, args.data(), sizeof(TravArgs<float>) * n_clouds,
                    cudaMemcpyHostToDevice) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    destroy(b);
    return PN_ERR_OUT_OF_MEMORY;
  }
  *out = b;
  return PN_OK;
}

int pn_batch_destroy(pn_batch* b) {
  if (b) destroy(b);
  return PN_OK;
}

int pn_batch_initialize(pn_batch* b, const void* y, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_batch_initialize");
  if (!b) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int rc = rebin(b, static_cast<const float*>(y), st);
  if (rc == PN_OK) b->initialized = true;
  return record(b, rc, st);
}

int pn_batch_update(pn_batch* b, const void* y, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_batch_update");
  if (!b) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (!b->initialized) return record(b, PN_ERR_NOT_INITIALIZED, st);
  return record(b, rebin(b, static_cast<const float*>(y), st), st);
}

int pn_batch_foreach_point_neighbor(pn_batch* b, int32_t functor, const void* y,
                                    const void* params, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_batch_foreach_point_neighbor");
  if (!b) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (!b->initialized) return record(b, PN_ERR_NOT_INITIALIZED, st);
  if (!params || !y) return record(b, PN_ERR_INVALID_ARG, st);
  int rc;
  if (functor == PN_F_WCSPH_STEP) {
    rc = prepare_params(b, 1, params);
    if (rc == PN_OK) {
      std::vector<pn_wcsph_params> w(static_cast<const pn_wcsph_params*>(params),
                                     static_cast<const pn_wcsph_params*>(params) + b->n_clouds);
      for (auto& e : w) e.reuse_state = 1;
      rc = prepare_params(b, 2, w.data());
    }
    if (rc == PN_OK) rc = wcsph_step(b, st);
    return record(b, rc, st);
  }
  const int kind = kind_of(functor);
  if (kind < 0) return record(b, PN_ERR_UNSUPPORTED_FUNCTOR, st);
  rc = prepare_params(b, kind, params);
  if (rc == PN_OK) rc = launch_kind(b, kind, b->sched[kind], kind, st);
  return record(b, rc, st);
}

int pn_batch_autotune(pn_batch* b, int32_t functor, const void* y, const void* params,
                      int32_t reps, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_batch_autotune");
  float best = 0.f;
  return autotune(b, functor, y, params, reps, (cudaStream_t)stream, &best);
}

int pn_batch_tune_key(const pn_batch* b, int32_t functor, char* key, int32_t key_size) {
  if (!b || !key || key_size <= 0 || kind_of(functor) < 0) return PN_ERR_INVALID_ARG;
  const std::string k = tune_key(b, functor);
  if ((int64_t)k.size() + 1 > key_size) return PN_ERR_CAPACITY;
  std::memcpy(key, k.c_str(), k.size() + 1);
  return PN_OK;
}

int pn_tune_cache_lookup(const char* path, const char* key, pn_batch_schedule* out,
                         int32_t* found) {
  if (!path || !key || !out || !found) return PN_ERR_INVALID_ARG;
  *found = 0;
  double ms = 0.0;
  for (const auto& e : read_cache(path))
    if (e.key == key) {
      *out = e.s;
      ms = e.ms;
      *found = 1;
    }
  (void)ms;
  return PN_OK;
}

int pn_tune_cache_store(const char* path, const char* key, const pn_batch_schedule* sched,
                        double ms) {
  if (!path || !key || !sched || !valid_schedule(*sched) || !valid_key(key))
    return PN_ERR_INVALID_ARG;
  std::vector<CacheEntry> es = read_cache(path);
  bool replaced = false;
  for (auto& e : es)
    if (e.key == key) {
      e.s = *sched;
      e.ms = ms;
      replaced = true;
    }
  if (!replaced) es.push_back(CacheEntry{key, *sched, ms});
  return write_cache(path, es) ? PN_OK : PN_ERR_INVALID_ARG;
}

int pn_batch_autotune_cached(pn_batch* b, int32_t functor, const void* y, const void* params,
                             int32_t reps, const char* cache_path, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_batch_autotune_cached");
  if (!b || !cache_path) return PN_ERR_INVALID_ARG;
  const int kind = kind_of(functor);
  if (kind < 0) return PN_ERR_UNSUPPORTED_FUNCTOR;
  const std::string key = tune_key(b, functor);
  pn_batch_schedule s{};
  int32_t found = 0;
  if (pn_tune_cache_lookup(cache_path, key.c_str(), &s, &found) == PN_OK && found &&
      valid_schedule(s)) {
    b->sched[kind] = s;
    return PN_OK;
  }
  float best = 0.f;
  const int rc = autotune(b, functor, y, params, reps, (cudaStream_t)stream, &best);
  if (rc != PN_OK) return rc;
  return pn_tune_cache_store(cache_path, key.c_str(), &b->sched[kind], (double)best);
}

}  // extern "C"

namespace pn {

int autotune(pn_batch* b, int32_t functor, const void* y, const void* params, int32_t reps,
             cudaStream_t st, float* best_ms) {
  if (!b || !params || !y || reps <= 0) return PN_ERR_INVALID_ARG;
  const int kind = kind_of(functor);
  if (kind < 0) return record(b, PN_ERR_UNSUPPORTED_FUNCTOR, st);
  if (!b->initialized) return record(b, PN_ERR_NOT_INITIALIZED, st);
  int rc = prepare_params(b, kind, params);
  if (rc != PN_OK) return record(b, rc, st);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return record(b, PN_ERR_CUDA, st);
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return record(b, PN_ERR_CUDA, st);
  }
  float best = std::numeric_limits<float>::infinity();
  pn_batch_schedule best_s = b->sched[kind];
  static const int kBlocks[3] = {64, 128, 256};
  for (int v = 0; v < 24 && rc == PN_OK; ++v) {
    const pn_batch_schedule s{kBlocks[v / 8], (v / 4) % 2, (v / 2) % 2, 1 + v % 2};
    rc = launch_kind(b, kind, s, kind, st);  // warm-up (and the tiles of this schedule)
    std::vector<float> t;
    for (int r = 0; r < reps && rc == PN_OK; ++r) {
      cudaEventRecord(e0, st);
      rc = launch_kind(b, kind, s, kind, st);
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = PN_ERR_CUDA;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      t.push_back(ms);
    }
    if (rc != PN_OK) break;
    std::sort(t.begin(), t.end());
    const float med = t[t.size() / 2];
    if (med < best) {
      best = med;
      best_s = s;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == PN_OK) {
    b->sched[kind] = best_s;
    *best_ms = best;
  }
  return record(b, rc, st);
}

}  // namespace pn

extern "C" {

int pn_batch_get_schedule(const pn_batch* b, int32_t functor, pn_batch_schedule* out) {
  const int kind = kind_of(functor);
  if (!b || !out || kind < 0) return PN_ERR_INVALID_ARG;
  *out = b->sched[kind];
  return PN_OK;
}

int pn_batch_set_schedule(pn_batch* b, int32_t functor, const pn_batch_schedule* sched) {
  const int kind = kind_of(functor);
  if (!b || !sched || kind < 0 || !valid_schedule(*sched)) return PN_ERR_INVALID_ARG;
  b->sched[kind] = *sched;
  return PN_OK;
}

int pn_batch_capture_step(pn_batch* b, const void* y, const pn_wcsph_params* params) {
  PN_NVTX_RANGE("pn_batch_capture_step");
  if (!b || !y || !params) return PN_ERR_INVALID_ARG;
  if (!b->initialized) return PN_ERR_NOT_INITIALIZED;
  int rc = prepare_params(b, 1, params);
  std::vector<pn_wcsph_params> w(params, params + b->n_clouds);
  for (auto& e : w) e.reuse_state = 1;
  if (rc == PN_OK) rc = prepare_params(b, 2, w.data());
  if (rc == PN_OK) rc = ensure_tiles(b, b->sched[1]);
  if (rc == PN_OK) rc = ensure_tiles(b, b->sched[2]);
  if (rc != PN_OK) return rc;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return PN_ERR_CUDA;
  rc = rebin(b, static_cast<const float*>(y), b->cap_stream);
  if (rc == PN_OK) rc = wcsph_step(b, b->cap_stream);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(b->cap_stream, &g);
  if (rc != PN_OK || ce != cudaSuccess || g == nullptr) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc != PN_OK ? rc : PN_ERR_CUDA;
  }
  if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    b->exec = nullptr;
    cudaGetLastError();
    return PN_ERR_CUDA;
  }
  b->graph = g;
  return PN_OK;
}

int pn_batch_launch_step(pn_batch* b, pn_stream_t stream) {
  PN_NVTX_RANGE("pn_batch_launch_step");
  if (!b || !b->exec) return PN_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int rc = cudaGraphLaunch(b->exec, st) == cudaSuccess ? PN_OK : PN_ERR_CUDA;
  return record(b, rc, st);
}

int pn_batch_sync(pn_batch* b) {
  if (!b) return PN_ERR_INVALID_ARG;
  if (cudaStreamSynchronize(b->last_stream) != cudaSuccess) return PN_ERR_CUDA;
  int32_t e = 0;
  if (cudaMemcpy(&e, b->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PN_ERR_CUDA;
  const int rc = b->host_error ? b->host_error : e;
  b->host_error = 0;
  if (e) cudaMemset(b->d_err, 0, sizeof(int32_t));
  return rc;
}

}  // extern "C"
