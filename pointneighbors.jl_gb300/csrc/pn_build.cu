// pn_build.cu -- cell-list build (initialize! / update! with ParallelUpdate), cell
// coordinates, cell export and the small scans/sorts used by the neighbour lists.
//
// The reference (nhs_grid.jl:255-281, vector_of_vectors.jl:93-112) pushes every point into
// a fixed-capacity column with one atomic per point.  Here the cell list is a counting
// sort into a CSR layout:
//   1. k_bin      per point: cell index (exact reference semantics, bounds check), then a
//                 warp-aggregated atomic increment of the cell histogram (lanes that share
//                 a cell issue one atomic) that also hands each point its rank.
//   2. k_scan     exclusive scan of the histogram -> cell starts, single pass with
//                 decoupled look-back (bounded waits), plus the max_points_per_cell check.
//   3. k_scatter  point -> slot start[cell] + rank.
//   4. k_finalize rank-sort each cell's points by their first coordinate, ties by point
//                 index (a deterministic order, independent of atomic timing; a stencil
//                 row's three cells are then one x-sorted run) and write the cell-sorted
//                 coordinates.
#include <algorithm>

#include "pn_internal.cuh"

namespace pn {

constexpr int BIN_THREADS = 256;
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr unsigned long long FLAG_AGG = 1ull << 32;
constexpr unsigned long long FLAG_INCL = 2ull << 32;
constexpr long long SCAN_SPIN_LIMIT = 1ll << 22;

// ParallelIncrementalUpdate decides on the device, after counting the movers, between
// keeping the main structure plus overflow lists and a full rebuild; the kernels of both
// paths are launched and each returns at once unless the decision word selects it.
constexpr int32_t GATE_OVERFLOW = 0, GATE_REBUILD = 1;

// ---------------------------------------------------------------- 1. histogram
template <typename T, int D, bool PER>
__global__ void __launch_bounds__(BIN_THREADS)
k_bin(const GridDev<T> g, const T* __restrict__ y, int64_t n_y, const int32_t* __restrict__ idx,
      int32_t m, int32_t* __restrict__ cell_of, int32_t* __restrict__ slot_of,
      int32_t* __restrict__ counts, int32_t* __restrict__ outside, int32_t* __restrict__ err,
      const int32_t* __restrict__ gate) {
  if (gate && *gate != GATE_REBUILD) return;
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = base + threadIdx.x;
    int32_t cell = -1;
    if (t < m) {
      const int64_t i = idx ? (int64_t)idx[t] : t;
      if (i < 0 || i >= n_y) {
        set_error(err, PN_ERR_INVALID_ARG);
      } else {
        bool ok = true;
        int32_t lin = 0, stride = 1;
        bool out = false;
#pragma unroll
        for (int k = 0; k < D; ++k) {
          int32_t c;
          const T xk = y[i * D + k];
          ok &= cell_coord_1d(g, PER, k, xk, c);
          if (PER) out |= outside_box(g, k, xk);
          lin += (c - 1) * stride;
          stride *= g.n[k];
        }
        if (ok) cell = lin;
        else set_error(err, PN_ERR_OUT_OF_DOMAIN);
        if (PER && out && *(volatile int32_t*)outside == 0) atomicExch(outside, 1);
      }
    }
    // `base` is uniform over the block, so every lane of the warp reaches this point.
    const unsigned valid = __ballot_sync(0xffffffffu, cell >= 0);
    if (cell >= 0) {
      const unsigned peers = __match_any_sync(valid, cell);
      const int leader = __ffs(peers) - 1;
      int32_t b = 0;
      if (lane == leader) b = atomicAdd(&counts[PN_IDX(err, BC_CELL, cell, g.n_total)],
                                         __popc(peers));
      b = __shfl_sync(peers, b, leader);
      slot_of[t] = b + __popc(peers & lanemask_lt());
    }
    if (t < m) cell_of[t] = cell;
  }
}

// ---------------------------------------------------------------- 2. scan
// Exclusive scan of counts[0..n) into start[0..n], start[n] = total.  Tiles are taken in
// launch order from a counter, so a tile only ever waits for tiles that are already
// running; every wait is bounded and reports PN_ERR_TIMEOUT if it gives up.
// stats (or null): stats[0] = the largest count (atomicMax, cleared by the caller),
// stats[1] = 1 when some count exceeds max_ppc (the build then skips the in-cell sort).
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_cells(const int32_t* __restrict__ counts, int32_t n, int32_t* __restrict__ start,
             unsigned long long* __restrict__ state, int32_t n_tiles, int32_t max_ppc,
             const int32_t* __restrict__ base_ptr, int32_t* __restrict__ err,
             const int32_t* __restrict__ gate, int32_t gate_want,
             int32_t* __restrict__ stats = nullptr) {
  if (gate && *gate != gate_want) return;  // the same word for every block
  __shared__ int s_tile, s_prefix;
  __shared__ int s_warp[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(&state[n_tiles], 1ull);
  __syncthreads();
  const int tile = s_tile;
  const int64_t base = (int64_t)tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  if (base + SCAN_ITEMS <= n) {
    const int4 a = *reinterpret_cast<const int4*>(counts + base);
    const int4 b = *reinterpret_cast<const int4*>(counts + base + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) v[i] = (base + i < n) ? counts[base + i] : 0;
  }
  int sum = 0, mx = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    sum += v[i];
    mx = max(mx, v[i]);
  }
  if (max_ppc > 0 && mx > max_ppc) {
    set_error(err, PN_ERR_CELL_FULL);
    if (stats) stats[1] = 1;
  }
  if (stats) {
    const int wmx = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0 && wmx > 0) atomicMax(&stats[0], wmx);
  }
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < SCAN_THREADS / 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < SCAN_THREADS / 32) s_warp[lane] = w;
  }
  __syncthreads();
  const int aggregate = s_warp[SCAN_THREADS / 32 - 1];
  const int thread_excl = (warp > 0 ? s_warp[warp - 1] : 0) + incl - sum;
  if (threadIdx.x == 0) {
    int prefix = 0;
    if (tile == 0) {
      atomicExch(&state[0], FLAG_INCL | (unsigned)aggregate);
    } else {
      atomicExch(&state[tile], FLAG_AGG | (unsigned)aggregate);
      int j = tile - 1;
      long long spins = 0;
      while (j >= 0) {
        const unsigned long long st = *(volatile unsigned long long*)&state[j];
        const unsigned long long flag = st & (3ull << 32);
        if (flag == 0) {
          if (++spins > SCAN_SPIN_LIMIT) {
            set_error(err, PN_ERR_TIMEOUT);
            break;
          }
          __nanosleep(32);
          continue;
        }
        prefix += (int)(unsigned)(st & 0xffffffffull);
        if (flag == FLAG_INCL) break;
        --j;
      }
      atomicExch(&state[tile], FLAG_INCL | (unsigned)(prefix + aggregate));
    }
    s_prefix = prefix;
  }
  __syncthreads();
  int run = s_prefix + thread_excl + (base_ptr ? *base_ptr : 0);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) {
      start[base + i] = run;
      run += v[i];
      if (base + i == n - 1) start[n] = run;
    }
  }
}

// ---------------------------------------------------------------- 3. scatter
__global__ void __launch_bounds__(256)
k_scatter(const int32_t* __restrict__ cell_of, const int32_t* __restrict__ slot_of,
          const int32_t* __restrict__ idx, int32_t m, const int32_t* __restrict__ start,
          int32_t* __restrict__ tmp_perm, int32_t* __restrict__ cell_of_slot,
          const int32_t* __restrict__ gate, int32_t* __restrict__ err = nullptr,
          int32_t n_cells = INT32_MAX, int64_t n_slots = INT64_MAX) {
  if (gate && *gate != GATE_REBUILD) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const int32_t c0 = cell_of[t];
  if (c0 < 0) return;
  const int32_t c = PN_IDX(err, BC_CELL, c0, n_cells);
  const int32_t p = PN_IDX(err, BC_SLOT, start[c] + slot_of[t], n_slots);
  tmp_perm[p] = idx ? idx[t] : (int32_t)t;
  cell_of_slot[p] = c;
}

// ---------------------------------------------------------------- 4. in-cell sort
template <typename T, int D>
__device__ __forceinline__ void store_pos(T* pos, int64_t k, const T* v) {
  constexpr int S = PS<D>::value;
#pragma unroll
  for (int c = 0; c < S; ++c) pos[k * S + c] = c < D ? v[c] : (T)0;
}

// Cells with more points than this are ranked by k_finalize_large (their keys streamed
// through shared memory) instead of one thread per slot reading the whole cell.
constexpr int32_t LARGE_CELL = 256;
constexpr int LARGE_TILE = 1024;

// stats (see k_scan_cells) or null: with stats, cells above LARGE_CELL are left to
// k_finalize_large, and after a failed max_points_per_cell check every slot keeps its
// scatter position (no sort: the build has failed, but the arrays hold valid indices).
template <typename T, int D>
__device__ __forceinline__ void finalize_slot(const int32_t* __restrict__ tmp_perm,
                                              const int32_t* __restrict__ cell_of_slot,
                                              const int32_t* __restrict__ start, int64_t k,
                                              const T* __restrict__ y, int32_t* __restrict__ perm,
                                              T* __restrict__ pos,
                                              const int32_t* __restrict__ stats = nullptr,
                                              float* __restrict__ xkey = nullptr) {
  const int32_t c = cell_of_slot[k];
  const int32_t s = start[c], e = start[c + 1];
  const int32_t v = tmp_perm[k];
  const bool failed = stats != nullptr && stats[1] != 0;
  if (stats != nullptr && !failed && e - s > LARGE_CELL) return;
  // inside the cell: ascending first coordinate, ties by point index (a total order, so
  // the layout is deterministic); a stencil row's three cells are then one x-sorted run
  const T xv = y[(int64_t)v * D];
  int32_t rank = (int32_t)k - s;
  if (!failed) {
    rank = 0;
    for (int32_t q = s; q < e; ++q) {
      const int32_t u = __ldg(&tmp_perm[q]);
      const T xu = __ldg(&y[(int64_t)u * D]);
      rank += (xu < xv) || (xu == xv && u < v);
    }
  }
  const int32_t dst = s + rank;
  perm[dst] = v;
  T p[D];
#pragma unroll
  for (int d = 0; d < D; ++d) p[d] = y[(int64_t)v * D + d];
  store_pos<T, D>(pos, dst, p);
  if constexpr (std::is_same<T, float>::value) {
    if (xkey != nullptr) xkey[dst] = p[0];  // the sort key: x when the cell was sorted
  }
}

template <typename T, int D>
__global__ void __launch_bounds__(256)
k_finalize(const int32_t* __restrict__ tmp_perm, const int32_t* __restrict__ cell_of_slot,
           const int32_t* __restrict__ start, int32_t n_total, const T* __restrict__ y,
           int32_t* __restrict__ perm, T* __restrict__ pos, const int32_t* __restrict__ gate,
           const int32_t* __restrict__ stats = nullptr, float* __restrict__ xkey = nullptr) {
  if (gate && *gate != GATE_REBUILD) return;
  // Only start[n_total] slots were filled: points that failed the bounds check were not
  // binned, so the slot count is read on the device.
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= start[n_total]) return;
  finalize_slot<T, D>(tmp_perm, cell_of_slot, start, k, y, perm, pos, stats, xkey);
}

// The in-cell rank of the slots of cells above LARGE_CELL points (cells, or hash lists with
// HASH, whose order is (cell key, first coordinate, point index)).  A block takes 256
// consecutive slots; when some of them lie in large cells, the block streams the keys of
// those cells through shared memory, LARGE_TILE at a time, and every thread counts the keys
// of its own cell that order before its own.  A cell of k points costs k^2 comparisons
// from shared memory instead of k^2 dependent global loads.  Grid-stride over the slots;
// returns at once when the build has no large cell (stats[0]) or failed the cell limit.
template <typename T, int D, bool HASH>
__global__ void __launch_bounds__(256)
k_finalize_large(const int32_t* __restrict__ tmp_perm, const int32_t* __restrict__ cell_of_slot,
                 const int4* __restrict__ key_tmp, const int32_t* __restrict__ start,
                 int32_t n_total, const T* __restrict__ y, int32_t* __restrict__ perm,
                 T* __restrict__ pos, int4* __restrict__ key, const int32_t* __restrict__ stats,
                 const int32_t* __restrict__ gate, float* __restrict__ xkey = nullptr) {
  if (gate && *gate != GATE_REBUILD) return;
  if (stats[0] <= LARGE_CELL || stats[1] != 0) return;
  __shared__ T s_x[LARGE_TILE];
  __shared__ int32_t s_u[LARGE_TILE];
  __shared__ int4 s_k[HASH ? LARGE_TILE : 1];
  __shared__ int32_t s_lo, s_hi;
  const int32_t n = start[n_total];
  for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x; t0 < n;
       t0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t0 + threadIdx.x;
    bool large = false;
    int32_t s = 0, e = 0, v = 0;
    T xv = (T)0;
    int4 kv = make_int4(0, 0, 0, 0);
    if (threadIdx.x == 0) {
      s_lo = INT32_MAX;
      s_hi = INT32_MIN;
    }
    __syncthreads();
    if (k < n) {
      const int32_t c = cell_of_slot[k];
      s = start[c];
      e = start[c + 1];
      large = e - s > LARGE_CELL;
    }
    if (large) {
      atomicMin(&s_lo, s);
      atomicMax(&s_hi, e);
      v = tmp_perm[k];
      xv = y[(int64_t)v * D];
      if (HASH) kv = key_tmp[k];
    }
    __syncthreads();
    const int32_t lo = s_lo, hi = s_hi;  // hi <= lo: no large cell in this block
    int32_t rank = 0;
    for (int32_t base = lo; base < hi; base += LARGE_TILE) {
      const int32_t m = min(LARGE_TILE, hi - base);
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int32_t u = tmp_perm[base + i];
        s_u[i] = u;
        s_x[i] = y[(int64_t)u * D];
        if (HASH) s_k[i] = key_tmp[base + i];
      }
      __syncthreads();
      if (large) {
        const int32_t i0 = max(s - base, 0), i1 = min(e - base, m);
        for (int32_t i = i0; i < i1; ++i) {
          const T xu = s_x[i];
          const int32_t u = s_u[i];
          bool before = (xu < xv) || (xu == xv && u < v);
          if (HASH) {
            const int4 ku = s_k[i];
            const bool eq = ku.x == kv.x && ku.y == kv.y && ku.z == kv.z;
            const bool lt = ku.x != kv.x ? ku.x < kv.x : (ku.y != kv.y ? ku.y < kv.y : ku.z < kv.z);
            before = lt || (eq && before);
          }
          rank += before;
        }
      }
      __syncthreads();
    }
    if (large) {
      const int32_t dst = s + rank;
      perm[dst] = v;
      if (HASH) key[dst] = kv;
      T p[D];
#pragma unroll
      for (int d = 0; d < D; ++d) p[d] = y[(int64_t)v * D + d];
      store_pos<T, D>(pos, dst, p);
      if constexpr (std::is_same<T, float>::value) {
        if (xkey != nullptr) xkey[dst] = p[0];
      }
    }
    __syncthreads();  // every thread has read s_lo / s_hi before they are reset
  }
}

// ---------------------------------------------------------------- incremental update
// ParallelIncrementalUpdate (nhs_grid.jl:408-467) moves only the points whose cell
// changed.  Here the main structure of the last full build stays in place; every update
// re-checks all points against their main cell and
//   - refreshes the coordinates of points still in their main cell (in place),
//   - vacates the main slot of every other point (perm = -1, NaN coordinates, which no
//     distance test accepts) and re-bins it into the overflow lists: a second CSR over the
//     same cells, stored in the slots after the main ones.
// The traversal visits both lists for every stencil row.  Because the overflow is rebuilt
// relative to the main structure on every update, it never accumulates; a full rebuild
// (which empties it) is taken when the movers exceed a threshold.
template <typename T, int D, bool PER>
__global__ void __launch_bounds__(256)
k_mark_movers(const GridDev<T> g, const int32_t* __restrict__ main_perm,
              const int32_t* __restrict__ cell_of_slot, const int32_t* __restrict__ n_main,
              const T* __restrict__ y, int32_t* __restrict__ perm, T* __restrict__ pos,
              int32_t* __restrict__ ovf_counts, int32_t* __restrict__ ovf_n,
              int32_t* __restrict__ ovf_list, int32_t* __restrict__ ovf_cell,
              int32_t* __restrict__ ovf_slot, int32_t* __restrict__ outside,
              int32_t* __restrict__ err, const float* __restrict__ xkey,
              int32_t* __restrict__ cell_of, int32_t* __restrict__ slot_of,
              int32_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int32_t nm = *n_main;
  int32_t ovf_max = 0;  // the largest overflow list this thread has seen grow
  float dmax = 0.0f;    // the largest |x - xkey| of a slot refreshed in place
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nm;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = base + threadIdx.x;
    int32_t cell = -1;
    bool moved = false;
    int32_t i = -1;
    int32_t hcell = -1;  // the point's current cell, for the rebuild's histogram
    if (k < nm) {
      i = main_perm[k];
      T p[D];
      bool ok = true, out = false;
      int32_t lin = 0, stride = 1;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        p[d] = y[(int64_t)i * D + d];
        int32_t c;
        ok &= cell_coord_1d(g, PER, d, p[d], c);
        if (PER) out |= outside_box(g, d, p[d]);
        lin += (c - 1) * stride;
        stride *= g.n[d];
      }
      if (PER && out && *(volatile int32_t*)outside == 0) atomicExch(outside, 1);
      if (ok) hcell = lin;
      if (!ok) {
        set_error(err, PN_ERR_OUT_OF_DOMAIN);
      } else if (lin == cell_of_slot[k]) {
        perm[k] = i;
        store_pos<T, D>(pos, k, p);
        if constexpr (std::is_same<T, float>::value) {
          if (xkey != nullptr) dmax = fmaxf(dmax, fabsf(__fsub_rn(p[0], xkey[k])));
        }
      } else {
        moved = true;
        cell = lin;
      }
      if (!ok || moved) {
        perm[k] = -1;
        T nan_p[D];
#pragma unroll
        for (int d = 0; d < D; ++d) nan_p[d] = (T)NAN;
        store_pos<T, D>(pos, k, nan_p);
      }
    }
    // The rebuild's histogram, as k_bin would make it (cell and rank per point index): the
    // rebuild path then needs no bin of its own.  `base` is uniform over the block, so
    // every lane of the warp reaches the ballots.
    const unsigned hv = __ballot_sync(0xffffffffu, hcell >= 0);
    if (hcell >= 0) {
      const unsigned peers = __match_any_sync(hv, hcell);
      const int leader = __ffs(peers) - 1;
      int32_t hb = 0;
      if (lane == leader)
        hb = atomicAdd(&counts[PN_IDX(err, BC_CELL, hcell, g.n_total)], __popc(peers));
      hb = __shfl_sync(peers, hb, leader);
      slot_of[i] = hb + __popc(peers & lanemask_lt());
    }
    if (k < nm) cell_of[i] = hcell;
    // Movers: one list entry each (warp-aggregated), plus their rank in the new cell.
    const unsigned mv = __ballot_sync(0xffffffffu, moved);
    if (mv) {
      int32_t b = 0;
      if (lane == __ffs(mv) - 1) b = atomicAdd(ovf_n, __popc(mv));
      b = __shfl_sync(0xffffffffu, b, __ffs(mv) - 1);
      if (moved) {
        const int32_t m = b + __popc(mv & lanemask_lt());
        const unsigned peers = __match_any_sync(mv, cell);
        const int leader = __ffs(peers) - 1;
        int32_t cb = 0;
        if (lane == leader) {
          cb = atomicAdd(&ovf_counts[cell], __popc(peers));
          ovf_max = max(ovf_max, cb + __popc(peers));  // the cell's overflow list so far
        }
        cb = __shfl_sync(peers, cb, leader);
        ovf_list[m] = i;
        ovf_cell[m] = cell;
        ovf_slot[m] = cb + __popc(peers & lanemask_lt());
      }
    }
  }
  // one atomic per block: the block's loop bounds are uniform, so every thread gets here.
  // dmax >= 0, so its bits order like the values.
  __shared__ int32_t s_max, s_dmax;
  if (threadIdx.x == 0) s_max = s_dmax = 0;
  __syncthreads();
  const int32_t wmax = __reduce_max_sync(0xffffffffu, ovf_max);
  const int32_t wd = __reduce_max_sync(0xffffffffu, __float_as_int(dmax));
  if (lane == 0 && wmax > 0) atomicMax(&s_max, wmax);
  if (lane == 0 && wd > 0) atomicMax(&s_dmax, wd);
  __syncthreads();
  if (threadIdx.x == 0 && s_max > 0) atomicMax(&ovf_n[1], s_max);
  if (threadIdx.x == 0 && s_dmax > 0) atomicMax(&err[ERR_DELTA], s_dmax);
}

// Movers -> their overflow slots (ovf_start is absolute: it starts after the main slots).
__global__ void __launch_bounds__(256)
k_scatter_movers(const int32_t* __restrict__ ovf_n, const int32_t* __restrict__ ovf_list,
                 const int32_t* __restrict__ ovf_cell, const int32_t* __restrict__ ovf_slot,
                 const int32_t* __restrict__ ovf_start, int32_t* __restrict__ tmp_perm,
                 int32_t* __restrict__ cell_of_slot, const int32_t* __restrict__ gate,
                 int32_t* __restrict__ err, int32_t n_cells, int64_t n_slots) {
  if (*gate != GATE_OVERFLOW) return;
  const int32_t n = *ovf_n;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < n;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = PN_IDX(err, BC_CELL, ovf_cell[m], n_cells);
    const int32_t p = PN_IDX(err, BC_SLOT, ovf_start[c] + ovf_slot[m], n_slots);
    tmp_perm[p] = ovf_list[m];
    cell_of_slot[p] = c;
  }
}

// In-cell sort + coordinates of the overflow slots [start_main[n_total], ovf_start[n_total]).
template <typename T, int D>
__global__ void __launch_bounds__(256)
k_finalize_movers(const int32_t* __restrict__ tmp_perm, const int32_t* __restrict__ cell_of_slot,
                  const int32_t* __restrict__ ovf_start, const int32_t* __restrict__ n_main,
                  int32_t n_total, const T* __restrict__ y, int32_t* __restrict__ perm,
                  T* __restrict__ pos, const int32_t* __restrict__ gate,
                  float* __restrict__ xkey) {
  if (*gate != GATE_OVERFLOW) return;
  const int32_t k0 = *n_main, k1 = ovf_start[n_total];
  for (int64_t k = k0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < k1;
       k += (int64_t)gridDim.x * blockDim.x)
    finalize_slot<T, D>(tmp_perm, cell_of_slot, ovf_start, k, y, perm, pos, nullptr, xkey);
}

// The decision: rebuild when the points outside their main cell exceed `fraction` of the
// binned points (the traversal cost of the overflow lists grows with them, while a full
// rebuild costs about as much as marking the movers), or when some cell's overflow list
// would exceed LARGE_CELL points (k_finalize_movers ranks one cell's list per thread).
// gate[1] ("unsorted") tells the traversal that the main slots are no longer sorted by x
// inside their cells (the overflow path refreshes positions in place).
__global__ void k_decide_update(const int32_t* __restrict__ ovf_n,
                                const int32_t* __restrict__ n_main, double fraction,
                                int32_t* __restrict__ gate) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const int32_t m = ((double)ovf_n[0] > fraction * (double)*n_main || ovf_n[1] > LARGE_CELL)
                          ? GATE_REBUILD : GATE_OVERFLOW;
    gate[0] = m;
    gate[1] = m == GATE_OVERFLOW ? 1 : 0;
  }
}

// Overflow path only: per cell the largest |x - xkey| of its main slots moved in place (the
// rows' clipping margins, cell_delta zeroed by the caller).  Slots are cell-sorted, so a
// warp's lanes mostly share a cell: one atomic per cell and warp; the distances are >= 0,
// so their bits order like the values.
template <int S>
__global__ void __launch_bounds__(256)
k_cell_delta(const float* __restrict__ pos, const float* __restrict__ xkey,
             const int32_t* __restrict__ perm, const int32_t* __restrict__ cell_of_slot,
             const int32_t* __restrict__ n_main, int32_t n_total, float* __restrict__ cell_delta,
             const int32_t* __restrict__ gate, int32_t* __restrict__ err) {
  if (*gate != GATE_OVERFLOW) return;
  const int32_t nm = *n_main;
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nm;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = base + threadIdx.x;
    int32_t cell = -1;
    float d = 0.0f;
    if (k < nm && perm[k] >= 0) {
      cell = cell_of_slot[k];
      d = fabsf(__fsub_rn(pos[k * S], xkey[k]));
    }
    const unsigned act = __ballot_sync(0xffffffffu, cell >= 0);
    if (cell >= 0) {
      const unsigned peers = __match_any_sync(act, cell);
      const int32_t mb = __reduce_max_sync(peers, __float_as_int(d));
      if (lane == __ffs(peers) - 1 && mb > 0)
        atomicMax(reinterpret_cast<int32_t*>(cell_delta) + PN_IDX(err, BC_CELL, cell, n_total),
                  mb);
    }
  }
}

// After a rebuild the new structure is the main one: empty overflow lists, main_perm = perm.
__global__ void __launch_bounds__(256)
k_reset_overflow(const int32_t* __restrict__ start, int32_t n_total,
                 const int32_t* __restrict__ perm, int32_t* __restrict__ main_perm,
                 int32_t* __restrict__ ovf_start, int32_t* __restrict__ ovf_n,
                 const int32_t* __restrict__ gate, int32_t* __restrict__ delta) {
  if (*gate != GATE_REBUILD) return;
  const int32_t nm = start[n_total];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c <= n_total; c += stride)
    ovf_start[c] = nm;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nm; k += stride)
    main_perm[k] = perm[k];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *ovf_n = 0;
    *delta = 0;  // every slot holds its sort key again
  }
}

// ---------------------------------------------------------------- host side
template <typename T, int D, bool PER>
static void launch_bin(pn_search* s, const T* y, int64_t n_y, const int32_t* idx, int32_t m,
                       cudaStream_t st, const int32_t* gate) {
  const int blocks = std::max(1, std::min(div_up(m, BIN_THREADS), 152 * 8));
  k_bin<T, D, PER><<<blocks, BIN_THREADS, 0, st>>>(make_grid<T>(s), y, n_y, idx, m,
                                                   s->d_cell_of, s->d_slot_of, s->d_counts,
                                                   s->d_err + 1, s->d_err, gate); count_launch();
}

template <typename T>
static void dispatch_bin(pn_search* s, const T* y, int64_t n_y, const int32_t* idx,
                         int32_t m, cudaStream_t st, const int32_t* gate = nullptr) {
  const bool per = s->periodic != 0;
  switch (s->ndims * 2 + (per ? 1 : 0)) {
    case 2: launch_bin<T, 1, false>(s, y, n_y, idx, m, st, gate); break;
    case 3: launch_bin<T, 1, true>(s, y, n_y, idx, m, st, gate); break;
    case 4: launch_bin<T, 2, false>(s, y, n_y, idx, m, st, gate); break;
    case 5: launch_bin<T, 2, true>(s, y, n_y, idx, m, st, gate); break;
    case 6: launch_bin<T, 3, false>(s, y, n_y, idx, m, st, gate); break;
    default: launch_bin<T, 3, true>(s, y, n_y, idx, m, st, gate); break;
  }
}

// The build's cell statistics (k_scan_cells): [0] largest cell, [1] cell limit exceeded.
static int32_t* build_stats(pn_search* s) { return s->d_err + 5; }

// The in-cell sort: k_finalize for cells up to LARGE_CELL points, then k_finalize_large
// (one wave of blocks; it returns at once when the build has no larger cell).
template <typename T>
static void launch_finalize(pn_search* s, const T* y, int32_t m, cudaStream_t st,
                            const int32_t* gate = nullptr) {
  const int blocks = div_up(m, 256);
  if (blocks == 0) return;
  T* pos = static_cast<T*>(s->d_pos);
  const int32_t nt = s->n_total;
  const int32_t* stats = build_stats(s);
  const int lb = std::min(blocks, 152 * 4);
  switch (s->ndims) {
    case 1:
      k_finalize<T, 1><<<blocks, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_start, nt, y, s->d_perm, pos, gate, stats, s->d_xkey);
      k_finalize_large<T, 1, false><<<lb, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, nullptr, s->d_start, nt, y, s->d_perm, pos, nullptr, stats, gate, s->d_xkey);
      break;
    case 2:
      k_finalize<T, 2><<<blocks, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_start, nt, y, s->d_perm, pos, gate, stats, s->d_xkey);
      k_finalize_large<T, 2, false><<<lb, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, nullptr, s->d_start, nt, y, s->d_perm, pos, nullptr, stats, gate, s->d_xkey);
      break;
    default:
      k_finalize<T, 3><<<blocks, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_start, nt, y, s->d_perm, pos, gate, stats, s->d_xkey);
      k_finalize_large<T, 3, false><<<lb, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, nullptr, s->d_start, nt, y, s->d_perm, pos, nullptr, stats, gate, s->d_xkey);
      break;
  }
  count_launch();
  count_launch();
}

// Exclusive scan of the cell histogram into s->d_start (one launch).
// start[c] = *base_ptr + sum(counts[0..c)) when base_ptr is given.
// The cell-list scans record the build's statistics; the overflow lists' scan does not.
static void scan_cells(pn_search* s, const int32_t* counts, int32_t* start, cudaStream_t st,
                       const int32_t* base_ptr = nullptr, int32_t max_ppc = 0,
                       const int32_t* gate = nullptr, int32_t gate_want = 0,
                       bool stats = true) {
  cudaMemsetAsync(s->d_scan_state, 0, sizeof(unsigned long long) * (s->scan_tiles + 1), st);
  k_scan_cells<<<s->scan_tiles, SCAN_THREADS, 0, st>>>(counts, s->n_total, start,
                                                       s->d_scan_state, s->scan_tiles,
                                                       max_ppc, base_ptr, s->d_err, gate,
                                                       gate_want,
                                                       stats ? build_stats(s) : nullptr);
  count_launch();
}

template <typename T>
int build(pn_search* s, const T* y, int64_t n_y, const int32_t* idx, int64_t n_idx,
          cudaStream_t st) {
  const int64_t m = idx ? n_idx : n_y;
  int rc = ensure_capacity(s, std::max(m, n_y));
  if (rc != PN_OK) return rc;
  cudaMemsetAsync(s->d_counts, 0, sizeof(int32_t) * s->n_total, st);
  cudaMemsetAsync(s->d_err + 1, 0, sizeof(int32_t), st);  // points outside the periodic box
  cudaMemsetAsync(s->d_err + 3, 0, sizeof(int32_t), st);  // cells sorted by x again
  cudaMemsetAsync(build_stats(s), 0, 2 * sizeof(int32_t), st);
  if (m > 0) dispatch_bin<T>(s, y, n_y, idx, (int32_t)m, st);
  scan_cells(s, s->d_counts, s->d_start, st, nullptr, s->cfg.max_points_per_cell);
  if (m > 0) {
    k_scatter<<<div_up(m, 256), 256, 0, st>>>(s->d_cell_of, s->d_slot_of, idx, (int32_t)m,
                                              s->d_start, s->d_tmp_perm, s->d_cell_of_slot,
                                              nullptr, s->d_err, s->n_total, slot_capacity(s));
    count_launch();
    // Points rejected by the bounds check are not binned; every kernel that walks the
    // slots bounds itself by start[n_total], read on the device.
    launch_finalize<T>(s, y, (int32_t)m, st);
  }
  cudaMemsetAsync(s->d_err + ERR_DELTA, 0, sizeof(int32_t), st);
  if (s->d_cell_delta) cudaMemsetAsync(s->d_cell_delta, 0, sizeof(float) * s->n_total, st);
  s->n_binned = m;
  s->pc_valid = false;
  s->ovf_active = false;
  s->main_perm_valid = false;
  s->n_ovf = 0;
  s->updates_since_build = 0;
  refresh_pos32(s, st);
  return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------- SpatialHashingCellList
// The same counting sort with the hash list as the bucket (spatial_hashing.jl:91-126 pushes
// into the hash lists).  Inside a list the points are ranked by cell, then by first
// coordinate and index, so that each cell is a contiguous, x-sorted run; a scan of the
// run heads numbers the cells, which become the entries (x, y, z, first slot) that the
// traversal matches against the cells of a stencil.  The reference instead stores one
// coordinate tuple and a collision flag per list and compares each point's cell while
// traversing (nhs_grid.jl:479-513); both visit exactly the points of the stencil's cells.
// Every point's cell (w = 1 when binned, 0 after an error) and the bounding box of the
// occupied cells (one atomic per warp and bound).
template <typename T, int D, bool PER>
__global__ void __launch_bounds__(BIN_THREADS)
k_hash_key(const GridDev<T> g, const T* __restrict__ y, int64_t n_y,
           const int32_t* __restrict__ idx, int32_t m, int4* __restrict__ key_of,
           int32_t* __restrict__ bbox, int32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = base + threadIdx.x;
    bool ok = false;
    int32_t c[3] = {0, 0, 0};
    if (t < m) {
      const int64_t i = idx ? (int64_t)idx[t] : t;
      if (i < 0 || i >= n_y) {
        set_error(err, PN_ERR_INVALID_ARG);
      } else {
        ok = true;
#pragma unroll
        for (int k = 0; k < D; ++k) ok &= hash_cell_1d(g, PER, k, y[i * D + k], c[k]);
        if (!ok) set_error(err, PN_ERR_OUT_OF_DOMAIN);
      }
    }
    const unsigned valid = __ballot_sync(0xffffffffu, ok);
    if (ok) {
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const int32_t lo = __reduce_min_sync(valid, c[k]);
        const int32_t hi = __reduce_max_sync(valid, c[k]);
        if (lane == __ffs(valid) - 1) {
          atomicMin(&bbox[k], lo);
          atomicMax(&bbox[3 + k], hi);
        }
      }
    }
    if (t < m) key_of[t] = make_int4(c[0], c[1], c[2], ok ? 1 : 0);
  }
}

// The hash list of every binned point and its rank in the list (a warp-aggregated
// histogram), for the per-list max_points_per_cell check and the hash-list layout.
template <int D>
__global__ void __launch_bounds__(BIN_THREADS)
k_hash_list_bin(const HashMod hm, const int4* __restrict__ key_of, int32_t m,
                int32_t* __restrict__ bucket_of, int32_t* __restrict__ slot_of,
                int32_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = base + threadIdx.x;
    int32_t bucket = -1;
    if (t < m) {
      const int4 k4 = key_of[t];
      const int32_t c[3] = {k4.x, k4.y, k4.z};
      if (k4.w) bucket = spatial_hash<D>(c, hm);
    }
    const unsigned valid = __ballot_sync(0xffffffffu, bucket >= 0);
    if (bucket >= 0) {
      const unsigned peers = __match_any_sync(valid, bucket);
      const int leader = __ffs(peers) - 1;
      int32_t b = 0;
      if (lane == leader) b = atomicAdd(&counts[bucket], __popc(peers));
      b = __shfl_sync(peers, b, leader);
      slot_of[t] = b + __popc(peers & lanemask_lt());
    }
    if (t < m) bucket_of[t] = bucket;
  }
}

__global__ void __launch_bounds__(256)
k_hash_scatter(const int32_t* __restrict__ bucket_of, const int32_t* __restrict__ slot_of,
               const int4* __restrict__ key_of, const int32_t* __restrict__ idx, int32_t m,
               const int32_t* __restrict__ start, int32_t* __restrict__ tmp_perm,
               int32_t* __restrict__ bucket_of_slot, int4* __restrict__ key_tmp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const int32_t b = bucket_of[t];
  if (b < 0) return;
  const int32_t p = start[b] + slot_of[t];
  tmp_perm[p] = idx ? idx[t] : (int32_t)t;
  bucket_of_slot[p] = b;
  key_tmp[p] = key_of[t];
}

__device__ __forceinline__ bool key_less(int4 a, int4 b) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z < b.z;
}
__device__ __forceinline__ bool key_eq(int4 a, int4 b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}

// Rank each slot inside its list by (cell, first coordinate, point index): a total order
// (NaN coordinates are not binned), so every slot gets a distinct destination.
template <typename T, int D>
__global__ void __launch_bounds__(256)
k_hash_finalize(const int32_t* __restrict__ tmp_perm, const int32_t* __restrict__ bucket_of_slot,
                const int4* __restrict__ key_tmp, const int32_t* __restrict__ start,
                int32_t n_total, const T* __restrict__ y, int32_t* __restrict__ perm,
                T* __restrict__ pos, int4* __restrict__ key, const int32_t* __restrict__ stats) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= start[n_total]) return;
  const int32_t b = bucket_of_slot[k];
  const int32_t s = start[b], e = start[b + 1];
  // as finalize_slot: large lists go to k_finalize_large, a failed limit check keeps order
  const bool failed = stats[1] != 0;
  if (!failed && e - s > LARGE_CELL) return;
  const int32_t v = tmp_perm[k];
  const int4 kv = key_tmp[k];
  const T xv = y[(int64_t)v * D];
  int32_t rank = (int32_t)k - s;
  if (!failed) {
    rank = 0;
    for (int32_t q = s; q < e; ++q) {
      const int32_t u = __ldg(&tmp_perm[q]);
      const int4 ku = __ldg(&key_tmp[q]);
      const T xu = __ldg(&y[(int64_t)u * D]);
      rank += key_less(ku, kv) || (key_eq(ku, kv) && ((xu < xv) || (xu == xv && u < v)));
    }
  }
  const int32_t dst = s + rank;
  perm[dst] = v;
  key[dst] = kv;
  T p[D];
#pragma unroll
  for (int d = 0; d < D; ++d) p[d] = y[(int64_t)v * D + d];
  store_pos<T, D>(pos, dst, p);
}

// head[k] = 1 where slot k starts a cell's run (slots [n, m) hold 0 for the scan).
__global__ void __launch_bounds__(256)
k_hash_heads(const int32_t* __restrict__ bucket_of_slot, const int4* __restrict__ key,
             const int32_t* __restrict__ n_slots, int32_t m, int32_t* __restrict__ head) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t n = *n_slots;
  int32_t h = 0;
  if (k < n)
    h = (k == 0 || bucket_of_slot[k] != bucket_of_slot[k - 1] || !key_eq(key[k], key[k - 1]))
            ? 1 : 0;
  head[k] = h;
}

// The cell entries (a sentinel entry after the last closes its run) and each list's first
// entry.
__global__ void __launch_bounds__(256)
k_hash_cells(const int32_t* __restrict__ head, const int32_t* __restrict__ cellidx,
             const int4* __restrict__ key, const int32_t* __restrict__ n_slots, int32_t m,
             int4* __restrict__ hcell) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t n = *n_slots;
  if (k < n && head[k]) {
    const int4 c = key[k];
    hcell[cellidx[k]] = make_int4(c.x, c.y, c.z, (int32_t)k);
  }
  if (k == 0) hcell[cellidx[m]] = make_int4(0, 0, 0, n);
}

__global__ void __launch_bounds__(256)
k_hash_buckets(const int32_t* __restrict__ start, const int32_t* __restrict__ cellidx,
               int32_t n_lists, int32_t* __restrict__ hbucket) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b <= n_lists) hbucket[b] = cellidx[start[b]];
}

__global__ void k_hash_bbox_init(int32_t* bbox) {
  if (threadIdx.x < 3) bbox[threadIdx.x] = INT32_MAX;
  else if (threadIdx.x < 6) bbox[threadIdx.x] = INT32_MIN;
}

// The dense layout: grid index = cell + off (1-based, column-major over n), binned like the
// full grid's k_bin from the cells found by k_hash_key.
template <int D>
__global__ void __launch_bounds__(BIN_THREADS)
k_hash_dense_bin(const int4* __restrict__ key_of, int32_t m, int3 off, int3 n,
                 int32_t* __restrict__ cell_of, int32_t* __restrict__ slot_of,
                 int32_t* __restrict__ counts, int32_t* __restrict__ err) {
  const int64_t n_cells = (int64_t)n.x * (D >= 2 ? n.y : 1) * (D == 3 ? n.z : 1);
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = base + threadIdx.x;
    int32_t cell = -1;
    const int4 c = t < m ? key_of[t] : make_int4(0, 0, 0, 0);
    if (c.w) {
      cell = c.x + off.x - 1;
      if (D >= 2) cell += (c.y + off.y - 1) * n.x;
      if (D == 3) cell += (c.z + off.z - 1) * n.x * n.y;
    }
    const unsigned valid = __ballot_sync(0xffffffffu, cell >= 0);
    if (cell >= 0) {
      const unsigned peers = __match_any_sync(valid, cell);
      const int leader = __ffs(peers) - 1;
      int32_t b = 0;
      if (lane == leader) b = atomicAdd(&counts[PN_IDX(err, BC_CELL, cell, n_cells)],
                                         __popc(peers));
      b = __shfl_sync(peers, b, leader);
      slot_of[t] = b + __popc(peers & lanemask_lt());
    }
    if (t < m) cell_of[t] = cell;
  }
}

static int ensure_hash_capacity(pn_search* s, int64_t n) {
  if (n <= s->hash_cap && s->d_hkey) return PN_OK;
  void* ptrs[] = {s->d_hkey_t, s->d_hkey_tmp, s->d_hkey, s->d_hcellidx, s->d_hcell,
                  s->d_hscan_state};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  s->d_hkey_t = s->d_hkey_tmp = s->d_hkey = s->d_hcell = nullptr;
  s->d_hcellidx = nullptr;
  s->d_hscan_state = nullptr;
  s->hash_cap = 0;
  const int64_t cap = std::max<int64_t>(s->cap, n);
  bool ok = cudaMalloc(&s->d_hkey_t, sizeof(int4) * cap) == cudaSuccess &&
            cudaMalloc(&s->d_hkey_tmp, sizeof(int4) * cap) == cudaSuccess &&
            cudaMalloc(&s->d_hkey, sizeof(int4) * (cap + 1)) == cudaSuccess &&
            cudaMalloc(&s->d_hcellidx, sizeof(int32_t) * (cap + 1)) == cudaSuccess &&
            cudaMalloc(&s->d_hcell, sizeof(int4) * (cap + 1)) == cudaSuccess &&
            cudaMalloc(&s->d_hscan_state,
                       sizeof(unsigned long long) * (scan_tile_count(cap) + 1)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return PN_ERR_OUT_OF_MEMORY;
  }
  s->hash_cap = cap;
  return PN_OK;
}

template <typename T>
int build_hash(pn_search* s, const T* y, int64_t n_y, const int32_t* idx, int64_t n_idx,
               cudaStream_t st) {
  const int64_t m = idx ? n_idx : n_y;
  int rc = ensure_capacity(s, std::max(m, n_y));
  if (rc == PN_OK) rc = ensure_hash_capacity(s, s->cap);
  if (rc != PN_OK) return rc;
  const int32_t nl = (int32_t)s->list_size;
  // 1. cells and their bounding box
  s->n_total = nl;
  s->hash_dense = false;
  cudaMemsetAsync(build_stats(s), 0, 2 * sizeof(int32_t), st);
  k_hash_bbox_init<<<1, 32, 0, st>>>(s->d_hbbox); count_launch();
  const int blocks = std::max(1, std::min(div_up(std::max<int64_t>(m, 1), BIN_THREADS), 152 * 8));
  if (m > 0) {
    const GridDev<T> g = make_grid<T>(s);
    const bool per = s->periodic != 0;
#define PN_HASH_KEY(DD, PP)                                                                  \
  k_hash_key<T, DD, PP><<<blocks, BIN_THREADS, 0, st>>>(g, y, n_y, idx, (int32_t)m,          \
                                                        s->d_hkey_t, s->d_hbbox, s->d_err)
    switch (s->ndims * 2 + (per ? 1 : 0)) {
      case 2: PN_HASH_KEY(1, false); break;
      case 3: PN_HASH_KEY(1, true); break;
      case 4: PN_HASH_KEY(2, false); break;
      case 5: PN_HASH_KEY(2, true); break;
      case 6: PN_HASH_KEY(3, false); break;
      default: PN_HASH_KEY(3, true); break;
    }
#undef PN_HASH_KEY
    count_launch();
  }
  // 2. the hash lists' histogram: for the per-list max_points_per_cell check, and for the
  // hash-list layout below
  auto list_bin = [&]() {
    cudaMemsetAsync(s->d_counts, 0, sizeof(int32_t) * nl, st);
    if (m > 0) {
      const HashMod hm = hash_mod(s->list_size);
      switch (s->ndims) {
        case 1: k_hash_list_bin<1><<<blocks, BIN_THREADS, 0, st>>>(hm, s->d_hkey_t, (int32_t)m, s->d_cell_of, s->d_slot_of, s->d_counts); break;
        case 2: k_hash_list_bin<2><<<blocks, BIN_THREADS, 0, st>>>(hm, s->d_hkey_t, (int32_t)m, s->d_cell_of, s->d_slot_of, s->d_counts); break;
        default: k_hash_list_bin<3><<<blocks, BIN_THREADS, 0, st>>>(hm, s->d_hkey_t, (int32_t)m, s->d_cell_of, s->d_slot_of, s->d_counts); break;
      }
      count_launch();
    }
    scan_cells(s, s->d_counts, s->d_start, st, nullptr, s->cfg.max_points_per_cell);
  };
  bool lists_binned = false;
  if (s->cfg.max_points_per_cell > 0) {
    list_bin();
    lists_binned = true;
  }
  // 3. the layout: a dense grid over the occupied cells' box when it has at most list_size
  // cells (read back: one synchronisation, like the reference's update!), else the lists
  cudaMemcpyAsync(s->h_hbbox, s->d_hbbox, sizeof(int32_t) * 6, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return PN_ERR_CUDA;
  const int32_t* bb = s->h_hbbox;
  int64_t dims[3] = {1, 1, 1}, cells = 1;
  bool dense = m > 0;
  for (int k = 0; k < s->ndims && dense; ++k) {
    if (bb[k] > bb[3 + k]) {
      dense = false;  // nothing binned
      break;
    }
    dims[k] = s->periodic ? s->n_cells[k] + 3 : (int64_t)bb[3 + k] - bb[k] + 5;
    cells *= dims[k];
    dense = cells <= (int64_t)nl;
  }
  for (int k = 0; k < 3; ++k) {
    s->grid_size[k] = 1;
    s->hash_off[k] = 0;
    s->min_pad[k] = s->max_pad[k] = 0.0;
  }
  if (dense) {
    // grid index = cell + off: the lowest cell at 3, two empty cells of padding on each
    // side (periodic: the cells 2..n_cells+1 themselves, like the full grid's)
    for (int k = 0; k < s->ndims; ++k) {
      s->grid_size[k] = dims[k];
      s->hash_off[k] = s->periodic ? 0 : 3 - bb[k];
      s->min_pad[k] = s->periodic ? 0.0 : ((double)bb[k] - 2.0) * s->cell_size[k];
      s->max_pad[k] = s->periodic ? 0.0 : ((double)bb[3 + k] + 3.0) * s->cell_size[k];
    }
    s->n_total = (int32_t)cells;
    s->hash_dense = true;
    cudaMemsetAsync(s->d_counts, 0, sizeof(int32_t) * cells, st);
    const int3 off = make_int3(s->hash_off[0], s->hash_off[1], s->hash_off[2]);
    const int3 n = make_int3((int32_t)dims[0], (int32_t)dims[1], (int32_t)dims[2]);
    switch (s->ndims) {
      case 1: k_hash_dense_bin<1><<<blocks, BIN_THREADS, 0, st>>>(s->d_hkey_t, (int32_t)m, off, n, s->d_cell_of, s->d_slot_of, s->d_counts, s->d_err); break;
      case 2: k_hash_dense_bin<2><<<blocks, BIN_THREADS, 0, st>>>(s->d_hkey_t, (int32_t)m, off, n, s->d_cell_of, s->d_slot_of, s->d_counts, s->d_err); break;
      default: k_hash_dense_bin<3><<<blocks, BIN_THREADS, 0, st>>>(s->d_hkey_t, (int32_t)m, off, n, s->d_cell_of, s->d_slot_of, s->d_counts, s->d_err); break;
    }
    count_launch();
    // (the search's scan state has room for the tiles of list_size >= cells counts)
    scan_counts(s->d_counts, (int32_t)cells, s->d_start, s->d_scan_state,
                scan_tile_count(cells), s->d_err, st, build_stats(s));
    k_scatter<<<div_up(m, 256), 256, 0, st>>>(s->d_cell_of, s->d_slot_of, idx, (int32_t)m,
                                              s->d_start, s->d_tmp_perm, s->d_cell_of_slot,
                                              nullptr, s->d_err, (int32_t)cells,
                                              slot_capacity(s));
    count_launch();
    launch_finalize<T>(s, y, (int32_t)m, st);
  } else if (m > 0) {
    // 4. the lists: each list's points ranked by (cell, x, index), one entry per cell
    if (!lists_binned) list_bin();
    const int b = div_up(m, 256);
    k_hash_scatter<<<b, 256, 0, st>>>(s->d_cell_of, s->d_slot_of, s->d_hkey_t, idx, (int32_t)m,
                                      s->d_start, s->d_tmp_perm, s->d_cell_of_slot,
                                      s->d_hkey_tmp); count_launch();
    T* pos = static_cast<T*>(s->d_pos);
    switch (s->ndims) {
      case 1: k_hash_finalize<T, 1><<<b, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_hkey_tmp, s->d_start, nl, y, s->d_perm, pos, s->d_hkey, build_stats(s));
              k_finalize_large<T, 1, true><<<std::min(b, 152 * 4), 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_hkey_tmp, s->d_start, nl, y, s->d_perm, pos, s->d_hkey, build_stats(s), nullptr); break;
      case 2: k_hash_finalize<T, 2><<<b, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_hkey_tmp, s->d_start, nl, y, s->d_perm, pos, s->d_hkey, build_stats(s));
              k_finalize_large<T, 2, true><<<std::min(b, 152 * 4), 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_hkey_tmp, s->d_start, nl, y, s->d_perm, pos, s->d_hkey, build_stats(s), nullptr); break;
      default: k_hash_finalize<T, 3><<<b, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_hkey_tmp, s->d_start, nl, y, s->d_perm, pos, s->d_hkey, build_stats(s));
              k_finalize_large<T, 3, true><<<std::min(b, 152 * 4), 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot, s->d_hkey_tmp, s->d_start, nl, y, s->d_perm, pos, s->d_hkey, build_stats(s), nullptr); break;
    }
    count_launch();
    count_launch();
    // the heads go into d_slot_of (free again after the scatter), their scan into hcellidx
    k_hash_heads<<<b, 256, 0, st>>>(s->d_cell_of_slot, s->d_hkey, s->d_start + nl, (int32_t)m,
                                    s->d_slot_of); count_launch();
    scan_counts(s->d_slot_of, (int32_t)m, s->d_hcellidx, s->d_hscan_state,
                scan_tile_count(m), s->d_err, st);
    k_hash_cells<<<b, 256, 0, st>>>(s->d_slot_of, s->d_hcellidx, s->d_hkey, s->d_start + nl,
                                    (int32_t)m, s->d_hcell); count_launch();
    k_hash_buckets<<<div_up((int64_t)nl + 1, 256), 256, 0, st>>>(s->d_start, s->d_hcellidx, nl,
                                                                 s->d_hbucket); count_launch();
  } else {
    cudaMemsetAsync(s->d_hbucket, 0, sizeof(int32_t) * ((int64_t)nl + 1), st);
  }
  s->n_binned = m;
  s->pc_valid = false;
  s->ovf_active = false;
  s->main_perm_valid = false;
  s->n_ovf = 0;
  s->updates_since_build = 0;
  return cuda_status(cudaGetLastError());
}

template int build_hash<float>(pn_search*, const float*, int64_t, const int32_t*, int64_t,
                               cudaStream_t);
template int build_hash<double>(pn_search*, const double*, int64_t, const int32_t*, int64_t,
                                cudaStream_t);

// ---------------------------------------------------------------- pieces of the batched build
// (pn_batch.cu bins the points of many clouds itself, then reuses these on the
// concatenated cell and slot arrays.)
void scan_counts(const int32_t* counts, int32_t n, int32_t* start, unsigned long long* state,
                 int32_t tiles, int32_t* err, cudaStream_t st, int32_t* stats) {
  cudaMemsetAsync(state, 0, sizeof(unsigned long long) * (tiles + 1), st);
  k_scan_cells<<<tiles, SCAN_THREADS, 0, st>>>(counts, n, start, state, tiles, 0, nullptr, err,
                                               nullptr, 0, stats); count_launch();
}

int32_t scan_tile_count(int64_t n) { return div_up(n, SCAN_TILE); }

// The scan's bounded look-back with a predecessor that never publishes: the tile counter
// starts at 1, so the one block launched takes tile 1 of 2 and waits for tile 0 until its
// iteration limit, then records PN_ERR_TIMEOUT.  Every access stays inside the private
// arrays (counts and start of 2 tiles, state of 2 tiles + the counter).
int selftest_bounded_wait(cudaStream_t st) {
  const int32_t n = 2 * SCAN_TILE;
  int32_t* counts = nullptr;
  int32_t* start = nullptr;
  int32_t* err = nullptr;
  unsigned long long* state = nullptr;
  cudaError_t e = cudaMalloc(&counts, sizeof(int32_t) * n);
  if (e == cudaSuccess) e = cudaMalloc(&start, sizeof(int32_t) * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&state, sizeof(unsigned long long) * 3);
  int32_t status = -1;
  if (e == cudaSuccess) {
    const unsigned long long first_tile = 1;
    cudaMemsetAsync(counts, 0, sizeof(int32_t) * n, st);
    cudaMemsetAsync(err, 0, sizeof(int32_t), st);
    cudaMemsetAsync(state, 0, sizeof(unsigned long long) * 3, st);
    e = cudaMemcpyAsync(state + 2, &first_tile, sizeof first_tile, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      k_scan_cells<<<1, SCAN_THREADS, 0, st>>>(counts, n, start, state, 2, 0, nullptr, err,
                                               nullptr, 0);
      count_launch();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&status, err, sizeof status, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  cudaFree(state);
  cudaFree(err);
  cudaFree(start);
  cudaFree(counts);
  return e == cudaSuccess ? status : cuda_status(e);
}

void scatter_slots(const int32_t* cell_of, const int32_t* slot_of, int32_t m,
                   const int32_t* start, int32_t* tmp_perm, int32_t* cell_of_slot,
                   cudaStream_t st) {
  if (m <= 0) return;
  k_scatter<<<div_up(m, 256), 256, 0, st>>>(cell_of, slot_of, nullptr, m, start, tmp_perm,
                                            cell_of_slot, nullptr); count_launch();
}

template <typename T>
void finalize_slots(int ndims, const int32_t* tmp_perm, const int32_t* cell_of_slot,
                    const int32_t* start, int32_t n_total, const T* y, int32_t m, int32_t* perm,
                    T* pos, cudaStream_t st) {
  const int blocks = div_up(m, 256);
  if (blocks == 0) return;
  switch (ndims) {
    case 1: k_finalize<T, 1><<<blocks, 256, 0, st>>>(tmp_perm, cell_of_slot, start, n_total, y, perm, pos, nullptr); break;
    case 2: k_finalize<T, 2><<<blocks, 256, 0, st>>>(tmp_perm, cell_of_slot, start, n_total, y, perm, pos, nullptr); break;
    default: k_finalize<T, 3><<<blocks, 256, 0, st>>>(tmp_perm, cell_of_slot, start, n_total, y, perm, pos, nullptr); break;
  }
  count_launch();
}
template void finalize_slots<float>(int, const int32_t*, const int32_t*, const int32_t*, int32_t,
                                    const float*, int32_t, int32_t*, float*, cudaStream_t);
template void finalize_slots<double>(int, const int32_t*, const int32_t*, const int32_t*, int32_t,
                                     const double*, int32_t, int32_t*, double*, cudaStream_t);

template <typename T, int D, bool PER>
static void launch_mark(pn_search* s, const T* y, cudaStream_t st) {
  const int blocks = std::max(1, std::min(div_up(s->n_binned, 256), 152 * 8));
  k_mark_movers<T, D, PER><<<blocks, 256, 0, st>>>(
      make_grid<T>(s), s->d_main_perm, s->d_cell_of_slot, s->d_start + s->n_total, y,
      s->d_perm, static_cast<T*>(s->d_pos), s->d_ovf_counts, s->d_ovf_n, s->d_ovf_list,
      s->d_ovf_cell, s->d_ovf_slot, s->d_err + 1, s->d_err, s->d_xkey, s->d_cell_of,
      s->d_slot_of, s->d_counts); count_launch();
}

template <typename T, int D>
static void launch_movers(pn_search* s, const T* y, cudaStream_t st) {
  const int32_t* gate = s->d_err + 2;
  k_scatter_movers<<<152 * 4, 256, 0, st>>>(s->d_ovf_n, s->d_ovf_list, s->d_ovf_cell,
                                             s->d_ovf_slot, s->d_ovf_start, s->d_tmp_perm,
                                             s->d_cell_of_slot, gate, s->d_err, s->n_total,
                                             slot_capacity(s)); count_launch();
  k_finalize_movers<T, D><<<152 * 4, 256, 0, st>>>(s->d_tmp_perm, s->d_cell_of_slot,
                                                   s->d_ovf_start, s->d_start + s->n_total,
                                                   s->n_total, y, s->d_perm,
                                                   static_cast<T*>(s->d_pos), gate, s->d_xkey);
  count_launch();
}

template <typename T>
int update_incremental(pn_search* s, const T* y, int64_t n_y, cudaStream_t st) {
  (void)n_y;
  if (!s->main_perm_valid) {
    cudaMemcpyAsync(s->d_main_perm, s->d_perm, sizeof(int32_t) * s->n_binned,
                    cudaMemcpyDeviceToDevice, st);
    s->main_perm_valid = true;
  }
  cudaMemsetAsync(s->d_ovf_counts, 0, sizeof(int32_t) * s->n_total, st);
  cudaMemsetAsync(s->d_ovf_n, 0, 2 * sizeof(int32_t), st);  // movers, largest overflow cell
  cudaMemsetAsync(build_stats(s), 0, 2 * sizeof(int32_t), st);
  cudaMemsetAsync(s->d_err + 1, 0, sizeof(int32_t), st);  // points outside the periodic box
  cudaMemsetAsync(s->d_err + ERR_DELTA, 0, sizeof(int32_t), st);
  cudaMemsetAsync(s->d_counts, 0, sizeof(int32_t) * s->n_total, st);  // the mark's histogram
  if (s->d_cell_delta) cudaMemsetAsync(s->d_cell_delta, 0, sizeof(float) * s->n_total, st);
  const bool per = s->periodic != 0;
  switch (s->ndims * 2 + (per ? 1 : 0)) {
    case 2: launch_mark<T, 1, false>(s, y, st); break;
    case 3: launch_mark<T, 1, true>(s, y, st); break;
    case 4: launch_mark<T, 2, false>(s, y, st); break;
    case 5: launch_mark<T, 2, true>(s, y, st); break;
    case 6: launch_mark<T, 3, false>(s, y, st); break;
    default: launch_mark<T, 3, true>(s, y, st); break;
  }
  int32_t* gate = s->d_err + 2;
  k_decide_update<<<1, 32, 0, st>>>(s->d_ovf_n, s->d_start + s->n_total, s->rebuild_fraction,
                                    gate); count_launch();
  // overflow path
  if (s->d_cell_delta != nullptr) {
    const int b = std::max(1, std::min(div_up(s->n_binned, 256), 152 * 8));
    const float* pos = static_cast<const float*>(s->d_pos);
    const int32_t* nmain = s->d_start + s->n_total;
    switch (s->ndims) {
      case 1: k_cell_delta<1><<<b, 256, 0, st>>>(pos, s->d_xkey, s->d_perm, s->d_cell_of_slot, nmain, s->n_total, s->d_cell_delta, gate, s->d_err); break;
      case 2: k_cell_delta<2><<<b, 256, 0, st>>>(pos, s->d_xkey, s->d_perm, s->d_cell_of_slot, nmain, s->n_total, s->d_cell_delta, gate, s->d_err); break;
      default: k_cell_delta<4><<<b, 256, 0, st>>>(pos, s->d_xkey, s->d_perm, s->d_cell_of_slot, nmain, s->n_total, s->d_cell_delta, gate, s->d_err); break;
    }
    count_launch();
  }
  scan_cells(s, s->d_ovf_counts, s->d_ovf_start, st, s->d_start + s->n_total, 0, gate,
             GATE_OVERFLOW, false);
  switch (s->ndims) {
    case 1: launch_movers<T, 1>(s, y, st); break;
    case 2: launch_movers<T, 2>(s, y, st); break;
    default: launch_movers<T, 3>(s, y, st); break;
  }
  // rebuild path (every point is binned: the incremental strategy has no eachindex_y); the
  // histogram is the mark kernel's
  const int32_t m = (int32_t)s->n_binned;
  scan_cells(s, s->d_counts, s->d_start, st, nullptr, s->cfg.max_points_per_cell, gate,
             GATE_REBUILD);
  k_scatter<<<div_up(m, 256), 256, 0, st>>>(s->d_cell_of, s->d_slot_of, nullptr, m, s->d_start,
                                            s->d_tmp_perm, s->d_cell_of_slot, gate, s->d_err,
                                            s->n_total, slot_capacity(s)); count_launch();
  launch_finalize<T>(s, y, m, st, gate);
  k_reset_overflow<<<152 * 4, 256, 0, st>>>(s->d_start, s->n_total, s->d_perm, s->d_main_perm,
                                            s->d_ovf_start, s->d_ovf_n, gate,
                                            s->d_err + ERR_DELTA); count_launch();
  s->ovf_active = true;
  s->pc_valid = false;
  refresh_pos32(s, st);
  // The mover count feeds the rebuild policy of the next update; it is read back lazily.
  cudaMemcpyAsync(s->h_ovf_n, s->d_ovf_n, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  cudaEventRecord(s->ev_ovf, st);
  s->ovf_pending = true;
  ++s->updates_since_build;
  return cuda_status(cudaGetLastError());
}

// The Float32 split of the cell-sorted coordinates: hi = fl32(x), lo = fl32(x - hi), lo2 =
// fl32(x - hi - lo) (each difference exact in Float64; lo2 has at most 5 significant bits,
// so x = hi + lo + lo2 exactly unless a part underflows); pos32lo / pos32lo2 null when not
// kept.  Vacated slots keep NaN.
template <int D>
__global__ void __launch_bounds__(256)
k_to_pos32(const double* __restrict__ pos, const int32_t* __restrict__ n_slots,
           int64_t n_max, float* __restrict__ pos32, float* __restrict__ pos32lo,
           float* __restrict__ pos32lo2) {
  const int64_t n = min((int64_t)*n_slots, n_max);
  constexpr int S = PS<D>::value;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    float h[4] = {0.0f, 0.0f, 0.0f, 0.0f}, l[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float l2[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double x = pos[k * S + d];
      h[d] = __double2float_rn(x);
      const double r = __dsub_rn(x, (double)h[d]);
      l[d] = __double2float_rn(r);
      l2[d] = __double2float_rn(__dsub_rn(r, (double)l[d]));
    }
#pragma unroll
    for (int d = 0; d < S; ++d) {
      pos32[k * S + d] = h[d];
      if (pos32lo != nullptr) pos32lo[k * S + d] = l[d];
      if (pos32lo2 != nullptr) pos32lo2[k * S + d] = l2[d];
    }
  }
}

// Kept for a mixed-precision search (hi and lo) and for a Float64 one (hi: the Float32
// traversal that finds its candidates, see Exact64 in pn_traverse.cuh).
void refresh_pos32(pn_search* s, cudaStream_t st) {
  if (s->d_pos32 == nullptr || s->n_binned == 0) return;
  const int32_t* n_slots = s->ovf_active ? s->d_ovf_start + s->n_total : s->d_start + s->n_total;
  const int64_t n_max = 2 * s->cap;
  const int b = std::max(1, std::min(div_up(n_max, 256), 152 * 8));
  const double* pos = static_cast<const double*>(s->d_pos);
  switch (s->ndims) {
    case 1: k_to_pos32<1><<<b, 256, 0, st>>>(pos, n_slots, n_max, s->d_pos32, s->d_pos32lo, nullptr); break;
    case 2: k_to_pos32<2><<<b, 256, 0, st>>>(pos, n_slots, n_max, s->d_pos32, s->d_pos32lo, nullptr); break;
    default: k_to_pos32<3><<<b, 256, 0, st>>>(pos, n_slots, n_max, s->d_pos32, s->d_pos32lo, s->d_pos32lo2); break;
  }
  count_launch();
}

template int update_incremental<float>(pn_search*, const float*, int64_t, cudaStream_t);
template int update_incremental<double>(pn_search*, const double*, int64_t, cudaStream_t);

template int build<float>(pn_search*, const float*, int64_t, const int32_t*, int64_t, cudaStream_t);
template int build<double>(pn_search*, const double*, int64_t, const int32_t*, int64_t, cudaStream_t);

// ---------------------------------------------------------------- cell_coords
template <typename T, int D>
__global__ void k_cell_coords(const GridDev<T> g, bool per, const T* __restrict__ x, int64_t n,
                              int64_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T xi[D];
#pragma unroll
  for (int k = 0; k < D; ++k) xi[k] = x[i * D + k];
  int64_t c[D];
  cell_coords_exact<T, D>(g, per, xi, c);
#pragma unroll
  for (int k = 0; k < D; ++k) out[i * D + k] = c[k];
}

template <typename T>
int cell_coords(pn_search* s, const T* x, int64_t n, int64_t* out, cudaStream_t st) {
  if (n <= 0) return PN_OK;
  const GridDev<T> g = make_grid<T>(s);
  const bool per = s->periodic != 0;
  const int b = div_up(n, 256);
  switch (s->ndims) {
    case 1: k_cell_coords<T, 1><<<b, 256, 0, st>>>(g, per, x, n, out); count_launch(); break;
    case 2: k_cell_coords<T, 2><<<b, 256, 0, st>>>(g, per, x, n, out); count_launch(); break;
    default: k_cell_coords<T, 3><<<b, 256, 0, st>>>(g, per, x, n, out); count_launch(); break;
  }
  return cuda_status(cudaGetLastError());
}

template int cell_coords<float>(pn_search*, const float*, int64_t, int64_t*, cudaStream_t);
template int cell_coords<double>(pn_search*, const double*, int64_t, int64_t*, cudaStream_t);

// ---------------------------------------------------------------- 64-bit scan
// Three-phase exclusive scan (tile sums, scan of the tile sums, apply) of int32 values
// into int64 offsets; out[n] = total.  Used for neighbour-list offsets.
constexpr int S64_THREADS = 256, S64_ITEMS = 8, S64_TILE = S64_THREADS * S64_ITEMS;

__device__ __forceinline__ long long block_excl_scan64(long long v, long long* s_warp,
                                                       long long& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < S64_THREADS / 32 ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < S64_THREADS / 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < S64_THREADS / 32) s_warp[lane] = w;
  }
  __syncthreads();
  total = s_warp[S64_THREADS / 32 - 1];
  const long long r = (warp > 0 ? s_warp[warp - 1] : 0) + incl - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(S64_THREADS)
k_s64_reduce(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ part) {
  __shared__ long long s_warp[S64_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * S64_TILE + (int64_t)threadIdx.x * S64_ITEMS;
  long long sum = 0;
  for (int i = 0; i < S64_ITEMS; ++i)
    if (base + i < n) sum += in[base + i];
  long long total;
  block_excl_scan64(sum, s_warp, total);
  if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(S64_THREADS)
k_s64_parts(int64_t* __restrict__ part, int64_t n_parts) {
  __shared__ long long s_warp[S64_THREADS / 32];
  long long carry = 0;
  for (int64_t b0 = 0; b0 < n_parts; b0 += S64_THREADS) {
    const int64_t i = b0 + threadIdx.x;
    const long long v = i < n_parts ? part[i] : 0;
    long long total;
    const long long ex = block_excl_scan64(v, s_warp, total);
    if (i < n_parts) part[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(S64_THREADS)
k_s64_apply(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ part,
            int64_t* __restrict__ out) {
  __shared__ long long s_warp[S64_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * S64_TILE + (int64_t)threadIdx.x * S64_ITEMS;
  int v[S64_ITEMS];
  long long sum = 0;
  for (int i = 0; i < S64_ITEMS; ++i) {
    v[i] = base + i < n ? in[base + i] : 0;
    sum += v[i];
  }
  long long total;
  long long run = part[blockIdx.x] + block_excl_scan64(sum, s_warp, total);
  for (int i = 0; i < S64_ITEMS; ++i) {
    if (base + i < n) {
      out[base + i] = run;
      run += v[i];
      if (base + i == n - 1) out[n] = run;
    }
  }
}

int scan64(pn_search* s, const int32_t* in, int64_t n, int64_t* out, cudaStream_t st) {
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(int64_t), st);
    return cuda_status(cudaGetLastError());
  }
  const int64_t parts = div_up(n, S64_TILE);
  if (parts > s->part_cap) {
    if (s->d_part) cudaFree(s->d_part);
    s->d_part = nullptr;
    if (cudaMalloc(&s->d_part, sizeof(int64_t) * parts) != cudaSuccess) return PN_ERR_OUT_OF_MEMORY;
    s->part_cap = parts;
  }
  k_s64_reduce<<<(unsigned)parts, S64_THREADS, 0, st>>>(in, n, s->d_part); count_launch();
  k_s64_parts<<<1, S64_THREADS, 0, st>>>(s->d_part, parts); count_launch();
  k_s64_apply<<<(unsigned)parts, S64_THREADS, 0, st>>>(in, n, s->d_part, out); count_launch();
  return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------- row sort
// One warp per row: rank every entry (entries of a row are distinct point indices) into
// the scratch, then copy the sorted row back.
__global__ void __launch_bounds__(256)
k_sort_rows(const int64_t* __restrict__ offsets, int64_t n_rows, int32_t* __restrict__ vals,
            int32_t* __restrict__ tmp, int64_t capacity) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n_rows || offsets[n_rows] > capacity) return;  // lists not written
  const int64_t s = offsets[row], e = offsets[row + 1];
  for (int64_t a = s + lane; a < e; a += 32) {
    const int32_t v = vals[a];
    int64_t rank = 0;
    for (int64_t b = s; b < e; ++b) rank += (vals[b] < v);
    tmp[s + rank] = v;
  }
  __syncwarp();
  for (int64_t a = s + lane; a < e; a += 32) vals[a] = tmp[a];
}

// `total` is the capacity of `vals`: rows are only sorted when they were written.
int sort_rows(pn_search* s, const int64_t* offsets, int64_t n_rows, int32_t* vals,
              int64_t total, cudaStream_t st) {
  if (n_rows == 0 || total == 0) return PN_OK;
  if (total > s->sort_tmp_cap) {
    if (s->d_sort_tmp) cudaFree(s->d_sort_tmp);
    s->d_sort_tmp = nullptr;
    if (cudaMalloc(&s->d_sort_tmp, sizeof(int32_t) * total) != cudaSuccess) return PN_ERR_OUT_OF_MEMORY;
    s->sort_tmp_cap = total;
  }
  k_sort_rows<<<div_up(n_rows * 32, 256), 256, 0, st>>>(offsets, n_rows, vals, s->d_sort_tmp,
                                                        total); count_launch();
  return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------- export
// counts[c] = points in cell c; points = every cell's points, ascending, cell by cell.
// With overflow lists active, a cell holds its main points that are still there (slots not
// vacated) followed by its overflow points, merged and sorted.
template <typename T, int D>
__global__ void k_export_counts(const int32_t* __restrict__ start, const int32_t* __restrict__ ovf_start,
                                const int32_t* __restrict__ perm, int32_t n_total,
                                int32_t* __restrict__ counts) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_total) return;
  int32_t n = 0;
  for (int32_t k = start[c]; k < start[c + 1]; ++k) n += perm[k] >= 0;
  if (ovf_start) n += ovf_start[c + 1] - ovf_start[c];
  counts[c] = n;
}

template <typename T, int D>
__global__ void k_export_points(const int32_t* __restrict__ start, const int32_t* __restrict__ perm,
                                const int32_t* __restrict__ ovf_start,
                                const int32_t* __restrict__ ovf_perm, const int64_t* __restrict__ out_start,
                                int32_t n_total, int32_t* __restrict__ points) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_total) return;
  int64_t o = out_start[c];
  const int64_t o0 = o;
  for (int32_t k = start[c]; k < start[c + 1]; ++k)
    if (perm[k] >= 0) points[o++] = perm[k];
  if (ovf_start)
    for (int32_t k = ovf_start[c]; k < ovf_start[c + 1]; ++k) points[o++] = ovf_perm[k];
  // ascending point index (a cell is stored sorted by coordinate); insertion sort
  for (int64_t a = o0 + 1; a < o; ++a) {
    const int32_t v = points[a];
    int64_t b = a - 1;
    while (b >= o0 && points[b] > v) {
      points[b + 1] = points[b];
      --b;
    }
    points[b + 1] = v;
  }
}

template <typename T, int D>
static int export_cells_t(pn_search* s, int32_t* counts, int32_t* points, cudaStream_t st) {
  const int b = div_up(s->n_total, 256);
  const int32_t* ovf = s->ovf_active ? s->d_ovf_start : nullptr;
  k_export_counts<T, D><<<b, 256, 0, st>>>(s->d_start, ovf, s->d_perm, s->n_total, counts); count_launch();
  int64_t* out_start = nullptr;
  if (cudaMallocAsync(&out_start, sizeof(int64_t) * (s->n_total + 1), st) != cudaSuccess)
    return PN_ERR_OUT_OF_MEMORY;
  int rc = scan64(s, counts, s->n_total, out_start, st);
  if (rc == PN_OK && points) {
    k_export_points<T, D><<<b, 256, 0, st>>>(s->d_start, s->d_perm, ovf, s->d_perm,
                                              out_start, s->n_total, points); count_launch();
  }
  cudaFreeAsync(out_start, st);
  return rc != PN_OK ? rc : cuda_status(cudaGetLastError());
}

// The reference's hash lists of a SpatialHashingCellList (either layout): every binned
// point's list from its stored coordinates, counts per list, then the points of each list
// ascending.
template <typename T, int D, bool PER>
__global__ void __launch_bounds__(256)
k_export_hash_count(const GridDev<T> g, const HashMod hm, const T* __restrict__ pos,
                    const int32_t* __restrict__ perm, const int32_t* __restrict__ n_slots,
                    int32_t* __restrict__ list_of_slot, int32_t* __restrict__ counts) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *n_slots) return;
  int32_t h = -1;
  if (perm[k] >= 0) {
    int32_t c[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) hash_cell_1d(g, PER, d, pos[k * PS<D>::value + d], c[d]);
    h = spatial_hash<D>(c, hm);
    atomicAdd(&counts[h], 1);
  }
  list_of_slot[k] = h;
}

__global__ void __launch_bounds__(256)
k_export_hash_scatter(const int32_t* __restrict__ list_of_slot, const int32_t* __restrict__ perm,
                      const int32_t* __restrict__ n_slots, unsigned long long* __restrict__ cursor,
                      int32_t* __restrict__ points) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *n_slots) return;
  const int32_t h = list_of_slot[k];
  if (h >= 0) points[atomicAdd(&cursor[h], 1ull)] = perm[k];
}

template <typename T, int D, bool PER>
static int export_hash_t(pn_search* s, int32_t* counts, int32_t* points, cudaStream_t st) {
  const int64_t nl = s->list_size;
  const int32_t* n_slots = s->d_start + s->n_total;
  const int64_t ns = s->n_binned;
  cudaMemsetAsync(counts, 0, sizeof(int32_t) * nl, st);
  const int b = div_up(std::max<int64_t>(ns, 1), 256);
  k_export_hash_count<T, D, PER><<<b, 256, 0, st>>>(make_grid<T>(s), hash_mod(nl),
                                                    static_cast<const T*>(s->d_pos), s->d_perm,
                                                    n_slots, s->d_cell_of, counts); count_launch();
  int64_t* out_start = nullptr;
  if (cudaMallocAsync(&out_start, sizeof(int64_t) * (nl + 1), st) != cudaSuccess)
    return PN_ERR_OUT_OF_MEMORY;
  int rc = scan64(s, counts, nl, out_start, st);
  if (rc == PN_OK && points) {
    k_export_hash_scatter<<<b, 256, 0, st>>>(s->d_cell_of, s->d_perm, n_slots,
                                             reinterpret_cast<unsigned long long*>(out_start),
                                             points); count_launch();
    rc = scan64(s, counts, nl, out_start, st);  // the cursors moved: the starts again
    if (rc == PN_OK) rc = sort_rows(s, out_start, nl, points, ns, st);
  }
  cudaFreeAsync(out_start, st);
  return rc != PN_OK ? rc : cuda_status(cudaGetLastError());
}

int export_hash_lists(pn_search* s, int32_t* counts, int32_t* points, cudaStream_t st) {
  const bool per = s->periodic != 0;
  const int key = (s->ndims - 1) * 2 + (per ? 1 : 0) + (s->dtype == PN_FLOAT64 ? 6 : 0);
  switch (key) {
    case 0: return export_hash_t<float, 1, false>(s, counts, points, st);
    case 1: return export_hash_t<float, 1, true>(s, counts, points, st);
    case 2: return export_hash_t<float, 2, false>(s, counts, points, st);
    case 3: return export_hash_t<float, 2, true>(s, counts, points, st);
    case 4: return export_hash_t<float, 3, false>(s, counts, points, st);
    case 5: return export_hash_t<float, 3, true>(s, counts, points, st);
    case 6: return export_hash_t<double, 1, false>(s, counts, points, st);
    case 7: return export_hash_t<double, 1, true>(s, counts, points, st);
    case 8: return export_hash_t<double, 2, false>(s, counts, points, st);
    case 9: return export_hash_t<double, 2, true>(s, counts, points, st);
    case 10: return export_hash_t<double, 3, false>(s, counts, points, st);
    default: return export_hash_t<double, 3, true>(s, counts, points, st);
  }
}

int export_cells(pn_search* s, int32_t* counts, int32_t* points, cudaStream_t st) {
  const int key = s->ndims + (s->dtype == PN_FLOAT64 ? 3 : 0);
  switch (key) {
    case 1: return export_cells_t<float, 1>(s, counts, points, st);
    case 2: return export_cells_t<float, 2>(s, counts, points, st);
    case 3: return export_cells_t<float, 3>(s, counts, points, st);
    case 4: return export_cells_t<double, 1>(s, counts, points, st);
    case 5: return export_cells_t<double, 2>(s, counts, points, st);
    default: return export_cells_t<double, 3>(s, counts, points, st);
  }
}

}  // namespace pn
