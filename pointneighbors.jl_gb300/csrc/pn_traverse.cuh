// pn_traverse.cuh -- neighbour traversal (foreach_point_neighbor) and its pair functions.
//
// Reference: neighborhood_search.jl:183-234 launches one thread per query point, which
// loops over the 3^d cells around its own cell (nhs_grid.jl:519-583) and gathers the
// neighbours' coordinates through the cell list's Int32 index columns.
//
// Here the candidates come from the cell-sorted coordinate copy: since cells are numbered
// column-major, the three cells (x-1, x, x+1) of one row of the stencil are one contiguous
// slot range, so a query walks 3^(d-1) contiguous ranges (each clipped to the query's reach,
// see TravArgs).  Query threads are taken in cell-sorted order (when x is y), so the lanes
// of a warp share their rows and most candidate loads are L1 hits.  Rows are visited in the
// reference's order (CartesianIndices over the 3^d cells, first dimension fastest), a row's
// candidates in slot order (inside a cell by first coordinate), so every sum is accumulated
// in a fixed, reproducible order.
//
// The distance test restates the reference bit for bit: pos_diff = xi - yj in T,
// d2 = ((pd1*pd1 + pd2*pd2) + pd3*pd3) without contraction, and with a periodic box,
// when d2 > r^2, pos_diff -= size .* round.(pos_diff ./ size) and d2 is recomputed
// (neighborhood_search.jl:428-436).  The correction is skipped when every |pos_diff_k| is
// below size_k/2: round() is then 0 and the correction is exactly the identity.
#pragma once

#include "pn_df.cuh"
#include "pn_internal.cuh"

namespace pn {

constexpr int TRAV_THREADS = 128;

template <typename T>
struct TravArgs {
  GridDev<T> g;
  const int32_t* start;         // [n_total + 1] main cell starts
  const int32_t* ovf_start;     // [n_total + 1] overflow cell starts (absolute slots) or null
  const int32_t* perm;          // slot -> point index (-1: slot vacated by an update)
  const int32_t* cell_of_slot;  // slot -> linear cell
  const T* pos;                 // cell-sorted coordinates, stride PS<D>
  const T* x;                   // query coordinates (list mode), stride D
  const int32_t* qlist;         // query point indices (list mode) or null = 0..n_q-1
  int64_t n_q;                  // list mode: number of queries
  int64_t n_x;                  // list mode: number of points in x
  T r2_lo, r2_hi;               // r^2 (1 -+ 32 eps): the FMA distance test decides outside
  const int32_t* outside;       // device flag: some binned point lies outside the periodic box
  int32_t* err;
  // bounds-checked builds: slots allocated (main, overflow and padding) and points a query
  // or a slot's permutation entry may name
  int64_t bc_slots, bc_points;
  // Row clipping: inside every cell the points are sorted by their first coordinate, so a
  // stencil row's three cells are one x-sorted run and a query only scans the part of it
  // within x +- sqrt(r^2 - dy^2 - dz^2) (dy, dz: distance to the row's band).  `unsorted`
  // (device flag, or null = sorted) is set while an incremental update keeps overflow lists
  // (positions refreshed in place): then the rows are clipped by `xkey` below, or not at all
  // where there is none; `clip_m` is a per-dimension margin that covers the rounding of the
  // cell edges, so the clipped run is always a superset of the neighbours.
  const int32_t* unsorted;
  T clip_m[3];
  // Float32 incremental searches with overflow lists (or null): the rows are clipped by the
  // sorted key xkey (each slot's x when its cell was last sorted) with the window widened by
  // *delta, the largest distance of a main slot's x from its key, so the clipped runs stay
  // supersets of the neighbours while the positions move in place; overflow runs are
  // clipped by their keys (their x: they are re-sorted at every update).
  const float* xkey;
  const float* delta;
  const float* cell_delta;  // per cell the largest |x - xkey| of its main slots
  // Precomputed neighbour lists (or null: the grid traversal).  Groups of 32 rows are stored
  // transposed in quads: row r's entries 4k..4k+3 are the int4 at
  // nb[nb_grp[r / 32] + 128 k + 4 (r % 32)], so a warp reads its rows' k-th quads in one
  // coalesced 512-byte load; nb_len[r] entries per row (nb_grp is a multiple of 4).
  const int32_t* nb;
  const int64_t* nb_grp;
  const int32_t* nb_len;
  const int32_t* nb_row_of;  // query point -> its row (lists built by slot), or null: row = point
  // pair cache: queries that could not be cached have a negative nb_len entry; the cached
  // walk skips them and a grid launch with the cache pointers cleared and nb_len set
  // traverses exactly those queries
  int32_t nb_fallback;
  // pair cache as hit masks: for query slot k and stencil row ri, the clipped run start
  // pc_b0[ri * pc_stride + k] and a 128-bit mask of its accepted candidates
  const int32_t* pc_b0;
  const ulonglong2* pc_mask;
  int64_t pc_stride;
  const int32_t* pc_ob0;                 // overflow runs (or null), see MaskParams
  const unsigned long long* pc_omask;
  const int32_t* pc_any_fallback;  // device flag: some query was marked for the fallback
  // SpatialHashingCellList (or null): list h's cells are the entries hash_cell[hash_list[h]
  // .. hash_list[h + 1]), each (x, y, z, first slot), a cell's run ending at the next
  // entry's first slot; hash_key[slot] is the slot's own cell
  const int32_t* hash_list;
  const int4* hash_cell;
  const int4* hash_key;
  HashMod hash_mod;
};

template <typename T, int D>
struct Query {
  int32_t i;   // point index in x
  int32_t q;   // position in the query list (CSR row)
  int32_t k;   // cell-sorted slot (sorted mode) or -1
  T x[D];
};

template <typename T, int D>
__device__ __forceinline__ void load_pos(const T* __restrict__ pos, int64_t k, T* v);

template <>
__device__ __forceinline__ void load_pos<float, 3>(const float* __restrict__ pos, int64_t k, float* v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(pos) + k);
  v[0] = a.x; v[1] = a.y; v[2] = a.z;
}
template <>
__device__ __forceinline__ void load_pos<float, 2>(const float* __restrict__ pos, int64_t k, float* v) {
  const float2 a = __ldg(reinterpret_cast<const float2*>(pos) + k);
  v[0] = a.x; v[1] = a.y;
}
template <>
__device__ __forceinline__ void load_pos<float, 1>(const float* __restrict__ pos, int64_t k, float* v) {
  v[0] = __ldg(pos + k);
}
template <>
__device__ __forceinline__ void load_pos<double, 3>(const double* __restrict__ pos, int64_t k, double* v) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(pos) + 2 * k);
  const double2 b = __ldg(reinterpret_cast<const double2*>(pos) + 2 * k + 1);
  v[0] = a.x; v[1] = a.y; v[2] = b.x;
}
template <>
__device__ __forceinline__ void load_pos<double, 2>(const double* __restrict__ pos, int64_t k, double* v) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(pos) + k);
  v[0] = a.x; v[1] = a.y;
}
template <>
__device__ __forceinline__ void load_pos<double, 1>(const double* __restrict__ pos, int64_t k, double* v) {
  v[0] = __ldg(pos + k);
}

// A candidate's coordinates and, in 3D, the stored 4th component (0 for the plain
// coordinate copy, p/rho^2 for the WCSPH state).
template <typename T, int D>
__device__ __forceinline__ T load_cand(const T* __restrict__ pos, int64_t k, T* v) {
  if constexpr (D == 3) {
    if constexpr (sizeof(T) == 4) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(pos) + k);
      v[0] = a.x; v[1] = a.y; v[2] = a.z;
      return a.w;
    } else {
      const double2 a = __ldg(reinterpret_cast<const double2*>(pos) + 2 * k);
      const double2 b = __ldg(reinterpret_cast<const double2*>(pos) + 2 * k + 1);
      v[0] = a.x; v[1] = a.y; v[2] = b.x;
      return b.y;
    }
  } else {
    load_pos<T, D>(pos, k, v);
    return (T)0;
  }
}

// 4-component per-slot state (WCSPH): float4 / two double2.
template <typename T>
struct V4 { T x, y, z, w; };

__device__ __forceinline__ V4<float> load4(const float* __restrict__ p, int64_t k) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p) + k);
  return {a.x, a.y, a.z, a.w};
}
__device__ __forceinline__ V4<double> load4(const double* __restrict__ p, int64_t k) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p) + 2 * k);
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 2 * k + 1);
  return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void store4(float* p, int64_t k, V4<float> v) {
  reinterpret_cast<float4*>(p)[k] = make_float4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ void store4(double* p, int64_t k, V4<double> v) {
  reinterpret_cast<double2*>(p)[2 * k] = make_double2(v.x, v.y);
  reinterpret_cast<double2*>(p)[2 * k + 1] = make_double2(v.z, v.w);
}

// Packed FP32 pairs (Blackwell f32x2 arithmetic, round to nearest like the scalar forms).
__device__ __forceinline__ uint64_t pack_f32x2(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack_f32x2(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t sub_f32x2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t mul_f32x2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t fma_f32x2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// Candidate groups: an inline pair function that needs only d^2 (the WCSPH density) takes
// the candidates of a stencil run GROUP at a time, with their exact d^2 (the accepted ones
// are those with d^2 <= r^2), and it accumulates its contribution over the whole group
// without a branch, so the lanes of a warp stay converged while their runs differ in
// length.
constexpr int GROUP = 4;

template <class F, class = void>
struct has_group { static constexpr bool value = false; };
template <class F>
struct has_group<F, decltype((void)F::kGroup)> { static constexpr bool value = F::kGroup; };

// Pair-function math (only the sums are compared with the FP64 oracle, within tolerance):
// FP32 uses the approximate hardware square root and divide; FP64 stays IEEE.
__device__ __forceinline__ float fsqrt(float a) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}
__device__ __forceinline__ double fsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }

// ================================================================== pair functions
// A functor provides Params, Acc, init(acc, p, query), pair(acc, p, query, slot, pd, d2,
// aux), finish(acc, p, query), fail(p, query) (a rejected query: write the empty result
// where later passes depend on it) and vacant(p, slot) (a slot vacated by an incremental
// update); kCountOnly functors take count(acc, n) for n accepted neighbours at once.
// `slot` indexes the cell-sorted arrays.

// by_row: 0 = indexed by point, 1 = by query row, 2 = by slot (cell-sorted queries)
template <typename T> struct CountParams { int32_t* counts; int32_t by_row; };
template <typename T> struct IndexSumParams { int64_t* sums; const int32_t* perm; };
template <typename T> struct EmitParams {
  const int64_t* offsets; int32_t* nbrs; const int32_t* perm; int64_t capacity; int64_t n_rows;
};
template <typename T> struct NBodyParams { const T* masses; const int32_t* perm; T G; T sqrt_eps; T* accel; };
// cutoff2 = cutoff^2: the truncation 0 < d < cutoff is decided as 0 < d^2 < cutoff^2, the
// same decision as a correctly rounded square root gives, without depending on the
// approximate root the pair arithmetic uses
template <typename T> struct PotentialParams {
  const T* masses; const int32_t* perm; T cutoff, inv_cutoff; T* energy; T cutoff2;
};

template <typename T, int D>
struct FCount {
  static constexpr bool kCountOnly = true;
  static constexpr bool kInline = false;
  using Params = CountParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  struct Acc { int32_t n; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) { a.n = 0; }
  static __device__ __forceinline__ void pair(Acc& a, const Params&, const Query<T, D>&, int32_t,
                                              const T*, T, T) { ++a.n; }
  static __device__ __forceinline__ void count(Acc& a, int n) { a.n += n; }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    p.counts[p.by_row == 2 ? q.k : (p.by_row ? q.q : q.i)] = a.n;
  }
  static __device__ __forceinline__ void fail(const Params& p, const Query<T, D>& q) {
    if (p.by_row == 1) p.counts[q.q] = 0;
  }
};

template <typename T, int D>
struct FIndexSum {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = IndexSumParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { int64_t s; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) { a.s = 0; }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T*, T, T) { a.s += (int64_t)__ldg(&p.perm[js]) + 1; }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    p.sums[q.i] = a.s;
  }
};

template <typename T, int D>
struct FEmit {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = EmitParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  struct Acc { int64_t o, end; };
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    a.o = p.offsets[q.q];
    a.end = p.offsets[q.q + 1];
    if (p.offsets[p.n_rows] > p.capacity) a.end = a.o;  // does not fit: write nothing
  }
  // The count pass fixed the row length; the bound check keeps a row inside its slot range
  // even if y changed in between (the reference would read a different neighbour set).
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T*, T, T) {
    if (a.o < a.end) p.nbrs[a.o++] = __ldg(&p.perm[js]);
  }
  static __device__ __forceinline__ void finish(Acc&, const Params&, const Query<T, D>&) {}
};

// The precomputed search's list build: every accepted candidate slot, in traversal order
// (ascending slots), into the query row's transposed list, a quad (int4) at a time.
// With `len`, the lists have a fixed capacity `cap` per row (groups of 32 rows at grp[g] =
// 32 cap g) and the emitting pass also writes the row lengths, flagging rows longer than
// the capacity (the reference's "cell list is full"); without, the rows were sized by a
// counting pass.
template <typename T> struct EmitListParams {
  int32_t* nb; const int64_t* grp; int32_t by_slot;
  int32_t cap;    // entries a row has room for (a multiple of 4), with `len`
  int32_t limit;  // max_neighbors: a longer row is an error ...
  int32_t* len; int32_t* err;
  int32_t fallback;  // ... or, with fallback, gets length -1 (walked through the stencil)
};

template <typename T, int D>
struct FEmitList {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = true;  // a store per accepted candidate: no compaction
  using Params = EmitListParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { int64_t o; int32_t n; int4 quad; };
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    const int32_t r = p.by_slot ? q.k : q.q;
    a.o = p.grp[r >> 5] / 4 + (r & 31);  // int4 index of the row's first quad
    a.n = 0;
    a.quad = make_int4(-1, -1, -1, -1);
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T*, T, T) {
    const int e = a.n & 3;
    a.quad.x = e == 0 ? js : a.quad.x;
    a.quad.y = e == 1 ? js : a.quad.y;
    a.quad.z = e == 2 ? js : a.quad.z;
    a.quad.w = e == 3 ? js : a.quad.w;
    ++a.n;
    if (e == 3) {
      if (p.len == nullptr || a.n <= p.cap) reinterpret_cast<int4*>(p.nb)[a.o] = a.quad;
      a.o += 32;
    }
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    if ((a.n & 3) && (p.len == nullptr || a.n <= p.cap))
      reinterpret_cast<int4*>(p.nb)[a.o] = a.quad;  // the last, partial quad
    if (p.len == nullptr) return;
    const int32_t r = p.by_slot ? q.k : q.q;
    p.len[r] = a.n > p.limit && p.fallback ? -1 : min(a.n, p.cap);
    if (a.n > p.limit && !p.fallback) set_error(p.err, PN_ERR_CELL_FULL);
  }
};

// A pair function that also stores the accepted candidates into the pair cache: both see
// the same accepted candidates in the same order.
// The pair cache: a pair function that also records, per stencil row of the query, the
// start of the row's clipped run and a bit for every accepted candidate of it (the run must
// be at most 128 slots).  traverse_query announces every row (row_begin) when the rows are
// clipped, contiguous runs; otherwise (periodic wrap, overflow lists) the query is marked
// for the stencil fallback (no_rows).
struct MaskParams {
  int32_t* b0;
  ulonglong2* mask;
  int64_t stride;
  int32_t* any_fallback;
  int32_t* err;
  // overflow lists in use (or null): per row the start of the clipped overflow run (-1: no
  // neighbour in it) and a 64-bit mask of its neighbours; written only when some point is
  // in an overflow list (*ovf_end > *main_end), which the cache's walk checks the same way
  int32_t* ob0;
  unsigned long long* omask;
  const int32_t* ovf_end;
  const int32_t* main_end;
};
template <class PF>
struct MaskPairParams {
  PF f;
  MaskParams m;
};

// Double-float sums of the Float64 WCSPH sweeps (the DF64 wrapper): the constants, the
// three-part Float32 split of the cell-sorted coordinates and the state the force reads.
struct DFConst {
  df inv_h, h, dw_coef, eps_h2, m_alpha_c0_h, m_mass, r_min2;
  df r2_lo, r2_hi;  // r^2 (1 -+ 1e-12): outside, the double-float d^2 decides
  // below this Float32 d^2 of the traversal a candidate is certainly a neighbour: the
  // traversal's distance is within rs - r of the exact one (rs: its widened radius), so
  // d_32 < 2r - rs means d < r
  float r_in2;
};
struct DF64Geom {
  const float* xa;  // x = xa + xb + xc exactly, cell-sorted, PS<D> floats per slot
  const float* xb;
  const float* xc;
  float4* sdf;      // per slot (p/rho^2, rho), (vx, vy), (vz, -) as double-float pairs
  DFConst k;
};
struct NoDF {};
template <class F, class = void>
struct df_acc { using type = NoDF; };
template <class F>
struct df_acc<F, std::void_t<typename F::AccDF>> { using type = typename F::AccDF; };

template <class F, class = void>
struct has_row_hook { static constexpr bool value = false; };
template <class F>
struct has_row_hook<F, decltype((void)F::kRowHook)> { static constexpr bool value = F::kRowHook; };

template <typename T, int D, class F>
struct WithMask {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = F::kInline;
  static constexpr bool kRowHook = true;
  using Params = MaskPairParams<typename F::Params>;  // the same type for every D
  // lo, hi: the row's main run from b0; om: its overflow run from ob0 (ovf: the row's
  // candidates now come from the overflow run); ovf_any: the overflow masks are written.
  // FA: F's accumulator (F::Acc, or F::AccDF for the double-float sums of DF64).
  // kShift: F can take the main runs in groups (the Float32 3D density).  For a row that
  // comes in groups, (hi, lo) is a 128-bit shift register: each group's hit bits enter at
  // the top, and the row's flush shifts the register down by `sh` = 128 - GROUP x (the
  // row's groups), which puts candidate b0 + t at bit t as record() does (sh = 0 for a row
  // recorded one candidate at a time).
  static constexpr bool kShift = has_group<F>::value && D == 3 && sizeof(T) == 4;
  template <class FA>
  struct AccT {
    FA f;
    int32_t ri, b0, ob0, sh;
    uint64_t lo, hi, om;
    bool fb, ovf, ovf_any;
  };
  using Acc = AccT<typename F::Acc>;
  using AccDF = AccT<typename df_acc<F>::type>;
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) { F::vacant(p.f, k); }
  static __device__ __forceinline__ void fail(const Params& p, const Query<T, D>& q) { F::fail(p.f, q); }
  template <class A>
  static __device__ __forceinline__ void init_mask(A& a, const Params& p) {
    a.ri = -1;
    a.b0 = a.ob0 = a.sh = 0;
    a.lo = a.hi = a.om = 0;
    a.fb = a.ovf = false;
    a.ovf_any = p.m.ob0 != nullptr && __ldg(p.m.ovf_end) > __ldg(p.m.main_end);
  }
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    F::init(a.f, p.f, q);
    init_mask(a, p);
  }
  template <class A>
  static __device__ __forceinline__ void flush(A& a, const Params& p, const Query<T, D>& q) {
    if (a.ri < 0) return;
    if constexpr (kShift) {
      // align the shift register (sh < 0: more than 128 slots, the query is marked for
      // the fallback and its masks are not read)
      const int sh = a.sh;
      if (sh >= 64) {
        a.lo = sh >= 128 ? 0ull : a.hi >> (sh - 64);
        a.hi = 0ull;
      } else if (sh > 0) {
        a.lo = (a.lo >> sh) | (a.hi << (64 - sh));
        a.hi >>= sh;
      }
    }
    const int64_t o =
        (int64_t)a.ri * p.m.stride + PN_IDX(p.m.err, BC_PAIR_CACHE, q.k, p.m.stride);
    p.m.b0[o] = a.b0;
    p.m.mask[o] = make_ulonglong2(a.lo, a.hi);
    if (a.ovf_any) {
      p.m.ob0[o] = a.om != 0 ? a.ob0 : -1;
      if (a.om != 0) p.m.omask[o] = a.om;
    }
  }
  // grouped: the run comes in groups (the traversal calls F directly); a wrapper that
  // decides the candidates itself (mixed precision, Float64) records them one by one
  template <class A>
  static __device__ __forceinline__ void row_begin(A& a, const Params& p, const Query<T, D>& q,
                                                   int ri, int32_t b0, int32_t e0,
                                                   bool grouped = kShift) {
    flush(a, p, q);
    a.ri = ri;
    a.b0 = b0;
    a.lo = a.hi = a.om = 0;
    a.ovf = false;
    if (e0 - b0 > 128) a.fb = true;
    if constexpr (kShift) a.sh = grouped ? 128 - GROUP * ((max(e0 - b0, 0) + GROUP - 1) / GROUP) : 0;
  }
  // the row's overflow run [ob0, oe0) follows its main run
  template <class A>
  static __device__ __forceinline__ void ovf_begin(A& a, int32_t ob0, int32_t oe0) {
    a.ovf = true;
    a.ob0 = ob0;
    if (oe0 > ob0 && (!a.ovf_any || oe0 - ob0 > 64)) a.fb = true;
  }
  template <class A>
  static __device__ __forceinline__ void no_rows(A& a) { a.fb = true; }
  // the accepted candidate js: its bit in the row's mask
  template <class A>
  static __device__ __forceinline__ void record(A& a, int32_t js) {
    if (a.ovf) {
      const uint32_t off = (uint32_t)(js - a.ob0);
      if (off < 64) a.om |= 1ull << off;
      return;
    }
    const uint32_t off = (uint32_t)(js - a.b0);
    if (off < 64) a.lo |= 1ull << off;
    else if (off < 128) a.hi |= 1ull << (off - 64);
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>& q,
                                              int32_t js, const T* pd, T d2, T aux) {
    F::pair(a.f, p.f, q, js, pd, d2, aux);
    record(a, js);
  }
  // double-float sums (DF64): F's, and the same bits recorded
  static __device__ __forceinline__ void init_df(AccDF& a, const Params& p,
                                                 const Query<T, D>& q, const DF64Geom& d) {
    F::init_df(a.f, p.f, q, d);
    init_mask(a, p);
  }
  static __device__ __forceinline__ void pair_df(AccDF& a, const Params& p, int32_t js,
                                                 const df* pd, df d2, const DF64Geom& d) {
    F::pair_df(a.f, p.f, js, pd, d2, d);
    record(a, js);
  }
  static __device__ __forceinline__ void finish_df(AccDF& a, const Params& p,
                                                   const Query<T, D>& q, const DF64Geom& d) {
    F::finish_df(a.f, p.f, q, d);
    end_query(a, p, q);
  }
  // a group of GROUP candidates from slot js0 (a multiple of GROUP past the row's start);
  // the accepted ones are those with d2[u] <= r2
  static constexpr bool kGroup = has_group<F>::value;
  static __device__ __forceinline__ void group(Acc& a, const Params& p, const Query<T, D>& q,
                                               int32_t js0, const float* d2, float r2) {
    F::group(a.f, p.f, q, js0, d2, r2);
    uint32_t hits = 0u;
#pragma unroll
    for (int u = 0; u < GROUP; ++u) hits |= d2[u] <= r2 ? 1u << u : 0u;
    // main runs only (overflow runs: pair()), group by group from b0: into the top of the
    // shift register
    static_assert(kShift, "groups are taken only by the Float32 3D density");
    a.lo = (a.lo >> GROUP) | (a.hi << (64 - GROUP));
    a.hi = (a.hi >> GROUP) | ((uint64_t)hits << (64 - GROUP));
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    F::finish(a.f, p.f, q);
    end_query(a, p, q);
  }
  template <class A>
  static __device__ __forceinline__ void end_query(A& a, const Params& p, const Query<T, D>& q) {
    flush(a, p, q);
    if (a.fb) {
      p.m.b0[PN_IDX(p.m.err, BC_PAIR_CACHE, q.k, p.m.stride)] = -1;  // row 0's entry marks
                                                                      // the query for the
                                                                      // stencil fallback
      if (*(volatile int32_t*)p.m.any_fallback == 0) atomicExch(p.m.any_fallback, 1);
    }
  }
};

// benchmarks/n_body.jl:41-56
template <typename T, int D>
struct FNBody {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = NBodyParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T a[D]; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) {
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] = (T)0;
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T* pd, T d2, T) {
    const T r = fsqrt(d2);
    if (r < p.sqrt_eps) return;
    const T s = fdiv(-p.G * __ldg(&p.masses[__ldg(&p.perm[js])]), r * r * r);
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] += s * pd[k];
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
#pragma unroll
    for (int k = 0; k < D; ++k) p.accel[(int64_t)q.i * D + k] = a.a[k];
  }
};

// e_i = sum_j m_i m_j (1/d - 1/R), 0 < d < R
template <typename T, int D>
struct FPotential {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = PotentialParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T e; T mi; };
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    a.e = (T)0;
    a.mi = p.masses[q.i];
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T*, T d2, T) {
    if (d2 > (T)0 && d2 < p.cutoff2)
      a.e += __ldg(&p.masses[__ldg(&p.perm[js])]) * (fdiv((T)1, fsqrt(d2)) - p.inv_cutoff);
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    p.energy[q.i] = a.mi * a.e;
  }
};

template <typename T>
__device__ __forceinline__ T ipow(T x, int n) {
  T r = (T)1;
  while (n > 0) {
    if (n & 1) r *= x;
    x *= x;
    n >>= 1;
  }
  return r;
}

// Weakly compressible SPH constants shared by the density and force functors.
template <typename T>
struct SphConst {
  T mass, h, inv_h, sigma, dw_coef;  // W = sigma t^4 (2q+1); grad W = dw_coef t^3 pd
  T c0, rho0, inv_rho0, eos_b, gamma; int32_t gamma_int;
  T alpha, eps_h2, r_min2;
};

template <typename T>
__device__ __forceinline__ T sph_pressure(const SphConst<T>& c, T rho) {
  const T x = rho * c.inv_rho0;
  const T xp = c.gamma_int > 0 ? ipow(x, c.gamma_int) : pow(x, c.gamma);
  return c.eos_b * (xp - (T)1);
}

template <typename T>
struct DensityParams {
  SphConst<T> c;
  T* density; T* pressure;          // original order
  const T* velocity;                // original order (for the sorted state)
  T* pa; T* pb;                     // sorted state (sorted mode), or null
};

template <typename T>
struct ForceParams {
  SphConst<T> c;
  const T* pa; const T* pb;  // sorted state: (x, p/rho^2), (v, rho)
  T* accel;                  // original order
};

template <typename T, int D>
struct FDensity {
  static constexpr bool kCountOnly = false;
  // inline: the kernel value is cheap, so it is evaluated on the candidate already in
  // registers instead of re-loading accepted candidates later
  static constexpr bool kInline = true;
  using Params = DensityParams<T>;
  // A slot vacated by an incremental update keeps NaN coordinates in the state too, so
  // that a force sweep reading its candidates from the state never accepts it.
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) {
    if (p.pa != nullptr) store4(p.pa, k, V4<T>{(T)NAN, (T)NAN, (T)NAN, (T)0});
  }
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T w; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) { a.w = (T)0; }
  // Every operation explicitly rounded (or an explicit fma), so that group()'s packed form
  // gives the same bits: a density does not depend on whether its pairs were found by the
  // stencil or walked from the pair cache.
  static __device__ __forceinline__ T kernel(const Params& p, T d2) {
    const T q = xmul(fsqrt(d2), p.c.inv_h);
    const T t = fmax(fma(q, (T)-0.5, (T)1), (T)0);  // zero beyond the support 2h
    const T t2 = xmul(t, t);
    return xmul(xmul(t2, t2), fma(q, (T)2, (T)1));
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t,
                                              const T*, T d2, T) {
    a.w = xadd(a.w, kernel(p, d2));
  }
  // Float32 groups: the kernel of GROUP candidates two per packed instruction, then added in
  // candidate order, a rejected candidate adding an exact zero: pair()'s sum bit for bit.
  static constexpr bool kGroup = sizeof(T) == 4;
  static __device__ __forceinline__ void group(Acc& a, const Params& p, const Query<T, D>&,
                                               int32_t, const float* d2, float r2) {
    const uint64_t inv_h = pack_f32x2(p.c.inv_h, p.c.inv_h);
    const uint64_t m_half = pack_f32x2(-0.5f, -0.5f), one = pack_f32x2(1.0f, 1.0f);
    const uint64_t two = pack_f32x2(2.0f, 2.0f);
#pragma unroll
    for (int u = 0; u < GROUP; u += 2) {
      const uint64_t q = mul_f32x2(pack_f32x2(fsqrt(d2[u]), fsqrt(d2[u + 1])), inv_h);
      float t0, t1;
      unpack_f32x2(fma_f32x2(q, m_half, one), t0, t1);
      const uint64_t t = pack_f32x2(fmaxf(t0, 0.0f), fmaxf(t1, 0.0f));
      const uint64_t t2 = mul_f32x2(t, t);
      float w0, w1;
      unpack_f32x2(mul_f32x2(mul_f32x2(t2, t2), fma_f32x2(q, two, one)), w0, w1);
      a.w = xadd(a.w, d2[u] <= r2 ? (T)w0 : (T)0);  // false for NaN and the tail's +inf
      a.w = xadd(a.w, d2[u + 1] <= r2 ? (T)w1 : (T)0);
    }
  }

  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    const T rho = p.c.mass * p.c.sigma * a.w;
    const T pr = sph_pressure(p.c, rho);
    p.density[q.i] = rho;
    p.pressure[q.i] = pr;
    if (p.pa != nullptr && q.k >= 0) {
      V4<T> va{(T)0, (T)0, (T)0, pr / (rho * rho)};
      V4<T> vb{(T)0, (T)0, (T)0, rho};
      T* xa = &va.x;
      T* xb = &vb.x;
#pragma unroll
      for (int k = 0; k < D; ++k) {
        xa[k] = q.x[k];
        xb[k] = p.velocity[(int64_t)q.i * D + k];
      }
      store4(p.pa, q.k, va);
      store4(p.pb, q.k, vb);
    }
  }

  // Double-float sum (DF64): the kernel of the Float64 form in double-float arithmetic, the
  // sum taken in candidate order; finish as the Float64 sum, and the double-float state for
  // the force sweep.
  struct AccDF { df w; };
  static __device__ __forceinline__ void init_df(AccDF& a, const Params&, const Query<T, D>&,
                                                 const DF64Geom&) {
    a.w = df_make(0.0f);
  }
  static __device__ __forceinline__ void pair_df(AccDF& a, const Params&, int32_t, const df*,
                                                 df d2, const DF64Geom& d) {
    const df q = df_mul(df_sqrt(d2), d.k.inv_h);
    const df t = df_add_f(df_make(__fmul_rn(-0.5f, q.hi), __fmul_rn(-0.5f, q.lo)), 1.0f);
    if (!(t.hi > 0.0f)) return;  // beyond the support 2h: the Float64 form adds a zero
    const df t2 = df_sqr(t);
    const df u = df_add_f(df_make(__fmul_rn(2.0f, q.hi), __fmul_rn(2.0f, q.lo)), 1.0f);
    a.w = df_add_pos(a.w, df_mul(df_sqr(t2), u));
  }
  static __device__ __forceinline__ void finish_df(AccDF& a, const Params& p, const Query<T, D>& q,
                                                   const DF64Geom& d) {
    Acc t;
    t.w = (T)df_to(a.w);
    finish(t, p, q);
    if (d.sdf != nullptr && q.k >= 0) {
      const T rho = p.density[q.i], pr = p.pressure[q.i];
      const df P = df_from((double)(pr / (rho * rho))), R = df_from((double)rho);
      df v[3] = {df_make(0.0f), df_make(0.0f), df_make(0.0f)};
#pragma unroll
      for (int k = 0; k < D; ++k) v[k] = df_from((double)p.velocity[(int64_t)q.i * D + k]);
      d.sdf[3 * (int64_t)q.k] = make_float4(P.hi, P.lo, R.hi, R.lo);
      d.sdf[3 * (int64_t)q.k + 1] = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
      d.sdf[3 * (int64_t)q.k + 2] = make_float4(v[2].hi, v[2].lo, 0.0f, 0.0f);
    }
  }
};

template <typename T, int D>
struct FForce {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = ForceParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T a[D]; T Pi, rhoi; T vi[D]; };
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    const V4<T> sa = load4(p.pa, q.k);
    const V4<T> sb = load4(p.pb, q.k);
    const T vb[3] = {sb.x, sb.y, sb.z};
    a.Pi = sa.w;
    a.rhoi = sb.w;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      a.a[k] = (T)0;
      a.vi[k] = vb[k];
    }
  }
  // In 3D the traversal reads the candidates from the state (x, y, z, p/rho^2), and `aux`
  // is the candidate's p/rho^2; otherwise it is loaded here.  The neighbour's (v, rho) is
  // loaded before the r_min test, so that its gather is in flight together with the
  // coordinates' instead of after them.
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T* pd, T d2, T aux) {
    const V4<T> sb = load4(p.pb, js);
    if (d2 < p.c.r_min2) return;
    const T Pj = D == 3 ? aux : load4(p.pa, js).w;
    const T vj[3] = {sb.x, sb.y, sb.z};
    const T q = fsqrt(d2) * p.c.inv_h;
    const T t = fmax((T)1 - (T)0.5 * q, (T)0);  // zero beyond the support 2h
    const T gw = p.c.dw_coef * t * t * t;       // grad W = gw * pd
    T vr = (T)0;
#pragma unroll
    for (int k = 0; k < D; ++k) vr += (a.vi[k] - vj[k]) * pd[k];
    // Monaghan: Pi = -alpha c0 mu / rho_mean, mu = h v.x / (d^2 + eps h^2), for approaching
    // pairs (v.x < 0), else 0 -- one quotient: -alpha c0 h v.x / ((d^2 + eps h^2) rho_mean)
    const T visc = vr < (T)0 ? fdiv(-p.c.alpha * p.c.c0 * p.c.h * vr,
                                    (d2 + p.c.eps_h2) * ((T)0.5 * (a.rhoi + sb.w)))
                             : (T)0;
    const T s = -p.c.mass * (a.Pi + Pj + visc) * gw;
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] += s * pd[k];
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
#pragma unroll
    for (int k = 0; k < D; ++k) p.accel[(int64_t)q.i * D + k] = a.a[k];
  }

  // Double-float sum (DF64): the Float64 form's arithmetic in double-float, the neighbours'
  // state (p/rho^2, rho, v) from the density sweep's double-float copy.
  struct AccDF { df a[3], Pi, rhoi, vi[3]; };
  static __device__ __forceinline__ void init_df(AccDF& a, const Params&, const Query<T, D>& q,
                                                 const DF64Geom& d) {
    const float4 s0 = d.sdf[3 * (int64_t)q.k], s1 = d.sdf[3 * (int64_t)q.k + 1],
                 s2 = d.sdf[3 * (int64_t)q.k + 2];
    a.Pi = df_make(s0.x, s0.y);
    a.rhoi = df_make(s0.z, s0.w);
    a.vi[0] = df_make(s1.x, s1.y);
    a.vi[1] = df_make(s1.z, s1.w);
    a.vi[2] = df_make(s2.x, s2.y);
#pragma unroll
    for (int k = 0; k < 3; ++k) a.a[k] = df_make(0.0f);
  }
  static __device__ __forceinline__ void pair_df(AccDF& a, const Params&, int32_t js,
                                                 const df* pd, df d2, const DF64Geom& d) {
    if (df_lt(d2, d.k.r_min2)) return;
    const float4 s0 = __ldg(&d.sdf[3 * (int64_t)js]), s1 = __ldg(&d.sdf[3 * (int64_t)js + 1]),
                 s2 = __ldg(&d.sdf[3 * (int64_t)js + 2]);
    const df vj[3] = {df_make(s1.x, s1.y), df_make(s1.z, s1.w), df_make(s2.x, s2.y)};
    const df q = df_mul(df_sqrt(d2), d.k.inv_h);
    const df t = df_add_f(df_make(__fmul_rn(-0.5f, q.hi), __fmul_rn(-0.5f, q.lo)), 1.0f);
    if (!(t.hi > 0.0f)) return;  // gw = 0: the Float64 form adds zeros
    const df gw = df_mul(d.k.dw_coef, df_mul(df_sqr(t), t));
    df vr = df_mul(df_sub(a.vi[0], vj[0]), pd[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) vr = df_add(vr, df_mul(df_sub(a.vi[k], vj[k]), pd[k]));
    // Monaghan: Pi = -alpha c0 h v.x / ((d^2 + eps h^2) rho_mean) for approaching pairs
    // (v.x < 0), else 0
    df sum = df_add(a.Pi, df_make(s0.x, s0.y));
    if (vr.hi < 0.0f) {
      const df rm = df_add(a.rhoi, df_make(s0.z, s0.w));
      const df den = df_mul(df_add(d2, d.k.eps_h2),
                            df_make(__fmul_rn(0.5f, rm.hi), __fmul_rn(0.5f, rm.lo)));
      sum = df_add(sum, df_div(df_mul(d.k.m_alpha_c0_h, vr), den));
    }
    const df sc = df_mul(df_mul(d.k.m_mass, sum), gw);
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] = df_add(a.a[k], df_mul(sc, pd[k]));
  }
  static __device__ __forceinline__ void finish_df(AccDF& a, const Params& p, const Query<T, D>& q,
                                                   const DF64Geom&) {
#pragma unroll
    for (int k = 0; k < D; ++k) p.accel[(int64_t)q.i * D + k] = (T)df_to(a.a[k]);
  }
};

// ================================================================== adjoint (loss, dL/dx)
// L = sum_i (rho_i - 1)^2 + lambda E, rho_i = sum_j m W(d_ij), E = 1/2 sum_i sum_j phi(d_ij),
// phi(d) = m^2 (1/d - 1/R) for 0 < d < R.  The forward sweep stores g = 2 (rho - 1) beside
// the coordinates in slot order; the backward sweep reads it for every candidate:
// dL/dx_k = sum_j [(g_k + g_j) m W'(d) / d + lambda phi'(d) / d] (x_k - x_j).
template <typename T>
struct AdjointParams {
  SphConst<T> c;         // mass, inv_h, sigma, dw_coef = -5 sigma / h^2
  T cutoff, inv_cutoff, lambda;
  T cutoff2;             // cutoff^2: the truncation is decided on d^2 (see PotentialParams)
  T* density;            // forward: out, original order
  T* terms;              // forward: out, original order
  T* pa;                 // sorted state (x, y, z, g): forward writes, backward reads
  T* grad;               // backward: out, original order
  const double* scale;   // backward: upstream dL (device), or null
};

template <typename T, int D>
struct FAdjointForward {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = true;
  using Params = AdjointParams<T>;
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) {
    if (p.pa != nullptr) store4(p.pa, k, V4<T>{(T)NAN, (T)NAN, (T)NAN, (T)0});
  }
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T w, e; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) {
    a.w = (T)0;
    a.e = (T)0;
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t,
                                              const T*, T d2, T) {
    const T r = fsqrt(d2);
    const T q = r * p.c.inv_h;
    const T t = fmax((T)1 - (T)0.5 * q, (T)0);
    const T t2 = t * t;
    a.w += t2 * t2 * ((T)2 * q + (T)1);
    if (d2 > (T)0 && d2 < p.cutoff2) a.e += fdiv((T)1, r) - p.inv_cutoff;
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    const T rho = p.c.mass * p.c.sigma * a.w;
    const T dr = rho - (T)1;
    p.density[q.i] = rho;
    p.terms[q.i] = dr * dr + (T)0.5 * p.lambda * p.c.mass * p.c.mass * a.e;
    if (p.pa != nullptr && q.k >= 0) {
      V4<T> va{(T)0, (T)0, (T)0, (T)2 * dr};
      T* xa = &va.x;
#pragma unroll
      for (int k = 0; k < D; ++k) xa[k] = q.x[k];
      store4(p.pa, q.k, va);
    }
  }
};

template <typename T, int D>
struct FAdjointBackward {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = AdjointParams<T>;
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T a[D]; T gk; };
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    a.gk = load4(p.pa, q.k).w;
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] = (T)0;
  }
  // In 3D the candidates come from the state itself and `aux` is their g.
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T* pd, T d2, T aux) {
    if (!(d2 > (T)0)) return;  // the point itself (and coincident points): no direction
    const T gj = D == 3 ? aux : load4(p.pa, js).w;
    const T r = fsqrt(d2);
    const T q = r * p.c.inv_h;
    const T t = fmax((T)1 - (T)0.5 * q, (T)0);
    T s = (a.gk + gj) * p.c.mass * p.c.dw_coef * (t * t * t);
    if (d2 < p.cutoff2) s -= fdiv(p.lambda * p.c.mass * p.c.mass, d2 * r);
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] += s * pd[k];
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    const T sc = p.scale != nullptr ? (T)*p.scale : (T)1;
#pragma unroll
    for (int k = 0; k < D; ++k) p.grad[(int64_t)q.i * D + k] = sc * a.a[k];
  }
};

// Pair functions that build the pair cache while they run.
// No pair arithmetic: with WithMask, a sweep that only records the pair cache.  The Float64
// WCSPH density in double-float (DF64) records its neighbours this way and then sums over
// the cache, so that the double-float work runs in the cache walk's lanes.
struct NoneParams { int32_t pad_; };
template <typename T, int D>
struct FNone {
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  using Params = NoneParams;
  struct Acc {};
  struct AccDF {};
  static __device__ __forceinline__ void vacant(const Params&, int32_t) {}
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  static __device__ __forceinline__ void init(Acc&, const Params&, const Query<T, D>&) {}
  static __device__ __forceinline__ void pair(Acc&, const Params&, const Query<T, D>&, int32_t,
                                              const T*, T, T) {}
  static __device__ __forceinline__ void finish(Acc&, const Params&, const Query<T, D>&) {}
  static __device__ __forceinline__ void init_df(AccDF&, const Params&, const Query<T, D>&,
                                                 const DF64Geom&) {}
  static __device__ __forceinline__ void pair_df(AccDF&, const Params&, int32_t, const df*, df,
                                                 const DF64Geom&) {}
  static __device__ __forceinline__ void finish_df(AccDF&, const Params&, const Query<T, D>&,
                                                   const DF64Geom&) {}
};
// Pair functions whose accepted pairs need no pos_diff or d^2 (DF64 decides them from the
// Float32 d^2 where that is certain)
template <class F>
struct df_no_geometry { static constexpr bool value = false; };
template <typename T, int D>
struct df_no_geometry<FNone<T, D>> { static constexpr bool value = true; };
template <typename T, int D, class G>
struct df_no_geometry<WithMask<T, D, G>> { static constexpr bool value = df_no_geometry<G>::value; };

template <typename T, int D> using FDensityMask = WithMask<T, D, FDensity<T, D>>;
template <typename T, int D> using FNoneMask = WithMask<T, D, FNone<T, D>>;
template <typename T, int D> using FAdjointForwardMask = WithMask<T, D, FAdjointForward<T, D>>;

// ================================================================== traversal kernel
__device__ __forceinline__ int32_t pwrap(int32_t c, int32_t nc) {
  return c < 2 ? c + nc : (c > nc + 1 ? c - nc : c);
}

template <typename T, int D>
__device__ __forceinline__ T d2_exact(const T* pd) {
  T d2 = xmul(pd[0], pd[0]);
#pragma unroll
  for (int k = 1; k < D; ++k) d2 = xadd(d2, xmul(pd[k], pd[k]));
  return d2;
}

// With FMA contraction: within 6 units in the last place of d2_exact (both are sums of
// three non-negative products with at most three roundings each).
template <typename T, int D>
__device__ __forceinline__ T d2_fast(const T* pd) {
  T d2 = pd[0] * pd[0];
#pragma unroll
  for (int k = 1; k < D; ++k) d2 = fma(pd[k], pd[k], d2);
  return d2;
}

template <typename T, int D>
__device__ __forceinline__ bool wrap_needed(const GridDev<T>& g, const T* pd) {
  bool w = false;
#pragma unroll
  for (int k = 0; k < D; ++k) w |= !(fabs(pd[k]) < g.half_box[k]);
  return w;
}

template <typename T, int D>
__device__ __forceinline__ void wrap(const GridDev<T>& g, T* pd) {
#pragma unroll
  for (int k = 0; k < D; ++k)
    pd[k] = xsub(pd[k], xmul(g.box_size[k], xrint(xdiv(pd[k], g.box_size[k]))));
}

// The reference's pair geometry: pos_diff and d2 exactly as neighborhood_search.jl:547-555
// and :428-436 compute them.
template <typename T, int D, bool PER>
__device__ __forceinline__ T pair_geom(const GridDev<T>& g, const T* xi, const T* yj, T* pd) {
#pragma unroll
  for (int k = 0; k < D; ++k) pd[k] = xsub(xi[k], yj[k]);
  T d2 = d2_exact<T, D>(pd);
  if (PER && d2 > g.r2 && wrap_needed<T, D>(g, pd)) {
    wrap<T, D>(g, pd);
    d2 = d2_exact<T, D>(pd);
  }
  return d2;
}


// ------------------------------------------------------------------ mixed precision
// Float64 coordinates with a Float32 search radius (PN_FLAG_FLOAT32_SEARCH): the reference
// converts pos_diff = xi - yj (computed in Float64) to Float32, then computes d2, the
// periodic correction and the test d2 <= r^2 in Float32 (neighborhood_search.jl:402-410,
// :428-436), and the pair function sees the Float32 pos_diff and distance.
// The traversal runs in Float64 with a radius widened past the rounding of that Float32
// arithmetic, so its candidates hold every such neighbour; Mixed<D, F> redoes the Float32
// geometry and test for each candidate and hands the accepted ones to the Float32 pair
// function F.
struct MixedGeom {
  float r2;            // fl32(r * r)
  float box[3];        // PeriodicBox size (Float32)
  int32_t per;         // periodic box present (the traversal's PER)
  const double* pos;   // cell-sorted coordinates (a candidate's Float64 values)
  const float* state;  // 3D force / adjoint sweeps: F's aux is state[4 js + 3], or null
  const float* hi;     // MixedFast: the coordinates split into Float32 hi + lo parts
  const float* lo;
  float eb;            // MixedFast: bound on what the split loses of x - y
};

// Error-free sum: s + e == a + b exactly (Knuth's TwoSum, additions only).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Float32(Float64(x - y)) for x = xh + xl + ex, y = yh + yl + ey (xh = fl32(x), xl =
// fl32(x - xh)), with Float32 operations only.  (s, t) and (p, q) hold xh - yh and xl - yl
// exactly; their sum, formed as zh + zl with zh its nearest Float32, is off from x - y by at
// most eb (the lost ex - ey plus the rounding of t + p + q).  zh is the answer when x - y and
// its Float64 rounding lie strictly inside zh's rounding interval: |zl| + eb + |zh| 2^-52
// below half a unit in zh's last place (a quarter below a power of two, where the interval
// is narrower underneath).  Returns false otherwise (then x - y is formed in Float64).
__device__ __forceinline__ bool diff_f32(float xh, float xl, float yh, float yl, float eb,
                                         float& r) {
  float s, t, p, q;
  two_sum(xh, -yh, s, t);
  two_sum(xl, -yl, p, q);
  const float w = __fadd_rn(__fadd_rn(t, p), q);
  float zh, zl;
  two_sum(s, w, zh, zl);
  const float az = fabsf(zh);
  if (!(az >= 1e-30f)) return false;  // tiny or zero (or NaN)
  const int bits = __float_as_int(az);
  float half_ulp = __int_as_float((bits & 0x7f800000) - (24 << 23));
  if ((bits & 0x007fffff) == 0) half_ulp = __fmul_rn(half_ulp, 0.5f);
  if (!(__fsub_rn(half_ulp, fabsf(zl)) > __fadd_rn(eb, __fmul_rn(az, 2.3e-16f)))) return false;
  r = zh;
  return true;
}
template <class PF>
struct MixedParams {
  PF f;
  MixedGeom m;
};

template <int D, class F>
struct Mixed {
  static constexpr bool kCountOnly = false;  // every candidate is re-tested in Float32
  static constexpr bool kInline = false;     // a costly pair step (see MixedFast)
  using Params = MixedParams<typename F::Params>;  // the same type for every D
  using Acc = typename F::Acc;
  static __device__ __forceinline__ Query<float, D> narrow(const Query<double, D>& q) {
    Query<float, D> r;
    r.i = q.i;
    r.q = q.q;
    r.k = q.k;
#pragma unroll
    for (int k = 0; k < D; ++k) r.x[k] = __double2float_rn(q.x[k]);
    return r;
  }
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) { F::vacant(p.f, k); }
  static __device__ __forceinline__ void fail(const Params& p, const Query<double, D>& q) {
    F::fail(p.f, narrow(q));
  }
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<double, D>& q) {
    F::init(a, p.f, narrow(q));
  }
  // pd: the traversal's Float64 pos_diff, the plain difference unless a periodic image was
  // taken -- with a periodic box the difference is recomputed from the candidate.
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<double, D>& q,
                                              int32_t js, const double* pd, double, double) {
    float pf[D];
    if (p.m.per) {
      double yj[D];
      load_pos<double, D>(p.m.pos, js, yj);
#pragma unroll
      for (int k = 0; k < D; ++k) pf[k] = __double2float_rn(xsub(q.x[k], yj[k]));
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) pf[k] = __double2float_rn(pd[k]);
    }
    float d2 = d2_exact<float, D>(pf);
    if (p.m.per && d2 > p.m.r2) {
#pragma unroll
      for (int k = 0; k < D; ++k)
        pf[k] = xsub(pf[k], xmul(p.m.box[k], xrint(xdiv(pf[k], p.m.box[k]))));
      d2 = d2_exact<float, D>(pf);
    }
    if (!(d2 <= p.m.r2)) return;
    const float aux = p.m.state != nullptr ? __ldg(&p.m.state[4 * (int64_t)js + 3]) : 0.0f;
    F::pair(a, p.f, narrow(q), js, pf, d2, aux);
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<double, D>& q) {
    F::finish(a, p.f, narrow(q));
  }
};

// Mixed<D, F<float, D>> as a pair-function template of the traversal's (T, D).
template <template <typename, int> class F>
struct MixedOf {
  template <typename T, int D>
  using type = Mixed<D, F<float, D>>;
};

// The same rule for the cell-sorted queries (x is y), with the traversal itself in Float32:
// its candidates come from a Float32 copy of the coordinates (or the Float32 WCSPH state)
// with the radius widened past that rounding.  This wrapper decides the reference's Float32
// test exactly -- on a hi/lo Float32 difference, and where d2 lies near r^2 on the exact
// Float32(Float64(xi - yj)) (diff_f32) -- and gives the pair function that difference
// (the exact one near r^2, else one within about 2^-22 of it).
template <int D, class F>
struct MixedFast {
  static constexpr bool kCountOnly = false;
  // candidates are classified in chunks, then each lane walks its own accepted ones (the
  // inline form, with lanes waiting at every candidate another lane accepts, measured the
  // same or slower)
  static constexpr bool kInline = false;
  // a pair cache (F = WithMask<...>) records only the pairs this wrapper accepts
  static constexpr bool kRowHook = has_row_hook<F>::value;
  using Params = MixedParams<typename F::Params>;
  struct Acc { typename F::Acc f; float xl[D]; };
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) { F::vacant(p.f, k); }
  static __device__ __forceinline__ void fail(const Params& p, const Query<float, D>& q) {
    F::fail(p.f, q);
  }
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<float, D>& q) {
    F::init(a.f, p.f, q);
    load_pos<float, D>(p.m.lo, q.k, a.xl);
  }
  static __device__ __forceinline__ void row_begin(Acc& a, const Params& p,
                                                   const Query<float, D>& q, int ri, int32_t b0,
                                                   int32_t e0) {
    if constexpr (kRowHook) F::row_begin(a.f, p.f, q, ri, b0, e0, false);
  }
  static __device__ __forceinline__ void no_rows(Acc& a) {
    if constexpr (kRowHook) F::no_rows(a.f);
  }
  static __device__ __forceinline__ void ovf_begin(Acc& a, int32_t ob0, int32_t oe0) {
    if constexpr (kRowHook) F::ovf_begin(a.f, ob0, oe0);
  }
  // The exact Float32(Float64(xi - yj)) from the hi/lo split (q.x holds the query's hi
  // part), in Float64 where the split cannot decide the rounding.
  static __device__ __forceinline__ void exact_diff(const Acc& a, const Params& p,
                                                    const Query<float, D>& q, int32_t js,
                                                    const float* yh, const float* yl,
                                                    float* pf) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < D; ++k) ok &= diff_f32(q.x[k], a.xl[k], yh[k], yl[k], p.m.eb, pf[k]);
    if (!ok) {
      double xi[D], yj[D];
      load_pos<double, D>(p.m.pos, q.k, xi);
      load_pos<double, D>(p.m.pos, js, yj);
#pragma unroll
      for (int k = 0; k < D; ++k) pf[k] = __double2float_rn(xsub(xi[k], yj[k]));
    }
  }
  static __device__ __forceinline__ void wrap_f32(const Params& p, float* pf) {
#pragma unroll
    for (int k = 0; k < D; ++k)
      pf[k] = xsub(pf[k], xmul(p.m.box[k], xrint(xdiv(pf[k], p.m.box[k]))));
  }
  // pos_diff as (xh - yh) + (xl - yl) in Float32: within about 2^-22 |pos_diff| of the
  // reference's Float32(Float64(xi - yj)), close enough for the pair function's sums.  The
  // neighbour test (and the periodic image) is decided on it unless d2 lies within a
  // relative 1e-5 of r^2, where the exact pos_diff decides instead.
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<float, D>& q,
                                              int32_t js, const float*, float, float aux) {
    float yh[D], yl[D], pf[D];
    load_pos<float, D>(p.m.hi, js, yh);
    load_pos<float, D>(p.m.lo, js, yl);
#pragma unroll
    for (int k = 0; k < D; ++k)
      pf[k] = js == q.k ? 0.0f : __fadd_rn(__fsub_rn(q.x[k], yh[k]), __fsub_rn(a.xl[k], yl[k]));
    const float band = __fmul_rn(p.m.r2, 1e-5f);
    float d2 = d2_exact<float, D>(pf);
    bool exact = fabsf(__fsub_rn(d2, p.m.r2)) <= band;
    if (!exact && p.m.per && d2 > p.m.r2) {
      wrap_f32(p, pf);
      d2 = d2_exact<float, D>(pf);
      exact = fabsf(__fsub_rn(d2, p.m.r2)) <= band;
    }
    if (exact && js != q.k) {
      exact_diff(a, p, q, js, yh, yl, pf);
      d2 = d2_exact<float, D>(pf);
      if (p.m.per && d2 > p.m.r2) {
        wrap_f32(p, pf);
        d2 = d2_exact<float, D>(pf);
      }
    }
    if (!(d2 <= p.m.r2)) return;
    F::pair(a.f, p.f, q, js, pf, d2, aux);
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<float, D>& q) {
    F::finish(a.f, p.f, q);
  }
};

template <template <typename, int> class F>
struct MixedFastOf {
  template <typename T, int D>
  using type = MixedFast<D, F<float, D>>;
};

// ------------------------------------------------------------------ Float64 via Float32
// A Float64 search's cell-sorted queries (x is y) are traversed in Float32: over the
// coordinates rounded to Float32 (d_pos32), with the radius widened past that rounding, so
// the Float32 candidates hold every Float64 neighbour and few others (a shell of relative
// width ~1e-4).  Exact64<D, F> then redoes the reference's Float64 geometry and test for
// each candidate from the Float64 coordinates -- pos_diff = xi - yj, d2 = dot, the periodic
// image when d2 > r^2, accepted when d2 <= r^2 -- and hands the accepted ones to the
// Float64 pair function F.  The candidate tests run on the Float32 units; only the
// neighbours' arithmetic runs on GB300's Float64 units, whose rate is 1/64 of Float32's.
// Neighbour sets, pos_diff and d2 are the Float64 traversal's exactly.
struct Exact64Geom {
  GridDev<double> g;    // the search's Float64 geometry (r^2, periodic box)
  const double* pos;    // cell-sorted Float64 coordinates
  const double* state;  // 3D force / adjoint-backward sweeps: candidates and aux, or null
  int32_t per;          // periodic box
  int32_t pad_;
};
template <class PF>
struct Exact64Params {
  PF f;
  Exact64Geom m;
};

template <int D, class F>
struct Exact64 {
  static constexpr bool kCountOnly = false;  // every candidate is decided in Float64
  static constexpr bool kInline = false;     // compacted: the pair step is Float64 work
  static constexpr bool kRowHook = has_row_hook<F>::value;  // a pair cache records F's pairs
  using Params = Exact64Params<typename F::Params>;  // the same type for every D
  struct Acc { typename F::Acc f; double x[D]; };
  static __device__ __forceinline__ Query<double, D> wide(const Query<float, D>& q,
                                                          const double* x) {
    Query<double, D> r;
    r.i = q.i;
    r.q = q.q;
    r.k = q.k;
#pragma unroll
    for (int k = 0; k < D; ++k) r.x[k] = x[k];
    return r;
  }
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) { F::vacant(p.f, k); }
  static __device__ __forceinline__ void fail(const Params& p, const Query<float, D>& q) {
    const double z[D] = {};
    F::fail(p.f, wide(q, z));
  }
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<float, D>& q) {
    load_pos<double, D>(p.m.pos, q.k, a.x);
    F::init(a.f, p.f, wide(q, a.x));
  }
  static __device__ __forceinline__ void row_begin(Acc& a, const Params& p,
                                                   const Query<float, D>& q, int ri, int32_t b0,
                                                   int32_t e0) {
    if constexpr (kRowHook) F::row_begin(a.f, p.f, wide(q, a.x), ri, b0, e0, false);
  }
  static __device__ __forceinline__ void no_rows(Acc& a) {
    if constexpr (kRowHook) F::no_rows(a.f);
  }
  static __device__ __forceinline__ void ovf_begin(Acc& a, int32_t ob0, int32_t oe0) {
    if constexpr (kRowHook) F::ovf_begin(a.f, ob0, oe0);
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<float, D>& q,
                                              int32_t js, const float*, float, float) {
    double yj[D], pd[D];
    const double aux = load_cand<double, D>(p.m.state != nullptr ? p.m.state : p.m.pos, js, yj);
    const double d2 = p.m.per ? pair_geom<double, D, true>(p.m.g, a.x, yj, pd)
                              : pair_geom<double, D, false>(p.m.g, a.x, yj, pd);
    if (!(d2 <= p.m.g.r2)) return;
    F::pair(a.f, p.f, wide(q, a.x), js, pd, d2, aux);
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<float, D>& q) {
    F::finish(a.f, p.f, wide(q, a.x));
  }
};

template <template <typename, int> class F>
struct Exact64Of {
  template <typename T, int D>
  using type = Exact64<D, F<double, D>>;
};

// A Float64 search's WCSPH sweeps with their sums in double-float (3D, no periodic box).
// Like Exact64, the Float32 traversal over the coordinates' Float32 roundings finds a
// superset of the neighbours; each candidate's pos_diff is then formed from the three-part
// Float32 splits of the two Float64 positions (df_diff3: the exact difference, kept to
// double-float precision) and d^2 from it in double-float.  The neighbour test is the
// Float64 one, decided by the double-float d^2 outside a band of 1e-12 r^2 around r^2 (its
// error is below 1e-13 d^2) and by the Float64 geometry inside the band.  The accepted
// pairs go to F's double-float pair function (pair_df).  Neighbour sets are the Float64
// ones; the sums agree with Float64 ones to about 1e-14 of their terms.
template <class PF>
struct DF64Params {
  PF f;
  Exact64Geom m;
  DF64Geom d;
};

template <int D, class F>
struct DF64 {
  static_assert(D == 3, "double-float sweeps are three-dimensional");
  static constexpr bool kCountOnly = false;
  static constexpr bool kInline = false;
  static constexpr bool kRowHook = has_row_hook<F>::value;
  using Params = DF64Params<typename F::Params>;
  struct Acc { typename df_acc<F>::type f; float xb[D], xc[D]; };
  static __device__ __forceinline__ Query<double, D> wide(const Query<float, D>& q,
                                                          const double* x) {
    Query<double, D> r;
    r.i = q.i;
    r.q = q.q;
    r.k = q.k;
#pragma unroll
    for (int k = 0; k < D; ++k) r.x[k] = x[k];
    return r;
  }
  static __device__ __forceinline__ void vacant(const Params& p, int32_t k) { F::vacant(p.f, k); }
  static __device__ __forceinline__ void fail(const Params& p, const Query<float, D>& q) {
    const double z[D] = {};
    F::fail(p.f, wide(q, z));
  }
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<float, D>& q) {
    const float4 b = __ldg(reinterpret_cast<const float4*>(p.d.xb) + q.k);
    const float4 c = __ldg(reinterpret_cast<const float4*>(p.d.xc) + q.k);
    a.xb[0] = b.x; a.xb[1] = b.y; a.xb[2] = b.z;
    a.xc[0] = c.x; a.xc[1] = c.y; a.xc[2] = c.z;
    double x[D];
    load_pos<double, D>(p.m.pos, q.k, x);
    F::init_df(a.f, p.f, wide(q, x), p.d);
  }
  static __device__ __forceinline__ void row_begin(Acc& a, const Params& p,
                                                   const Query<float, D>& q, int ri, int32_t b0,
                                                   int32_t e0) {
    if constexpr (kRowHook) {
      const double z[D] = {};
      F::row_begin(a.f, p.f, wide(q, z), ri, b0, e0, false);
    }
  }
  static __device__ __forceinline__ void no_rows(Acc& a) {
    if constexpr (kRowHook) F::no_rows(a.f);
  }
  static __device__ __forceinline__ void ovf_begin(Acc& a, int32_t ob0, int32_t oe0) {
    if constexpr (kRowHook) F::ovf_begin(a.f, ob0, oe0);
  }
  // q.x: the query's Float32 part xa (the traversal's coordinates); d2_32: the traversal's
  // Float32 d^2
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<float, D>& q,
                                              int32_t js, const float*, float d2_32, float) {
    if constexpr (df_no_geometry<F>::value) {  // only the decision is wanted
      if (d2_32 < p.d.k.r_in2) {
        F::pair_df(a.f, p.f, js, nullptr, df_make(0.0f), p.d);
        return;
      }
    }
    const float4 ya = __ldg(reinterpret_cast<const float4*>(p.d.xa) + js);
    const float4 yb = __ldg(reinterpret_cast<const float4*>(p.d.xb) + js);
    const float4 yc = __ldg(reinterpret_cast<const float4*>(p.d.xc) + js);
    df pd[3];
    pd[0] = df_diff3(q.x[0], a.xb[0], a.xc[0], ya.x, yb.x, yc.x);
    pd[1] = df_diff3(q.x[1], a.xb[1], a.xc[1], ya.y, yb.y, yc.y);
    pd[2] = df_diff3(q.x[2], a.xb[2], a.xc[2], ya.z, yb.z, yc.z);
    const df d2 = df_add_pos(df_add_pos(df_sqr(pd[0]), df_sqr(pd[1])), df_sqr(pd[2]));
    bool accept;
    if (df_lt(d2, p.d.k.r2_lo)) {
      accept = true;
    } else if (df_gt(d2, p.d.k.r2_hi)) {
      accept = false;
    } else {  // the band: the Float64 geometry decides
      double xi[D], yj[D], pd64[D];
      load_pos<double, D>(p.m.pos, q.k, xi);
      load_pos<double, D>(p.m.pos, js, yj);
      accept = pair_geom<double, D, false>(p.m.g, xi, yj, pd64) <= p.m.g.r2;
    }
    if (accept) F::pair_df(a.f, p.f, js, pd, d2, p.d);
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<float, D>& q) {
    double x[D];
    load_pos<double, D>(p.m.pos, q.k, x);
    F::finish_df(a.f, p.f, wide(q, x), p.d);
  }
};

template <template <typename, int> class F>
struct DF64Of {
  template <typename T, int D>
  using type = DF64<3, F<double, 3>>;
};

// The Float64 pair functions with double-float sums: the WCSPH density (with or without
// recording the pair cache) and force.
template <class F>
struct df64_ok { static constexpr bool value = false; };
template <>
struct df64_ok<FDensity<double, 3>> { static constexpr bool value = true; };
template <>
struct df64_ok<FForce<double, 3>> { static constexpr bool value = true; };
template <>
struct df64_ok<WithMask<double, 3, FDensity<double, 3>>> { static constexpr bool value = true; };

template <class F>
struct is_exact64 { static constexpr bool value = false; };
template <int D, class G>
struct is_exact64<Exact64<D, G>> { static constexpr bool value = true; };

// The Float64 pair functions that take the Float32 traversal (the others keep the Float64
// one): those of the WCSPH, n-body, count and adjoint sweeps, with or without a pair cache.
template <class F>
struct exact64_ok { static constexpr bool value = false; };
template <int D>
struct exact64_ok<FCount<double, D>> { static constexpr bool value = true; };
template <int D>
struct exact64_ok<FNBody<double, D>> { static constexpr bool value = true; };
template <int D>
struct exact64_ok<FDensity<double, D>> { static constexpr bool value = true; };
template <int D>
struct exact64_ok<FForce<double, D>> { static constexpr bool value = true; };
template <int D>
struct exact64_ok<FAdjointForward<double, D>> { static constexpr bool value = true; };
template <int D>
struct exact64_ok<FAdjointBackward<double, D>> { static constexpr bool value = true; };
template <int D, class G>
struct exact64_ok<WithMask<double, D, G>> { static constexpr bool value = exact64_ok<G>::value; };


// ------------------------------------------------------------------ candidate scan
// Candidates are classified without branches.  The exact path (classify, kExact) gives
// `hit` when the FMA form of d2 is clearly inside r^2 and `slow` when the exact form must
// decide (d2 in the band around r^2) or, with WRAP, when the pair may need its periodic
// image.  The fast path (classify_superset) only tests the FMA form against the band's
// upper edge: a superset of the neighbours whose band members the pair step re-checks
// exactly (it recomputes the geometry anyway).
template <typename T, int D, bool WRAP>
__device__ __forceinline__ void classify(const TravArgs<T>& a, const T* xi, const T* yj,
                                         uint32_t bit, uint32_t& hit, uint32_t& slow) {
  T pd[D];
#pragma unroll
  for (int k = 0; k < D; ++k) pd[k] = xsub(xi[k], yj[k]);
  const T f = d2_fast<T, D>(pd);
  const bool near = f <= a.r2_lo;  // false for NaN (vacated slots, NaN points)
  bool s = !near & (f <= a.r2_hi);
  if (WRAP) s |= !near & wrap_needed<T, D>(a.g, pd);  // the exact path rejects NaN
  hit |= near ? bit : 0u;
  slow |= s ? bit : 0u;
}

template <typename T, int D>
__device__ __forceinline__ void classify_superset(const TravArgs<T>& a, const T* xi, const T* yj,
                                                  uint32_t bit, uint32_t& hit) {
  T pd[D];
#pragma unroll
  for (int k = 0; k < D; ++k) pd[k] = xsub(xi[k], yj[k]);
  hit |= d2_fast<T, D>(pd) <= a.r2_hi ? bit : 0u;  // false for NaN
}

// Apply the pair function to candidate slot js.  The geometry is recomputed with the
// periodic image the neighbour test used; with VERIFY (a superset classification) a
// candidate inside the band around r^2 is first decided exactly.
template <typename T, int D, bool WRAP, bool VERIFY, class F>
__device__ __forceinline__ void apply_pair(const TravArgs<T>& a, const typename F::Params& p,
                                           typename F::Acc& acc, const Query<T, D>& q,
                                           int32_t js) {
  T yj[D], pd[D];
  const T aux = load_cand<T, D>(a.pos, js, yj);
#pragma unroll
  for (int k = 0; k < D; ++k) pd[k] = xsub(q.x[k], yj[k]);
  T d2 = d2_fast<T, D>(pd);
  if (VERIFY && d2 > a.r2_lo && !(d2_exact<T, D>(pd) <= a.g.r2)) return;
  if (WRAP && d2 > a.r2_lo) {
    const T de = d2_exact<T, D>(pd);
    if (de > a.g.r2 && wrap_needed<T, D>(a.g, pd)) {
      wrap<T, D>(a.g, pd);
      d2 = d2_fast<T, D>(pd);
    }
  }
  F::pair(acc, p, q, js, pd, d2, aux);
}

// Classify the candidates [base, base + n) (n <= 32; none when n <= 0) into one word of
// bits, in groups of eight loads in flight with compile-time bit positions.  Every lane
// runs the same code; only the number of groups differs, so lanes whose runs end at
// different points never execute two different code paths.  The last group may read up to
// seven slots past the run (the slot arrays carry that much padding); their bits are
// masked off.
template <typename T, int D, bool WRAP, bool SUPERSET>
__device__ __forceinline__ void classify_span(const TravArgs<T>& a, const T* xi, int32_t base,
                                              int n, uint32_t& hit, uint32_t& slow) {
  hit = 0u;
  slow = 0u;
#pragma unroll 1
  for (int e = 0; e < n; e += 8) {
    uint32_t gh = 0u, gs = 0u;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      T yj[D];
      load_cand<T, D>(a.pos, base + e + u, yj);
      if (SUPERSET) classify_superset<T, D>(a, xi, yj, 1u << u, gh);
      else classify<T, D, WRAP>(a, xi, yj, 1u << u, gh, gs);
    }
    const int left = n - e;
    const uint32_t live = left >= 8 ? 0xFFu : (1u << left) - 1u;
    hit |= (gh & live) << e;
    slow |= (gs & live) << e;
  }
}

// The candidates of one chunk of NW x 32 slots starting at c0: resolve the rare `slow` ones
// exactly, then apply the pair function to every accepted one in slot order (so a lane's
// sum runs in the reference's candidate order) with the warp's lanes converged.
template <typename T, int D, bool PER, bool WRAP, bool SUPERSET, class F, int NW>
__device__ __forceinline__ void chunk_done(const TravArgs<T>& a, const typename F::Params& p,
                                           typename F::Acc& acc, const Query<T, D>& q,
                                           int32_t c0, uint32_t* hit, uint32_t* slow) {
  if (!SUPERSET) {
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      while (slow[w]) {
        const int e = __ffs(slow[w]) - 1;
        slow[w] &= slow[w] - 1;
        T yj[D], pd[D];
        load_cand<T, D>(a.pos, c0 + 32 * w + e, yj);
        if (pair_geom<T, D, PER>(a.g, q.x, yj, pd) <= a.g.r2) hit[w] |= 1u << e;
      }
    }
  }
  if constexpr (F::kCountOnly) {
    int n = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) n += __popc(hit[w]);
    F::count(acc, n);
  } else {
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      uint32_t h = hit[w];
      while (h) {
        const int e = __ffs(h) - 1;
        h &= h - 1;
        apply_pair<T, D, WRAP, SUPERSET, F>(a, p, acc, q, c0 + 32 * w + e);
      }
    }
  }
}

// Candidates [beg, end) of one stencil run for this thread's query, in chunks of up to
// CHUNK_WORDS x 32: the tests are
// straight-line code, and the pair function runs once per chunk over its accepted
// candidates, so the lanes of a warp have similar amounts of pair work between the points
// where they reconverge.
constexpr int CHUNK_WORDS = 2;

// NOGROUP: one candidate at a time even for a group functor (the overflow runs).
template <typename T, int D, bool PER, bool WRAP, class F, bool NOGROUP = false>
__device__ __forceinline__ void scan_run(const TravArgs<T>& a, const typename F::Params& p,
                                         typename F::Acc& acc, const Query<T, D>& q,
                                         int32_t beg, int32_t end) {
  if constexpr (F::kInline) {
    // one candidate at a time with the exact test and the pair function applied in place
    // on the registers just loaded (a cheap pair function needs no compaction)
    if constexpr (sizeof(T) == 4 && D == 3 && !WRAP && has_group<F>::value && !NOGROUP) {
      // GROUP candidates per step, each d^2 formed exactly as in the loop below; the last
      // group reads up to GROUP - 1 slots past the run (the slot arrays' padding holds
      // them) and masks them off
      const uint64_t qxy = pack_f32x2(q.x[0], q.x[1]);
      const float r2 = a.g.r2;
      const int32_t n = end - beg;
      for (int32_t e = 0; e < n; e += GROUP) {
        float d2[GROUP];
        const float4* cg = reinterpret_cast<const float4*>(a.pos) + beg + e;
#pragma unroll
        for (int u = 0; u < GROUP; ++u) {
          const float4 cj = __ldg(cg + u);
          const uint64_t dxy = sub_f32x2(qxy, pack_f32x2(cj.x, cj.y));
          float sx, sy;
          unpack_f32x2(mul_f32x2(dxy, dxy), sx, sy);
          const float dz = __fsub_rn(q.x[2], cj.z);
          d2[u] = __fadd_rn(__fadd_rn(sx, sy), __fmul_rn(dz, dz));
        }
        if (n - e < GROUP) {  // the last group: the slots past the run are never accepted
#pragma unroll
          for (int u = 1; u < GROUP; ++u)
            if (u >= n - e) d2[u] = __int_as_float(0x7f800000);
        }
        F::group(acc, p, q, beg + e, d2, r2);  // accepted: d2 <= r2 (false for NaN)
      }
    } else if constexpr (sizeof(T) == 4 && D == 3 && !WRAP) {
      // the x and y differences and squares as packed pairs (sub/mul.rn.f32x2: the same
      // correctly rounded operations as the scalar exact form, two per instruction)
      const uint64_t qxy = pack_f32x2(q.x[0], q.x[1]);
      for (int32_t js = beg; js < end; ++js) {
        const float4 cj = __ldg(reinterpret_cast<const float4*>(a.pos) + js);
        const uint64_t dxy = sub_f32x2(qxy, pack_f32x2(cj.x, cj.y));
        float sx, sy;
        unpack_f32x2(mul_f32x2(dxy, dxy), sx, sy);
        const float dz = __fsub_rn(q.x[2], cj.z);
        const float d2 = __fadd_rn(__fadd_rn(sx, sy), __fmul_rn(dz, dz));
        if (d2 <= a.g.r2) {
          T pd[3];
          unpack_f32x2(dxy, pd[0], pd[1]);
          pd[2] = dz;
          F::pair(acc, p, q, js, pd, d2, (T)0);
        }
      }
    } else {
      for (int32_t js = beg; js < end; ++js) {
        T yj[D], pd[D];
        load_cand<T, D>(a.pos, js, yj);
        const T d2 = WRAP ? pair_geom<T, D, true>(a.g, q.x, yj, pd)
                          : pair_geom<T, D, false>(a.g, q.x, yj, pd);
        if (d2 <= a.g.r2) F::pair(acc, p, q, js, pd, d2, (T)0);
      }
    }
    return;
  }
  constexpr bool SUPERSET = !WRAP && !F::kCountOnly;
  for (int32_t c0 = beg; c0 < end; c0 += 32 * CHUNK_WORDS) {
    uint32_t hit[CHUNK_WORDS], slow[CHUNK_WORDS];
#pragma unroll
    for (int w = 0; w < CHUNK_WORDS; ++w)
      classify_span<T, D, WRAP, SUPERSET>(a, q.x, c0 + 32 * w, min(32, end - (c0 + 32 * w)),
                                          hit[w], slow[w]);
    chunk_done<T, D, PER, WRAP, SUPERSET, F, CHUNK_WORDS>(a, p, acc, q, c0, hit, slow);
  }
}

template <typename T, int D, bool PER, class F, bool NOGROUP = false>
__device__ __forceinline__ void scan_any(const TravArgs<T>& a, const typename F::Params& p,
                                         typename F::Acc& acc, const Query<T, D>& q,
                                         bool wrap, int32_t beg, int32_t end) {
  if (PER && wrap) scan_run<T, D, PER, PER, F, NOGROUP>(a, p, acc, q, beg, end);
  else scan_run<T, D, PER, false, F, NOGROUP>(a, p, acc, q, beg, end);
}

// Rows this short are scanned whole: the two binary searches would cost more than the
// candidates they skip.
constexpr int32_t CLIP_MIN_RUN = 32;

// First slot of the x-sorted run [b, e) with key >= v (lower) or key > v (upper); the key
// of slot k is key[k * S].
template <typename T, int S, bool UPPER>
__device__ __forceinline__ int32_t bound_x(const T* __restrict__ key, int32_t b, int32_t e, T v) {
  int32_t n = e - b;
  while (n > 0) {
    const int32_t h = n >> 1;
    const T xk = __ldg(&key[(int64_t)(b + h) * S]);
    if (UPPER ? !(v < xk) : (xk < v)) {
      b += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return b;
}

// Clip the x-sorted run [b0, e0) of the stencil row (oy, oz) to the query's reach
// x +- sqrt(r^2 - dy^2 - dz^2); an unreachable row becomes empty.  below/above: the query's
// distance (less the margin) to the lower/upper edge of its cell in y and z.  keyed: the
// run is searched by its sort keys (xkey) with the reach widened by `margin`.
template <typename T, int D>
__device__ __forceinline__ void clip_row(const TravArgs<T>& a, const Query<T, D>& q,
                                         const T* below, const T* above, int oy, int oz,
                                         int32_t& b0, int32_t& e0, T margin, bool keyed) {
  if (e0 - b0 <= CLIP_MIN_RUN) return;
  const T dy = oy < 0 ? below[1] : (oy > 0 ? above[1] : (T)0);
  const T dz = oz < 0 ? below[2] : (oz > 0 ? above[2] : (T)0);
  // slack for the rounding of these few operations (the exact test decides)
  const T rem = a.g.r2 * (T)1.00001 - dy * dy - dz * dz;
  if (rem < (T)0) {
    e0 = b0;
    return;
  }
  const T w = fsqrt(rem) * (T)1.00001 + a.clip_m[0] + margin;
  if constexpr (std::is_same<T, float>::value) {
    if (keyed) {
      b0 = bound_x<float, 1, false>(a.xkey, b0, e0, q.x[0] - w);
      e0 = bound_x<float, 1, true>(a.xkey, b0, e0, q.x[0] + w);
      return;
    }
  }
  b0 = bound_x<T, PS<D>::value, false>(a.pos, b0, e0, q.x[0] - w);
  e0 = bound_x<T, PS<D>::value, true>(a.pos, b0, e0, q.x[0] + w);
}

// One query per thread.  A warp holds consecutive queries (in sorted mode: consecutive
// cell-sorted slots), so its lanes walk the same or shifted stencil rows in lockstep and
// share most candidate loads.  Rows are visited in the reference's CartesianIndices
// order; within a row the three cells x-1, x, x+1 are one slot run (main list, then the
// overflow list), or three runs where a periodic box wraps.
// With a periodic box the per-candidate image check is needed only near the box's faces:
// when every point lies inside the box and the query's cell is in [4, n_cells - 1] in every
// dimension, all its stencil cells are alias-free and |pos_diff| < 2 cell sizes < size / 2,
// so the reference's correction is the identity.
template <typename T, int D, bool PER, class F>
__device__ __forceinline__ void traverse_query(const TravArgs<T>& a, const typename F::Params& p,
                                               Query<T, D>& q, const int32_t* c, bool valid) {
  typename F::Acc acc;
  if (valid) F::init(acc, p, q);
  const GridDev<T>& g = a.g;
  bool wrap = false;
  if (PER) {
    wrap = a.outside == nullptr || *a.outside != 0;
#pragma unroll
    for (int k = 0; k < D; ++k) wrap |= c[k] < 4 || c[k] > g.ncell[k] - 1;
  }
  // row clipping (see TravArgs): the query's distance to the lower and upper edge of its
  // cell in y and z, reduced by the margin; rows near a periodic face are not clipped
  // the sort keys stand in for the positions while main slots have moved in place or been
  // vacated (overflow lists hold points); after a rebuild the positions are the keys
  T margin = (T)0;
  bool keyed = false;
  if (std::is_same<T, float>::value && a.xkey != nullptr) {
    margin = (T)__ldg(a.delta);
    keyed = margin > (T)0 || __ldg(&a.ovf_start[g.n_total]) > __ldg(&a.start[g.n_total]);
  }
  const bool clip = valid && !(PER && wrap) &&
                    (keyed || a.unsorted == nullptr || *a.unsorted == 0);
  if constexpr (has_row_hook<F>::value) {
    if (valid && !clip) F::no_rows(acc);  // rows are not single clipped runs here
  }
  T below[3] = {(T)0, (T)0, (T)0}, above[3] = {(T)0, (T)0, (T)0};
  if (clip) {
#pragma unroll
    for (int k = 1; k < D; ++k) {
      const T lo = g.min_pad[k] + (T)(c[k] - 1) * g.cell_size[k];  // the query cell's edge
      below[k] = fmax(q.x[k] - lo - a.clip_m[k], (T)0);
      above[k] = fmax(lo + g.cell_size[k] - q.x[k] - a.clip_m[k], (T)0);
    }
  }
  constexpr int OZ = D == 3 ? 1 : 0;
  constexpr int OY = D >= 2 ? 1 : 0;
#pragma unroll 1
  for (int oz = -OZ; oz <= OZ; ++oz) {
#pragma unroll 1
    for (int oy = -OY; oy <= OY; ++oy) {
      if (!valid) continue;
      int32_t row = 0;
      if (D == 3) row = ((PER ? pwrap(c[2] + oz, g.ncell[2]) : c[2] + oz) - 1) * g.n[0] * g.n[1];
      if (D >= 2) row += ((PER ? pwrap(c[1] + oy, g.ncell[1]) : c[1] + oy) - 1) * g.n[0];
      if (!PER || (c[0] >= 3 && c[0] <= g.ncell[0])) {
        const int32_t l0 = PN_IDX(a.err, BC_CELL, row + c[0] - 2, (int64_t)g.n_total - 2);
        int32_t b0 = __ldg(&a.start[l0]), e0 = __ldg(&a.start[l0 + 3]);
        PN_RUN(a.err, b0, e0, a.bc_slots);
        if (clip) {
          // the row's margin: the largest move in its three cells
          T rm = margin;
          if (keyed && a.cell_delta != nullptr)
            rm = (T)fmaxf(fmaxf(__ldg(&a.cell_delta[l0]), __ldg(&a.cell_delta[l0 + 1])),
                          __ldg(&a.cell_delta[l0 + 2]));
          clip_row<T, D>(a, q, below, above, oy, oz, b0, e0, rm, keyed);
          if constexpr (has_row_hook<F>::value)
            F::row_begin(acc, p, q, (oz + OZ) * (2 * OY + 1) + (oy + OY), b0, e0);
        }
        if (b0 < e0) scan_any<T, D, PER, F>(a, p, acc, q, wrap, b0, e0);
        if (a.ovf_start) {
          int32_t ob = __ldg(&a.ovf_start[l0]), oe = __ldg(&a.ovf_start[l0 + 3]);
          PN_RUN(a.err, ob, oe, a.bc_slots);
          if (clip && keyed) clip_row<T, D>(a, q, below, above, oy, oz, ob, oe, (T)0, true);
          if constexpr (has_row_hook<F>::value) {
            if (clip) F::ovf_begin(acc, ob, oe);
          }
          if (ob < oe) scan_any<T, D, PER, F, true>(a, p, acc, q, wrap, ob, oe);
        }
      } else {
#pragma unroll 1
        for (int ox = -1; ox <= 1; ++ox) {
          const int32_t l =
              PN_IDX(a.err, BC_CELL, row + pwrap(c[0] + ox, g.ncell[0]) - 1, g.n_total);
          int32_t b = __ldg(&a.start[l]), e = __ldg(&a.start[l + 1]);
          PN_RUN(a.err, b, e, a.bc_slots);
          scan_any<T, D, PER, F>(a, p, acc, q, wrap, b, e);
          if (a.ovf_start) {
            b = __ldg(&a.ovf_start[l]);
            e = __ldg(&a.ovf_start[l + 1]);
            PN_RUN(a.err, b, e, a.bc_slots);
            scan_any<T, D, PER, F>(a, p, acc, q, wrap, b, e);
          }
        }
      }
    }
  }
  if (valid) F::finish(acc, p, q);
}

// Sorted mode: queries are the cell-sorted slots (x is y, every point binned).  Slots
// [0, start[n_total]) are the main structure, then the overflow slots up to
// ovf_start[n_total]; vacated slots (perm < 0) are skipped.
template <typename T, int D, bool PER, class F>
__device__ __forceinline__ void sorted_query(const TravArgs<T>& a, const typename F::Params& p,
                                             int64_t k, int32_t n_slots) {
  Query<T, D> q;
  bool valid = k < n_slots;
  q.i = valid ? a.perm[PN_IDX(a.err, BC_QUERY_SLOT, k, a.bc_slots)] : -1;
  if (valid && q.i < 0) F::vacant(p, (int32_t)k);
  valid = valid && q.i >= 0;
  if (valid) q.i = PN_IDX(a.err, BC_POINT, q.i, a.bc_points);
  if (a.nb_len != nullptr && valid) valid = __ldg(&a.nb_len[k]) < 0;  // pair-cache rows only
  q.q = q.i;
  q.k = (int32_t)k;
  int32_t c[3] = {1, 1, 1};
  if (valid) {
    load_pos<T, D>(a.pos, k, q.x);
    const int32_t lin = PN_IDX(a.err, BC_CELL, a.cell_of_slot[k], a.g.n_total);
    c[0] = lin % a.g.n[0] + 1;
    if (D >= 2) c[1] = (lin / a.g.n[0]) % a.g.n[1] + 1;
    if (D == 3) c[2] = lin / (a.g.n[0] * a.g.n[1]) + 1;
  } else {
#pragma unroll
    for (int d = 0; d < D; ++d) q.x[d] = (T)0;
  }
  traverse_query<T, D, PER, F>(a, p, q, c, valid);
}

// Resident blocks per SM the traversal is compiled for: 8 (64 registers a thread), and 5
// for the Float64 pair functions behind the Float32 traversal, whose Float64 values take
// register pairs (and whose sweeps are bound by the Float64 units, not by occupancy).
template <class F>
struct trav_blocks { static constexpr int value = 8; };
template <int D, class G>
struct trav_blocks<Exact64<D, G>> { static constexpr int value = 5; };
template <int D, class G>
struct trav_blocks<DF64<D, G>> { static constexpr int value = 5; };
// the recording sweep of the double-float density: mostly the Float32 traversal (its
// double-float work only for the rare band candidates), so it keeps 8 blocks per SM
template <>
struct trav_blocks<DF64<3, WithMask<double, 3, FNone<double, 3>>>> {
  static constexpr int value = 8;
};

template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, trav_blocks<F>::value)
k_trav_sorted(const TravArgs<T> a, const typename F::Params p) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t n_slots = a.ovf_start ? a.ovf_start[a.g.n_total] : a.start[a.g.n_total];
  if ((int64_t)blockIdx.x * blockDim.x >= n_slots) return;  // whole block idle
  sorted_query<T, D, PER, F>(a, p, k, n_slots);
}

// The stencil traversal of the queries that a pair cache or precomputed lists could not
// hold (nb_len < 0), as a grid-stride loop over the slots on one wave of blocks: with the
// pair cache's flag clear (no such query) every block returns at once.
template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, trav_blocks<F>::value)
k_trav_fallback(const TravArgs<T> a, const typename F::Params p) {
  if (a.pc_any_fallback != nullptr && *a.pc_any_fallback == 0) return;
  const int32_t n_slots = a.ovf_start ? a.ovf_start[a.g.n_total] : a.start[a.g.n_total];
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n_slots;
       base += (int64_t)gridDim.x * blockDim.x)
    sorted_query<T, D, PER, F>(a, p, base + threadIdx.x, n_slots);
}

// List mode: queries are x[:, qlist[q]] (or q) in the given order.  A query whose
// neighbouring cells fall outside the grid is the reference's BoundsError.
template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, 8)
k_trav_list(const TravArgs<T> a, const typename F::Params p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if ((int64_t)blockIdx.x * blockDim.x >= a.n_q) return;  // whole block idle
  Query<T, D> q;
  bool valid = t < a.n_q;
  q.i = valid ? (a.qlist ? a.qlist[t] : (int32_t)t) : -1;
  q.q = (int32_t)t;
  q.k = -1;
  int32_t c[3] = {1, 1, 1};
  if (valid && (q.i < 0 || q.i >= a.n_x)) {
    set_error(a.err, PN_ERR_INVALID_ARG);
    F::fail(p, q);
    valid = false;
  }
  if (valid && a.g.hashed) {
    // a SpatialHashingCellList in a dense grid: the query's own cell; one outside the grid's
    // padding has no neighbours (the domain is unbounded)
    bool ok = true, inside = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      q.x[k] = a.x[(int64_t)q.i * D + k];
      int32_t ch = 0;
      ok &= hash_cell_1d(a.g, PER, k, q.x[k], ch);
      const int64_t i = (int64_t)ch + a.g.cell_off[k];
      inside &= i >= 2 && i <= a.g.n[k] - 1;
      c[k] = inside ? (int32_t)i : 2;
    }
    if (!ok) {
      set_error(a.err, PN_ERR_OUT_OF_DOMAIN);
      F::fail(p, q);
      valid = false;
    } else if (!inside) {
      typename F::Acc acc;
      F::init(acc, p, q);
      F::finish(acc, p, q);
      valid = false;
    }
  } else if (valid) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      q.x[k] = a.x[(int64_t)q.i * D + k];
      ok &= cell_coord_1d(a.g, PER, k, q.x[k], c[k]);
    }
    if (!ok) {
      set_error(a.err, PN_ERR_BOUNDS);
      F::fail(p, q);
      valid = false;
    }
  }
  if (!valid) {
#pragma unroll
    for (int d = 0; d < D; ++d) q.x[d] = (T)0;
  }
  traverse_query<T, D, PER, F>(a, p, q, c, valid);
}

// ================================================================== spatial hashing
// The run of cell cc: its hash list's entries are searched for the cell (one entry unless
// cells collide in the list); an empty run when the cell has no points.
template <int D>
__device__ __forceinline__ void hash_run(const int32_t* __restrict__ list,
                                         const int4* __restrict__ cell, const HashMod& hm,
                                         const int32_t* cc, int32_t& b, int32_t& e) {
  const int32_t h = spatial_hash<D>(cc, hm);
  const int32_t e1 = __ldg(&list[h + 1]);
  b = e = 0;
  for (int32_t k = __ldg(&list[h]); k < e1; ++k) {
    const int4 c = __ldg(&cell[k]);
    if (c.x == cc[0] && (D < 2 || c.y == cc[1]) && (D < 3 || c.z == cc[2])) {
      b = c.w;
      e = __ldg(&cell[k + 1]).w;
      return;
    }
  }
}

// One query over a SpatialHashingCellList: the 3^d cells in the reference's
// CartesianIndices order, each cell's run in slot order.  Cells need not line up with a
// periodic box's faces here, so with one every candidate is checked for its image.
// (Skipping the neighbouring cells that lie farther than r from the query saves nothing:
// the lanes of a warp are queries of one cell at different positions, and some lane
// nearly always needs each of the 3^d cells.)
template <typename T, int D, bool PER, class F>
__device__ __forceinline__ void traverse_query_hash(const TravArgs<T>& a,
                                                    const typename F::Params& p,
                                                    Query<T, D>& q, const int32_t* c,
                                                    bool valid) {
  typename F::Acc acc;
  if (!valid) return;
  F::init(acc, p, q);
  constexpr int OZ = D == 3 ? 1 : 0;
  constexpr int OY = D >= 2 ? 1 : 0;
#pragma unroll 1
  for (int oz = -OZ; oz <= OZ; ++oz) {
#pragma unroll 1
    for (int oy = -OY; oy <= OY; ++oy) {
#pragma unroll 1
      for (int ox = -1; ox <= 1; ++ox) {
        int32_t cc[3] = {c[0] + ox, c[1] + oy, c[2] + oz};
        if (PER) {
#pragma unroll
          for (int k = 0; k < D; ++k) cc[k] = pwrap(cc[k], a.g.ncell[k]);
        }
        int32_t b, e;
        hash_run<D>(a.hash_list, a.hash_cell, a.hash_mod, cc, b, e);
        PN_RUN(a.err, b, e, a.bc_slots);
        scan_any<T, D, PER, F>(a, p, acc, q, PER, b, e);
      }
    }
  }
  F::finish(acc, p, q);
}

template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, 8)
k_trav_hash_sorted(const TravArgs<T> a, const typename F::Params p) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t n_slots = a.start[a.g.n_total];
  if ((int64_t)blockIdx.x * blockDim.x >= n_slots) return;  // whole block idle
  Query<T, D> q;
  const bool valid = k < n_slots;
  q.i = valid ? PN_IDX(a.err, BC_POINT, a.perm[PN_IDX(a.err, BC_QUERY_SLOT, k, a.bc_slots)],
                       a.bc_points)
              : -1;
  q.q = q.i;
  q.k = (int32_t)k;
  int32_t c[3] = {0, 0, 0};
  if (valid) {
    load_pos<T, D>(a.pos, k, q.x);
    const int4 key = __ldg(&a.hash_key[k]);
    c[0] = key.x;
    c[1] = key.y;
    c[2] = key.z;
  }
  traverse_query_hash<T, D, PER, F>(a, p, q, c, valid);
}

template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, 8)
k_trav_hash_list(const TravArgs<T> a, const typename F::Params p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if ((int64_t)blockIdx.x * blockDim.x >= a.n_q) return;  // whole block idle
  Query<T, D> q;
  bool valid = t < a.n_q;
  q.i = valid ? (a.qlist ? a.qlist[t] : (int32_t)t) : -1;
  q.q = (int32_t)t;
  q.k = -1;
  int32_t c[3] = {0, 0, 0};
  if (valid && (q.i < 0 || q.i >= a.n_x)) {
    set_error(a.err, PN_ERR_INVALID_ARG);
    F::fail(p, q);
    valid = false;
  }
  if (valid) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      q.x[k] = a.x[(int64_t)q.i * D + k];
      ok &= hash_cell_1d(a.g, PER, k, q.x[k], c[k]);
    }
    if (!ok) {
      set_error(a.err, PN_ERR_OUT_OF_DOMAIN);
      F::fail(p, q);
      valid = false;
    }
  }
  traverse_query_hash<T, D, PER, F>(a, p, q, c, valid);
}

// ================================================================== precomputed lists
// nhs_precomputed.jl:206-247: every stored neighbour of the query, with pos_diff and d2
// recomputed exactly (and the periodic image when d2 > r^2); no distance check, like the
// reference.  `row` is the query's list.
template <typename T, int D, bool PER, class F>
__device__ __forceinline__ void list_query(const TravArgs<T>& a, const typename F::Params& p,
                                           Query<T, D>& q, int32_t row, bool valid) {
  typename F::Acc acc;
  if (!valid) return;
  F::init(acc, p, q);
  const int32_t n = __ldg(&a.nb_len[row]);
  const int4* nb = reinterpret_cast<const int4*>(a.nb) + __ldg(&a.nb_grp[row >> 5]) / 4 +
                   (row & 31);
  for (int32_t t = 0; t < n; t += 4) {
    const int4 quad = __ldg(&nb[8 * t]);  // quad t / 4 of the row: 32 int4 further per quad
    const int32_t js4[4] = {quad.x, quad.y, quad.z, quad.w};
    const int m = min(4, n - t);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (e < m) {
        const int32_t js = PN_IDX(a.err, BC_NEIGHBOUR, js4[e], a.bc_slots);
        T yj[D], pd[D];
        const T aux = load_cand<T, D>(a.pos, js, yj);
        const T d2 = pair_geom<T, D, PER>(a.g, q.x, yj, pd);
        F::pair(acc, p, q, js, pd, d2, aux);
      }
    }
  }
  F::finish(acc, p, q);
}

// Cell-sorted queries (lists built with x is y): row = slot.
template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, 8)
k_lists_sorted(const TravArgs<T> a, const typename F::Params p) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t n_slots = a.ovf_start ? a.ovf_start[a.g.n_total] : a.start[a.g.n_total];
  if ((int64_t)blockIdx.x * blockDim.x >= n_slots) return;  // whole block idle
  Query<T, D> q;
  bool valid = k < n_slots;
  q.i = valid ? a.perm[PN_IDX(a.err, BC_QUERY_SLOT, k, a.bc_slots)] : -1;
  if (valid && q.i < 0) F::vacant(p, (int32_t)k);
  valid = valid && q.i >= 0;
  if (valid) q.i = PN_IDX(a.err, BC_POINT, q.i, a.bc_points);
  q.q = q.i;
  q.k = (int32_t)k;
  if (valid) load_pos<T, D>(a.pos, k, q.x);
  if (valid && __ldg(&a.nb_len[k]) < 0) return;  // the grid launch after this one
  list_query<T, D, PER, F>(a, p, q, (int32_t)k, valid);
}

// One loop over all the query's neighbours, row by row: the main run's low and high mask
// word, then (OVF) the overflow run's word.  A lane moves to its next word when it has used
// up the current one, so lanes with different counts per row do not wait for one another
// row by row.  The next row's starts and masks are loaded when a row is entered, so a lane
// that moves on finds them in registers instead of stalling its warp on the load.  A
// neighbour's slot is the word's base slot plus its bit.
template <typename T, int D, bool PER, class F, bool OVF>
__device__ __forceinline__ void walk_masks(const TravArgs<T>& a, const typename F::Params& p,
                                           typename F::Acc& acc, const Query<T, D>& q,
                                           int64_t k) {
  constexpr int NR = D == 3 ? 9 : (D == 2 ? 3 : 1);
  if constexpr (!OVF) {
    // wi = 2 row + half indexes the query's 2 NR mask words
    int wi = 0;
    int32_t rb0 = __ldg(&a.pc_b0[k]);
    ulonglong2 m = __ldg(&a.pc_mask[k]);
    int32_t nb0 = 0;
    ulonglong2 nm = make_ulonglong2(0ull, 0ull);
    if (NR > 1) {
      nb0 = __ldg(&a.pc_b0[a.pc_stride + k]);
      nm = __ldg(&a.pc_mask[a.pc_stride + k]);
    }
    uint64_t w = m.x;
    for (;;) {
      while (w == 0) {
        if (++wi >= 2 * NR) break;
        if (wi & 1) {
          w = m.y;
        } else {
          rb0 = nb0;
          m = nm;
          w = m.x;
          const int nr = (wi >> 1) + 1;
          if (nr < NR) {
            const int64_t o = (int64_t)nr * a.pc_stride + k;
            nb0 = __ldg(&a.pc_b0[o]);
            nm = __ldg(&a.pc_mask[o]);
          }
        }
      }
      if (w == 0) break;
      const int e = __ffsll((long long)w) - 1;
      w &= w - 1;
      const int32_t js = PN_IDX(a.err, BC_NEIGHBOUR, rb0 + 64 * (wi & 1) + e, a.bc_slots);
      T yj[D], pd[D];
      const T aux = load_cand<T, D>(a.pos, js, yj);
      const T d2 = pair_geom<T, D, PER>(a.g, q.x, yj, pd);
      F::pair(acc, p, q, js, pd, d2, aux);
    }
    return;
  }
  constexpr int NP = 3;  // mask words per row: main low, main high, overflow
  int32_t rb0 = __ldg(&a.pc_b0[k]), nb0 = 0;
  ulonglong2 m = __ldg(&a.pc_mask[k]), nm = make_ulonglong2(0ull, 0ull);
  int32_t rob0 = -1, nob0 = -1;
  uint64_t om = 0ull, nom = 0ull;
  if constexpr (OVF) {
    rob0 = __ldg(&a.pc_ob0[k]);
    if (rob0 >= 0) om = __ldg(&a.pc_omask[k]);
  }
  if (NR > 1) {
    const int64_t o = a.pc_stride + k;
    nb0 = __ldg(&a.pc_b0[o]);
    nm = __ldg(&a.pc_mask[o]);
    if constexpr (OVF) {
      nob0 = __ldg(&a.pc_ob0[o]);
      if (nob0 >= 0) nom = __ldg(&a.pc_omask[o]);
    }
  }
  int row = 0, part = 0;
  int32_t base = rb0;
  uint64_t w = m.x;
  for (;;) {
    while (w == 0) {
      if (++part < NP) {
        if (part == 1) {
          w = m.y;
          base = rb0 + 64;
        } else {
          w = om;
          base = rob0;
        }
        continue;
      }
      if (++row >= NR) break;
      part = 0;
      rb0 = nb0;
      m = nm;
      w = m.x;
      base = rb0;
      if constexpr (OVF) {
        rob0 = nob0;
        om = nom;
      }
      if (row + 1 < NR) {
        const int64_t o = (int64_t)(row + 1) * a.pc_stride + k;
        nb0 = __ldg(&a.pc_b0[o]);
        nm = __ldg(&a.pc_mask[o]);
        if constexpr (OVF) {
          nob0 = __ldg(&a.pc_ob0[o]);
          nom = nob0 >= 0 ? __ldg(&a.pc_omask[o]) : 0ull;
        }
      }
    }
    if (w == 0) break;
    const int e = __ffsll((long long)w) - 1;
    w &= w - 1;
    const int32_t js = PN_IDX(a.err, BC_NEIGHBOUR, base + e, a.bc_slots);
    T yj[D], pd[D];
    const T aux = load_cand<T, D>(a.pos, js, yj);
    const T d2 = pair_geom<T, D, PER>(a.g, q.x, yj, pd);
    F::pair(acc, p, q, js, pd, d2, aux);
  }
}

// Cell-sorted queries over the pair cache's hit masks: for every stencil row, the accepted
// candidates of the row's clipped run, in slot order; queries marked for the fallback are
// left to the stencil launch after this one.
template <typename T, int D, bool PER, class F, bool OVF>
__device__ __forceinline__ void mask_query(const TravArgs<T>& a, const typename F::Params& p,
                                           int64_t k, int32_t n_slots);

// OVF: the instance for a cache with overflow masks while overflow lists hold points; the
// other instance returns at once then (each reads the same two words), so the common case
// keeps the smaller walk and its registers.  STRIDE: grid-stride over the queries (launched
// on one wave of blocks, so that it costs little when it returns at once; the host takes it
// when the last update it knows of kept no point in an overflow list).
template <typename T, int D, bool PER, class F, bool OVF = false, bool STRIDE = false>
__global__ void __launch_bounds__(TRAV_THREADS, trav_blocks<F>::value)
k_masks_sorted(const TravArgs<T> a, const typename F::Params p) {
  const int32_t n_slots = a.ovf_start ? a.ovf_start[a.g.n_total] : a.start[a.g.n_total];
  const bool ovf_walk = a.pc_ob0 != nullptr && n_slots > __ldg(&a.start[a.g.n_total]);
  if (ovf_walk != OVF) return;
  if constexpr (STRIDE) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n_slots; k += stride)
      mask_query<T, D, PER, F, OVF>(a, p, k, n_slots);
  } else {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((int64_t)blockIdx.x * blockDim.x >= n_slots) return;  // whole block idle
    mask_query<T, D, PER, F, OVF>(a, p, k, n_slots);
  }
}

// One cell-sorted query of the pair cache's walk.
template <typename T, int D, bool PER, class F, bool OVF>
__device__ __forceinline__ void mask_query(const TravArgs<T>& a, const typename F::Params& p,
                                           int64_t k, int32_t n_slots) {
  Query<T, D> q;
  bool valid = k < n_slots;
  q.i = valid ? a.perm[PN_IDX(a.err, BC_QUERY_SLOT, k, a.bc_slots)] : -1;
  if (valid && q.i < 0) F::vacant(p, (int32_t)k);
  valid = valid && q.i >= 0;
  if (!valid || __ldg(&a.pc_b0[PN_IDX(a.err, BC_PAIR_CACHE, k, a.pc_stride)]) < 0) return;
  q.i = PN_IDX(a.err, BC_POINT, q.i, a.bc_points);
  q.q = q.i;
  q.k = (int32_t)k;
  load_pos<T, D>(a.pos, k, q.x);
  typename F::Acc acc;
  F::init(acc, p, q);
  walk_masks<T, D, PER, F, OVF>(a, p, acc, q, k);
  F::finish(acc, p, q);
}

// Queries x[:, qlist[t]] (or t) in the given order: row = t.
template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS, 8)
k_lists_query(const TravArgs<T> a, const typename F::Params p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  Query<T, D> q;
  bool valid = t < a.n_q;
  q.i = valid ? (a.qlist ? a.qlist[t] : (int32_t)t) : -1;
  q.q = (int32_t)t;
  q.k = -1;
  if (valid && (q.i < 0 || q.i >= a.n_x)) {
    set_error(a.err, PN_ERR_INVALID_ARG);
    valid = false;
  }
  int32_t row = 0;
  if (valid) {
#pragma unroll
    for (int k = 0; k < D; ++k) q.x[k] = a.x[(int64_t)q.i * D + k];
    row = a.nb_row_of ? a.nb_row_of[q.i] : q.i;
    q.k = a.nb_row_of ? row : -1;  // the query's own slot, when the rows are slots
  }
  list_query<T, D, PER, F>(a, p, q, row, valid);
}

}  // namespace pn
