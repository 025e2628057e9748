// pn_internal.cuh -- device-side building blocks shared by the build, update and
// traversal kernels of libpn_gb300.
//
// Floating-point rules follow the reference (Julia, no fast-math): the arithmetic that
// decides cell membership and neighbour sets uses explicitly rounded intrinsics
// (__fsub_rn/__fmul_rn/__fadd_rn/__fdiv_rn and the double forms) so nvcc cannot contract
// a*b+c into an FMA or substitute an approximate divide.  Pair functions (the physics)
// are free to use fast math: only their sums are compared, within a tolerance.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pn_gb300.h"

namespace pn {

// ------------------------------------------------------------------ exact arithmetic
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float xfloor(float a) { return floorf(a); }
__device__ __forceinline__ double xfloor(double a) { return floor(a); }
__device__ __forceinline__ float xrint(float a) { return rintf(a); }
__device__ __forceinline__ double xrint(double a) { return rint(a); }

// Julia Int64 arithmetic wraps around.
__host__ __device__ __forceinline__ int64_t wadd(int64_t a, int64_t b) {
  return (int64_t)((uint64_t)a + (uint64_t)b);
}
__host__ __device__ __forceinline__ int64_t wsub(int64_t a, int64_t b) {
  return (int64_t)((uint64_t)a - (uint64_t)b);
}
// Julia `mod(x, n)` for n > 0.
__host__ __device__ __forceinline__ int64_t jl_mod(int64_t x, int64_t n) {
  int64_t r = x % n;
  if (r != 0 && ((r < 0) != (n < 0))) r += n;
  return r;
}

// util.jl:19-34 floor_to_int: saturating floor (NaN and >= 2^63 -> typemax).
template <typename T>
__device__ __forceinline__ int64_t floor_to_int(T x) {
  const T r = xfloor(x);
  if (isnan(r) || r >= (T)9223372036854775808.0) return INT64_MAX;
  if (r <= -(T)9223372036854775808.0) return INT64_MIN;
  return (int64_t)r;
}

// ------------------------------------------------------------------ grid description
// Storage stride (in T) of one point in the cell-sorted coordinate array: 3D points are
// padded to 4 components so that a point is one 16-byte (float) / 32-byte (double) load.
template <int D>
struct PS {
  static constexpr int value = (D == 3) ? 4 : D;
};

template <typename T>
struct GridDev {
  int32_t n[3];        // padded FullGridCellList size per dimension
  int32_t ncell[3];    // periodic cells per dimension (0 when not periodic)
  int32_t n_total;     // prod(n), or the hash lists of a SpatialHashingCellList
  int32_t hashed;      // SpatialHashingCellList: cells floor(x / cell_size), no offset
  int32_t cell_off[3]; // SpatialHashingCellList in a dense grid: grid index = cell + cell_off
  int32_t pad_;
  T min_pad[3];        // padded min corner (cell (1,1,1) starts here)
  T cell_size[3];
  T box_min[3], box_max[3];  // periodic box corners
  T box_size[3];       // periodic box size
  T half_box[3];       // box_size / 2
  T r, r2;             // search radius and r*r (both in T)
};

// nhs_grid.jl:622-638 + full_grid.jl:84-94: the reference's cell coordinates, exactly,
// for arbitrary inputs (saturation and Int64 wrap-around included).
template <typename T, int D>
__device__ __forceinline__ void cell_coords_exact(const GridDev<T>& g, bool periodic,
                                                  const T* x, int64_t* c) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const T q = g.hashed ? xdiv(x[k], g.cell_size[k])
                         : xdiv(xsub(x[k], g.min_pad[k]), g.cell_size[k]);
    int64_t ck = wadd(floor_to_int(q), g.hashed ? 0 : 1);
    if (periodic) ck = wadd(jl_mod(wsub(ck, 2), (int64_t)g.ncell[k]), 2);
    c[k] = ck;
  }
}

// Fast form used by the kernels: the 1-based cell coordinate of one dimension as int32,
// and whether it is a valid cell (2 <= c <= n-1, full_grid.jl:205-212).  Identical to
// cell_coords_exact for every input: the saturated cases all fall outside the grid, or
// take the int64 path in the periodic case.
template <typename T>
__device__ __forceinline__ bool cell_coord_1d(const GridDev<T>& g, bool periodic, int k,
                                              T xk, int32_t& c) {
  const T q = xdiv(xsub(xk, g.min_pad[k]), g.cell_size[k]);
  const T fl = xfloor(q);
  if (!periodic) {
    // c = fl + 1 in 2..n-1  <=>  1 <= fl <= n-2 (false for NaN)
    const bool ok = (fl >= (T)1) && (fl <= (T)(g.n[k] - 2));
    c = ok ? (int32_t)fl + 1 : 0;
    return ok;
  }
  const int64_t nc = g.ncell[k];
  int64_t m;
  if (fl >= (T)-4611686018427387904.0 && fl <= (T)4611686018427387904.0) {
    m = (int64_t)fl - 1;  // (fl + 1) - 2, no overflow in this range
    if (m < 0 && m >= -nc) m += nc;
    else if (m >= nc && m < 2 * nc) m -= nc;
    else if (m < 0 || m >= nc) m = jl_mod(m, nc);
  } else {
    m = jl_mod(wsub(wadd(floor_to_int(q), 1), 2), nc);
  }
  // periodic cells are 2..ncell+1; check_cell_bounds still applies (full_grid.jl:205-212)
  c = (int32_t)(m + 2);
  return c <= g.n[k] - 1;
}

// SpatialHashingCellList cell coordinate (nhs_grid.jl:636-638): floor(x / cell_size), with
// a periodic box mod(c - 2, n_cells) + 2.  False when the cell or one of its neighbours
// would leave Int32 (the reference's InexactError in coordinates_flattened) or x is NaN.
template <typename T>
__device__ __forceinline__ bool hash_cell_1d(const GridDev<T>& g, bool periodic, int k, T xk,
                                             int32_t& c) {
  const T q = xdiv(xk, g.cell_size[k]);
  if (!periodic) {
    const double fl = (double)xfloor(q);
    const bool ok = fl >= -2147483647.0 && fl <= 2147483646.0;  // false for NaN
    c = ok ? (int32_t)fl : 0;
    return ok;
  }
  c = (int32_t)(jl_mod(wsub(floor_to_int(q), 2), (int64_t)g.ncell[k]) + 2);
  return !(xk != xk);
}

// The number of hash lists with its reciprocal magic = floor((2^64 - 1) / size), so that
// x mod size is one high multiply, one multiply and at most two corrections (the estimate
// floor(x magic / 2^64) is at most 2 below floor(x / size) for x < 2^64, size < 2^31).
struct HashMod {
  int64_t size;
  uint64_t magic;
};
inline HashMod hash_mod(int64_t size) {
  return HashMod{size, size > 0 ? ~0ull / (uint64_t)size : 0ull};
}

// spatial_hash (spatial_hashing.jl:142-156, Ihmsen et al.): Int64 products and xor that
// wrap around like Julia's, then Julia's mod(h, list_size) (non-negative); 0-based.
template <int D>
__device__ __forceinline__ int32_t spatial_hash(const int32_t* c, const HashMod& hm) {
  uint64_t h = (uint64_t)(int64_t)c[0] * 73856093ull;
  if (D >= 2) h ^= (uint64_t)(int64_t)c[1] * 19349663ull;
  if (D >= 3) h ^= (uint64_t)(int64_t)c[2] * 83492791ull;
  const bool neg = (int64_t)h < 0;
  const uint64_t ax = neg ? 0ull - h : h;  // |h|, 2^63 for typemin
  const uint64_t sz = (uint64_t)hm.size;
  uint64_t r = ax - __umul64hi(ax, hm.magic) * sz;
  if (r >= sz) r -= sz;
  if (r >= sz) r -= sz;
  return (int32_t)(neg && r != 0 ? sz - r : r);
}

// A point outside the periodic box [min, max) (the periodic traversal then checks every
// candidate for a periodic image; inside the box it can skip that check in the interior).
template <typename T>
__device__ __forceinline__ bool outside_box(const GridDev<T>& g, int k, T xk) {
  return !(xk >= g.box_min[k] && xk < g.box_max[k]);
}

// ------------------------------------------------------------------ errors
// Sticky per-search error word: the first error code set by any kernel wins.
__device__ __forceinline__ void set_error(int32_t* err, int32_t code) {
  if (*(volatile int32_t*)err == 0) atomicCAS(err, 0, code);
}

// Bounds-checked builds (-DPN_BOUNDS_CHECK, libpn_gb300_bc.so): PN_IDX(err, site, i, n)
// checks 0 <= i < n before an index reaches memory.  Outside that range the first failure's
// site and index are kept in err[ERR_BC_SITE] and err[ERR_BC_INDEX], the sticky error
// becomes PN_ERR_INDEX, and the access goes to element 0 instead (every checked array has an
// element 0), so a checked run reports the bad index rather than faulting.  In the normal
// build PN_IDX is the index itself.
enum BoundsSite : int32_t {
  BC_QUERY_SLOT = 1,     // a cell-sorted query slot
  BC_CELL = 2,           // a linear cell index (cell starts, counts)
  BC_RUN = 3,            // a candidate run [begin, end) of slots
  BC_POINT = 4,          // a point index read from perm (outputs, per-point inputs)
  BC_PAIR_CACHE = 5,     // a pair-cache entry (row, slot)
  BC_SLOT = 6,           // a slot written by the build (scatter, movers)
  BC_NEIGHBOUR = 7,      // a neighbour slot taken from the pair cache
};
constexpr int ERR_BC_SITE = 8, ERR_BC_INDEX = 9, ERR_WORDS = 16;
// err word (as Float32 bits): the largest |x - xkey| of a main slot after an incremental
// update that kept overflow lists (0 after a build or rebuild)
constexpr int ERR_DELTA = 10;

static __device__ __noinline__ void bounds_failure(int32_t* err, int32_t site, int64_t i) {
  if (err == nullptr) return;  // a kernel launched without an error word
  if (atomicCAS(err + ERR_BC_SITE, 0, site) == 0) err[ERR_BC_INDEX] = (int32_t)i;
  set_error(err, PN_ERR_INDEX);
}

template <typename I>
__device__ __forceinline__ I bc_index(int32_t* err, int32_t site, I i, int64_t n) {
  if ((int64_t)i < 0 || (int64_t)i >= n) {
    bounds_failure(err, site, (int64_t)i);
    return (I)0;
  }
  return i;
}

#ifdef PN_BOUNDS_CHECK
#define PN_IDX(err, site, i, n) ::pn::bc_index((err), (site), (i), (int64_t)(n))
// a run [b, e) of an array of n elements: an empty run when it does not fit
#define PN_RUN(err, b, e, n)                                                         \
  do {                                                                               \
    if ((e) > (b) && ((int64_t)(b) < 0 || (int64_t)(e) > (int64_t)(n))) {           \
      ::pn::bounds_failure((err), ::pn::BC_RUN, (int64_t)(b));                       \
      (e) = (b);                                                                     \
    }                                                                                \
  } while (0)
#else
#define PN_IDX(err, site, i, n) (i)
#define PN_RUN(err, b, e, n) \
  do {                       \
  } while (0)
#endif

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ------------------------------------------------------------------ launch helpers
inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace pn

// ------------------------------------------------------------------ host -> device grid
#include "pn_host.h"

namespace pn {

template <typename T>
inline GridDev<T> make_grid(const pn_search* s) {
  GridDev<T> g{};
  g.n_total = s->n_total;
  g.hashed = s->hashed;
  for (int k = 0; k < 3; ++k) g.cell_off[k] = s->hash_off[k];
  for (int k = 0; k < 3; ++k) {
    const bool used = k < s->ndims;
    g.n[k] = used ? (int32_t)s->grid_size[k] : 1;
    g.ncell[k] = (used && s->periodic) ? (int32_t)s->n_cells[k] : 0;
    g.min_pad[k] = used ? (T)s->min_pad[k] : (T)0;
    g.cell_size[k] = used ? (T)s->cell_size[k] : (T)1;
    g.box_size[k] = used && s->periodic ? (T)s->box_size[k] : (T)0;
    g.box_min[k] = used && s->periodic ? (T)s->cfg.periodic_min[k] : (T)0;
    g.box_max[k] = used && s->periodic ? (T)s->cfg.periodic_max[k] : (T)0;
    g.half_box[k] = g.box_size[k] / (T)2;
  }
  g.r = (T)s->radius;
  g.r2 = g.r * g.r;
  return g;
}

}  // namespace pn
