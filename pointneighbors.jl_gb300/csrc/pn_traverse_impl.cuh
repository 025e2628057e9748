// pn_traverse_impl.cuh -- host dispatch of foreach_point_neighbor for one coordinate type T
// and pair-arithmetic type V (V = T, or Float32 with Float64 coordinates); included by
// pn_traverse_f32.cu, pn_traverse_f64.cu and pn_traverse_mixed.cu.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <type_traits>

#include "pn_traverse.cuh"

namespace pn {

// Writes PN_ERR_CAPACITY when the neighbour lists do not fit (total read on the device).
static __global__ void k_check_capacity(const int64_t* total, int64_t capacity, int32_t* err) {
  if (*total > capacity) set_error(err, PN_ERR_CAPACITY);
}

// Sorted WCSPH state from user arrays (original order) for a standalone FORCE call
// (coordinates in TP, state in T).
template <typename TP, typename T, int D>
__global__ void __launch_bounds__(256)
k_gather_state(const int32_t* __restrict__ perm, const TP* __restrict__ pos, int32_t n_slots_max,
               const int32_t* __restrict__ n_slots, const T* __restrict__ density,
               const T* __restrict__ pressure, const T* __restrict__ velocity,
               T* __restrict__ pa, T* __restrict__ pb, float4* __restrict__ sdf = nullptr) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_slots_max || k >= *n_slots) return;
  const int32_t i = perm[k];
  if (i < 0) {  // vacated by an incremental update: never a neighbour
    store4(pa, k, V4<T>{(T)NAN, (T)NAN, (T)NAN, (T)0});
    return;
  }
  if (sdf != nullptr) {  // the double-float copy (Float64 3D searches)
    const double rho = (double)density[i];
    const df P = df_from((double)pressure[i] / (rho * rho)), R = df_from(rho);
    df v[3] = {df_make(0.0f), df_make(0.0f), df_make(0.0f)};
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = df_from((double)velocity[(int64_t)i * D + d]);
    sdf[3 * k] = make_float4(P.hi, P.lo, R.hi, R.lo);
    sdf[3 * k + 1] = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
    sdf[3 * k + 2] = make_float4(v[2].hi, v[2].lo, 0.0f, 0.0f);
  }
  TP x[D];
  load_pos<TP, D>(pos, k, x);
  const T rho = density[i];
  V4<T> va{(T)0, (T)0, (T)0, pressure[i] / (rho * rho)};
  V4<T> vb{(T)0, (T)0, (T)0, rho};
  T* xa = &va.x;
  T* xb = &vb.x;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    xa[d] = (T)x[d];
    xb[d] = velocity[(int64_t)i * D + d];
  }
  store4(pa, k, va);
  store4(pb, k, vb);
}

// Adjoint state (x, g = 2 (rho - 1)) in slot order from a density array (original order).
template <typename TP, typename T, int D>
__global__ void __launch_bounds__(256)
k_gather_adjoint(const int32_t* __restrict__ perm, const TP* __restrict__ pos,
                 int32_t n_slots_max, const int32_t* __restrict__ n_slots,
                 const T* __restrict__ density, T* __restrict__ pa) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_slots_max || k >= *n_slots) return;
  const int32_t i = perm[k];
  if (i < 0) {
    store4(pa, k, V4<T>{(T)NAN, (T)NAN, (T)NAN, (T)0});
    return;
  }
  TP x[D];
  load_pos<TP, D>(pos, k, x);
  V4<T> va{(T)0, (T)0, (T)0, (T)2 * (density[i] - (T)1)};
  T* xa = &va.x;
#pragma unroll
  for (int d = 0; d < D; ++d) xa[d] = (T)x[d];
  store4(pa, k, va);
}

// Deterministic FP64 sum of n values: block b sums a fixed contiguous range in a fixed
// order, then one block sums the SUM_BLOCKS partials.
__device__ __forceinline__ double block_sum_f64(double v, double* sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
  return t;  // valid in thread 0
}

template <typename T>
__global__ void __launch_bounds__(256)
k_sum_partials(const T* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double sm[8];
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = (int64_t)blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  double acc = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) acc += (double)v[i];
  const double t = block_sum_f64(acc, sm);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

static __global__ void __launch_bounds__(256)
k_sum_final(const double* __restrict__ part, int n_part, double* __restrict__ out) {
  __shared__ double sm[8];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n_part; i += blockDim.x) acc += part[i];
  const double t = block_sum_f64(acc, sm);
  if (threadIdx.x == 0) *out = t;
}

template <typename P>
static int pc_grow(P** p, int64_t* cap, int64_t need) {
  if (need <= *cap) return PN_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const int64_t n = need + need / 8;
  if (cudaMalloc(p, sizeof(P) * n) != cudaSuccess) {
    cudaGetLastError();
    return PN_ERR_OUT_OF_MEMORY;
  }
  *cap = n;
  return PN_OK;
}

// Storage of the pair cache for n_rows sorted queries: 3^(d-1) stencil rows each.
static int pc_prepare(pn_search* s, int64_t n_rows, MaskParams* m, cudaStream_t st) {
  const int64_t nr = s->ndims == 3 ? 9 : (s->ndims == 2 ? 3 : 1);
  int rc = pc_grow(&s->d_pc_b0, &s->pc_b0_cap, nr * n_rows + 1);
  if (rc == PN_OK) rc = pc_grow(&s->d_pc_mask, &s->pc_mask_cap, 2 * (nr * n_rows + 1));
  if (rc != PN_OK) return rc;
  // overflow lists of a Float32 incremental search: the overflow runs' masks as well
  const bool ovf = s->ovf_active && s->d_xkey != nullptr;
  if (ovf) {
    rc = pc_grow(&s->d_pc_ob0, &s->pc_ob0_cap, nr * n_rows + 1);
    if (rc == PN_OK) rc = pc_grow(&s->d_pc_omask, &s->pc_omask_cap, nr * n_rows + 1);
    if (rc != PN_OK) return rc;
  }
  cudaMemsetAsync(s->d_err + 4, 0, sizeof(int32_t), st);
  *m = MaskParams{s->d_pc_b0, reinterpret_cast<ulonglong2*>(s->d_pc_mask), n_rows,
                  s->d_err + 4, s->d_err,
                  ovf ? s->d_pc_ob0 : nullptr, ovf ? s->d_pc_omask : nullptr,
                  s->d_ovf_start + s->n_total, s->d_start + s->n_total};
  s->pc_rows = n_rows;
  s->pc_ovf = ovf;
  return PN_OK;
}

// Pair functions that only ever run on the cell-sorted queries (MixedFast): the stencil
// traversal, the pair cache's walk and its fallback; the other kernels are not instantiated
// for them.
template <class F>
struct sorted_only { static constexpr bool value = false; };
template <int D, class G>
struct sorted_only<MixedFast<D, G>> { static constexpr bool value = true; };
// Pair functions that never walk a pair cache (Mixed, the Float64 traversal of a mixed
// search's other queries): its walk and fallback kernels are not instantiated for them.
template <class F>
struct never_cached { static constexpr bool value = false; };
template <int D, class G>
struct never_cached<Mixed<D, G>> { static constexpr bool value = true; };

// The pair cache's walk: with overflow masks, also the instance that walks them (each
// instance returns at once unless the device state is its case).  ovf_likely: the last
// update known to the host kept points in overflow lists; the overflow instance then gets
// the full grid, else one wave of blocks (grid-stride), which costs little when it returns
// at once.  Either grid covers every query.
template <typename T, int D, bool PER, class F>
static void launch_masks(const TravArgs<T>& a, const typename F::Params& p, int blocks,
                         cudaStream_t st, bool ovf_likely = false) {
  k_masks_sorted<T, D, PER, F, false><<<blocks, TRAV_THREADS, 0, st>>>(a, p);
  if (a.pc_ob0 != nullptr) {
    if (ovf_likely)
      k_masks_sorted<T, D, PER, F, true, false><<<blocks, TRAV_THREADS, 0, st>>>(a, p);
    else
      k_masks_sorted<T, D, PER, F, true, true>
          <<<std::min(blocks, 152 * trav_blocks<F>::value), TRAV_THREADS, 0, st>>>(a, p);
    count_launch();
  }
}

template <typename T, template <typename, int> class F>
static int launch_trav(const pn_search* s, const TravArgs<T>& a, const typename F<T, 1>::Params& p,
                       bool sorted, int64_t n_launch, cudaStream_t st) {
  const int blocks = div_up(n_launch, TRAV_THREADS);
  if (blocks == 0) return PN_OK;
  const int key = s->ndims * 2 + (s->periodic ? 1 : 0);
#define PN_TRAV_CASE(KEY, DD, PP)                                                       \
  case KEY:                                                                             \
    if constexpr (is_exact64<F<T, DD>>::value) {                                        \
      if constexpr (DD >= 2) {                                                          \
        k_trav_sorted<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p);      \
        count_launch();                                                                 \
      } else {                                                                          \
        return PN_ERR_INVALID_ARG;                                                      \
      }                                                                                 \
    } else if constexpr (sorted_only<F<T, DD>>::value) {                                \
      if (a.pc_mask != nullptr)                                                         \
        launch_masks<T, DD, PP, F<T, DD>>(a, p, blocks, st, s->n_ovf > 0);              \
      else                                                                              \
        k_trav_sorted<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p);      \
      count_launch();                                                                   \
    } else if (a.pc_mask != nullptr && sorted) {                                        \
      if constexpr (!never_cached<F<T, DD>>::value) {                                   \
        launch_masks<T, DD, PP, F<T, DD>>(a, p, blocks, st, s->n_ovf > 0);              \
        count_launch();                                                                 \
      }                                                                                 \
    } else if (a.nb != nullptr) {                                                       \
      if (sorted)                                                                       \
        k_lists_sorted<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p);     \
      else                                                                              \
        k_lists_query<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p);      \
      count_launch();                                                                   \
    } else if (a.hash_cell != nullptr) {                                                \
      if constexpr (!has_row_hook<F<T, DD>>::value) {                                   \
        if (sorted)                                                                     \
          k_trav_hash_sorted<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p); \
        else                                                                            \
          k_trav_hash_list<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p); \
        count_launch();                                                                 \
      }                                                                                 \
    } else if (sorted) {                                                                \
      k_trav_sorted<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p);        \
      count_launch();                                                                   \
    } else {                                                                            \
      k_trav_list<T, DD, PP, F<T, DD>><<<blocks, TRAV_THREADS, 0, st>>>(a, p);          \
      count_launch();                                                                   \
    }                                                                                   \
    break;
  switch (key) {
    PN_TRAV_CASE(2, 1, false)
    PN_TRAV_CASE(3, 1, true)
    PN_TRAV_CASE(4, 2, false)
    PN_TRAV_CASE(5, 2, true)
    PN_TRAV_CASE(6, 3, false)
    PN_TRAV_CASE(7, 3, true)
    default: return PN_ERR_INVALID_ARG;
  }
#undef PN_TRAV_CASE
  if constexpr (never_cached<F<T, 1>>::value || is_exact64<F<T, 1>>::value) {
    return cuda_status(cudaGetLastError());
  } else if ((a.nb != nullptr || a.pc_mask != nullptr) && a.nb_fallback && sorted) {
    // queries the pair cache or the lists could not hold: the stencil traversal, for
    // those only (the full grid's; neither is offered over hash lists)
    TravArgs<T> g = a;
    g.nb = nullptr;
    g.pc_mask = nullptr;
    g.pc_b0 = nullptr;
    g.nb_fallback = 0;
    const int fb = std::min(blocks, 152 * 8);
    switch (key) {
      case 2: k_trav_fallback<T, 1, false, F<T, 1>><<<fb, TRAV_THREADS, 0, st>>>(g, p); break;
      case 3: k_trav_fallback<T, 1, true, F<T, 1>><<<fb, TRAV_THREADS, 0, st>>>(g, p); break;
      case 4: k_trav_fallback<T, 2, false, F<T, 2>><<<fb, TRAV_THREADS, 0, st>>>(g, p); break;
      case 5: k_trav_fallback<T, 2, true, F<T, 2>><<<fb, TRAV_THREADS, 0, st>>>(g, p); break;
      case 6: k_trav_fallback<T, 3, false, F<T, 3>><<<fb, TRAV_THREADS, 0, st>>>(g, p); break;
      default: k_trav_fallback<T, 3, true, F<T, 3>><<<fb, TRAV_THREADS, 0, st>>>(g, p); break;
    }
    count_launch();
  }
  return cuda_status(cudaGetLastError());
}

template <typename T>
static SphConst<T> sph_const(const pn_search* s, const pn_wcsph_params* w) {
  SphConst<T> c{};
  const double h = w->h;
  const double pi = 3.14159265358979323846;
  const double sigma = s->ndims == 3 ? 21.0 / (16.0 * pi * h * h * h)
                     : s->ndims == 2 ? 7.0 / (4.0 * pi * h * h)
                                     : 5.0 / (8.0 * h);
  c.mass = (T)w->mass;
  c.h = (T)h;
  c.inv_h = (T)(1.0 / h);
  c.sigma = (T)sigma;
  c.dw_coef = (T)(-5.0 * sigma / (h * h));
  c.c0 = (T)w->c0;
  c.rho0 = (T)w->rho0;
  c.inv_rho0 = (T)(1.0 / w->rho0);
  c.gamma = (T)w->gamma_exp;
  c.gamma_int = (w->gamma_exp == std::floor(w->gamma_exp) && w->gamma_exp >= 1.0 &&
                 w->gamma_exp <= 64.0) ? (int32_t)w->gamma_exp : 0;
  c.eos_b = (T)(w->c0 * w->c0 * w->rho0 / w->gamma_exp);
  c.alpha = (T)w->alpha;
  c.eps_h2 = (T)(w->eps_visc * h * h);
  c.r_min2 = (T)(w->r_min * w->r_min);
  return c;
}

// Traversal arguments of a search for the queries x[:, points] against y; `sorted`: the
// queries are the cell-sorted slots (x is y, every point binned).
template <typename T>
static TravArgs<T> trav_args(const pn_search* s, const T* x, int64_t n_x, const int32_t* points,
                             int64_t n_q) {
  TravArgs<T> a{};
  a.g = make_grid<T>(s);
  a.start = s->d_start;
  a.ovf_start = s->ovf_active ? s->d_ovf_start : nullptr;
  a.perm = s->d_perm;
  a.cell_of_slot = s->d_cell_of_slot;
  a.pos = static_cast<const T*>(s->d_pos);
  a.x = x;
  a.qlist = points;
  a.n_q = n_q;
  a.n_x = n_x;
  a.err = s->d_err;
  a.bc_slots = slot_capacity(s);
  a.bc_points = s->n_y;
  a.outside = s->d_err + 1;
  a.unsorted = s->d_err + 3;
  a.xkey = s->ovf_active ? s->d_xkey : nullptr;
  a.cell_delta = s->ovf_active ? s->d_cell_delta : nullptr;
  a.delta = reinterpret_cast<const float*>(s->d_err + ERR_DELTA);
  if (s->hashed && !s->hash_dense) {  // the hash lists' traversal
    a.hash_list = s->d_hbucket;
    a.hash_cell = s->d_hcell;
    a.hash_key = s->d_hkey;
    a.hash_mod = hash_mod(s->list_size);
  }
  // hashed cells need not line up with a periodic box's faces: check every image
  if (s->hashed) a.outside = nullptr;
  for (int k = 0; k < 3; ++k)
    a.clip_m[k] = (T)(16.0 * (double)std::numeric_limits<T>::epsilon() *
                      (std::fabs(s->min_pad[k]) + std::fabs(s->max_pad[k]) + s->cell_size[k]));
  {
    // Band around r^2 outside which the FMA distance test is decisive: 32 units in the
    // last place on each side (the two forms differ by at most 6).
    const double u = std::numeric_limits<T>::epsilon() / 2;
    const double r2 = (double)a.g.r2;
    a.r2_lo = (T)(r2 * (1.0 - 32.0 * u));
    a.r2_hi = (T)(r2 * (1.0 + 32.0 * u));
  }
  return a;
}

// ------------------------------------------------------------------ mixed precision
// The Float64 traversal of a Float32 search: its radius is widened past the rounding of the
// reference's Float32 arithmetic.  The Float32 d2 of a pair is within 6 units of 2^-24 of
// the exact squared distance of the Float64 points, plus, after a periodic correction,
// 2^-24 |pos_diff| per component (the Float32 difference is rounded before the box is
// subtracted; |pos_diff| is at most the grid's extent).  The margins below exceed both, so
// every pair the Float32 test accepts is a candidate; Mixed<D, F> decides.
static MixedGeom mixed_geom(const pn_search* s, TravArgs<double>* a) {
  MixedGeom m{};
  const float r = (float)s->radius;
  m.r2 = r * r;
  double rs = (double)r * (1.0 + 1e-5);
  for (int k = 0; k < s->ndims; ++k) {
    m.box[k] = (float)s->box_size[k];
    if (s->periodic) rs += 4.0 * std::ldexp(1.0, -24) * (s->max_pad[k] - s->min_pad[k]);
  }
  m.per = s->periodic;
  m.pos = static_cast<const double*>(s->d_pos);
  m.state = nullptr;
  a->g.r = rs;
  a->g.r2 = rs * rs * (1.0 + 1e-9);
  const double u = std::numeric_limits<double>::epsilon() / 2;
  a->r2_lo = a->g.r2 * (1.0 - 32.0 * u);
  a->r2_hi = a->g.r2 * (1.0 + 32.0 * u);
  return m;
}

// Launch pair function F: F<T, D> itself, or, with Float32 pair arithmetic over Float64
// coordinates, Mixed<D, F<float, D>> with the geometry m.
// Float64 sorted queries without a pair cache to walk take the Float32 traversal `fast64`
// with Exact64<F> when `g64` is given and F is one of exact64_ok's.
// ------------------------------------------------------------------ double-float sums
// A Float64 search's 3D WCSPH sweeps take the double-float sums (DF64) when the three-part
// split of its coordinates is kept (3D, not hashed) and it has no periodic box.
static bool df64_usable(const pn_search* s) {
  return s->d_pos32lo2 != nullptr && s->d_sdf != nullptr && s->ndims == 3 && !s->periodic;
}

static DF64Geom df64_geom(const pn_search* s, const SphConst<double>& c, float* sdf,
                          double rs = 0.0) {
  DF64Geom d{};
  d.xa = s->d_pos32;
  d.xb = s->d_pos32lo;
  d.xc = s->d_pos32lo2;
  d.sdf = reinterpret_cast<float4*>(sdf);
  d.k.inv_h = df_from(c.inv_h);
  d.k.h = df_from(c.h);
  d.k.dw_coef = df_from(c.dw_coef);
  d.k.eps_h2 = df_from(c.eps_h2);
  d.k.m_alpha_c0_h = df_from(-c.alpha * c.c0 * c.h);
  d.k.m_mass = df_from(-c.mass);
  d.k.r_min2 = df_from(c.r_min2);
  const double r2 = s->radius * s->radius;
  d.k.r2_lo = df_from(r2 * (1.0 - 1e-12));
  d.k.r2_hi = df_from(r2 * (1.0 + 1e-12));
  const double r_in = 2.0 * s->radius - rs;  // rs = 0: no Float32 decision
  d.k.r_in2 = rs > 0.0 && r_in > 0.0 ? (float)(r_in * r_in * (1.0 - 1e-6)) : 0.0f;
  return d;
}
// the WCSPH constants and the double-float state: written by a density sweep that keeps
// the sorted state, read by the force
static DF64Geom df64_geom_of(const pn_search* s, const DensityParams<double>& p) {
  return df64_geom(s, p.c, p.pa != nullptr ? s->d_sdf : nullptr);
}
static DF64Geom df64_geom_of(const pn_search* s, const ForceParams<double>& p) {
  return df64_geom(s, p.c, s->d_sdf);
}
template <class P>
static DF64Geom df64_geom_of(const pn_search* s, const MaskPairParams<P>& p) {
  return df64_geom_of(s, p.f);
}

// The double-float sweep: the pair cache's walk (and its stencil fallback) when the cache
// is on, else the stencil traversal; the Float32 traversal arguments of the search.
template <class G>
static int launch_df64(const TravArgs<float>& a, const typename G::Params& p, int64_t n_launch,
                       cudaStream_t st) {
  const int blocks = div_up(n_launch, TRAV_THREADS);
  if (blocks == 0) return PN_OK;
  if (a.pc_mask != nullptr) {
    launch_masks<float, 3, false, G>(a, p, blocks, st);
    count_launch();
    if (a.nb_fallback) {
      TravArgs<float> g = a;
      g.nb = nullptr;
      g.pc_mask = nullptr;
      g.pc_b0 = nullptr;
      g.nb_fallback = 0;
      k_trav_fallback<float, 3, false, G><<<std::min(blocks, 152 * 8), TRAV_THREADS, 0, st>>>(
          g, p);
      count_launch();
    }
  } else {
    k_trav_sorted<float, 3, false, G><<<blocks, TRAV_THREADS, 0, st>>>(a, p);
    count_launch();
  }
  return cuda_status(cudaGetLastError());
}

// the pair-cache fields of a search's traversal arguments, onto its Float32 traversal's
static void copy_cache_args(TravArgs<float>& d, const TravArgs<double>& a) {
  d.pc_b0 = a.pc_b0;
  d.pc_mask = a.pc_mask;
  d.pc_stride = a.pc_stride;
  d.pc_ob0 = a.pc_ob0;
  d.pc_omask = a.pc_omask;
  d.nb_len = a.nb_len;
  d.nb_fallback = a.nb_fallback;
  d.pc_any_fallback = a.pc_any_fallback;
}

template <typename T, typename V, template <typename, int> class F>
static int launch_pair(const pn_search* s, const TravArgs<T>& a, const typename F<V, 1>::Params& p,
                       const MixedGeom& m, bool sorted, int64_t n_launch, cudaStream_t st,
                       const TravArgs<float>* fast = nullptr,
                       const TravArgs<float>* fast64 = nullptr,
                       const Exact64Geom* g64 = nullptr) {
  if constexpr (std::is_same<T, V>::value) {
    (void)m;
    (void)fast;
    if constexpr (std::is_same<T, double>::value && df64_ok<F<double, 3>>::value) {
      if (fast64 != nullptr && g64 != nullptr && sorted && df64_usable(s)) {
        TravArgs<float> a32 = *fast64;
        if (a.pc_mask != nullptr) copy_cache_args(a32, a);
        const DF64Params<typename F<double, 1>::Params> dp{p, *g64, df64_geom_of(s, p)};
        return launch_df64<DF64<3, F<double, 3>>>(a32, dp, n_launch, st);
      }
    }
    if constexpr (std::is_same<T, double>::value && exact64_ok<F<double, 3>>::value) {
      if (fast64 != nullptr && g64 != nullptr && a.pc_mask == nullptr && sorted &&
          s->ndims >= 2) {
        const Exact64Params<typename F<double, 1>::Params> ep{p, *g64};
        return launch_trav<float, Exact64Of<F>::template type>(s, *fast64, ep, sorted,
                                                               n_launch, st);
      }
    }
    (void)fast64;
    (void)g64;
    return launch_trav<T, F>(s, a, p, sorted, n_launch, st);
  } else {
    const MixedParams<typename F<V, 1>::Params> mp{p, m};
    if (fast != nullptr)  // sorted queries: the Float32 traversal
      return launch_trav<float, MixedFastOf<F>::template type>(s, *fast, mp, sorted, n_launch,
                                                                st);
    return launch_trav<T, MixedOf<F>::template type>(s, a, mp, sorted, n_launch, st);
  }
}

// The Float32 traversal of a mixed search's sorted queries: over the Float32 copy of the
// coordinates, with the radius widened past its rounding.  Each rounded coordinate is off by
// at most u |x| (u = 2^-24), so a pos_diff component by at most u (|xi| + |xj| + |pd|); the
// margin below covers that for every coordinate of the grid, plus the periodic correction's
// and the Float32 distance test's own rounding.
static TravArgs<float> mixed_fast_args(const pn_search* s, int64_t n_q) {
  TravArgs<float> a = trav_args<float>(s, nullptr, 0, nullptr, n_q);
  a.pos = s->d_pos32;
  const double u = std::ldexp(1.0, -24);
  double ext = 0.0, box = 0.0;
  for (int k = 0; k < s->ndims; ++k) {
    ext = std::max(ext, std::max(std::fabs(s->min_pad[k]), std::fabs(s->max_pad[k])));
    box += s->box_size[k];
  }
  const double rs = s->radius * (1.0 + 1e-5) +
                    4.0 * std::sqrt((double)s->ndims) * u * (2.0 * ext + 2.0 * s->radius) +
                    4.0 * u * box;
  a.g.r = (float)rs;
  a.g.r2 = (float)(rs * rs * (1.0 + 1e-6));
  const double uf = std::numeric_limits<float>::epsilon() / 2;
  a.r2_lo = (float)((double)a.g.r2 * (1.0 - 32.0 * uf));
  a.r2_hi = (float)((double)a.g.r2 * (1.0 + 32.0 * uf));
  return a;
}

// One foreach_point_neighbor call after its checks: the traversal arguments and the launch
// shape that every pair function uses.
template <typename T>
struct TravCall {
  TravArgs<T> a;
  MixedGeom m;
  bool sorted;    // the queries are the cell-sorted slots (x is y, every point binned)
  bool cache_on;  // the pair cache is walked or built by this call
  int64_t n_q, n_sorted, n_launch;
  bool fast;               // mixed precision, sorted queries: the Float32 traversal a32
  TravArgs<float> a32;
  const TravArgs<float>* fast_args() const { return fast ? &a32 : nullptr; }
  bool fast64;             // Float64, sorted queries: the Float32 traversal a32 + Exact64
  Exact64Geom g64;
  const TravArgs<float>* fast64_args() const { return fast64 ? &a32 : nullptr; }
  const Exact64Geom* geom64() const { return fast64 ? &g64 : nullptr; }
};

// In 3D the WCSPH / adjoint state (x, y, z, aux) has the coordinates' layout: the force and
// backward sweeps read their candidates from it and get aux with the same load.  A mixed
// search's Float32 traversal does the same on its Float32 state; its Float64 traversal (list
// mode) keeps the coordinates as candidates and Mixed loads aux.
template <typename T, typename V>
static void use_state(const pn_search* s, TravArgs<T>& a, MixedGeom& m, TravCall<T>& c,
                      const V* state) {
  if (s->ndims != 3) return;
  if constexpr (std::is_same<T, V>::value) {
    a.pos = state;
    if constexpr (std::is_same<T, double>::value) c.g64.state = state;
  } else if (c.fast) {
    c.a32.pos = state;
  } else {
    m.state = state;
  }
}

// Walk the pair cache (valid since the last density / adjoint-forward sweep).
template <typename T>
static void use_pair_cache(const pn_search* s, TravArgs<T>& a) {
  a.pc_b0 = s->d_pc_b0;
  a.pc_mask = reinterpret_cast<const ulonglong2*>(s->d_pc_mask);
  a.pc_stride = s->pc_rows;
  a.pc_ob0 = s->pc_ovf ? s->d_pc_ob0 : nullptr;
  a.pc_omask = s->pc_ovf ? s->d_pc_omask : nullptr;
  a.nb_len = s->d_pc_b0;  // row 0: negative marks the stencil fallback
  a.nb_fallback = 1;
  a.pc_any_fallback = s->d_err + 4;
}

template <typename T, typename V>
static int prepare_call(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y,
                        const int32_t* points, int64_t n_points, const void* params,
                        const ListsRef* lists, TravCall<T>& c) {
  constexpr bool kMixed = !std::is_same<T, V>::value;
  if (!s->initialized || s->is_template) return PN_ERR_NOT_INITIALIZED;
  if (n_y != s->n_y || n_x < 0 || (points == nullptr && n_points != 0 && n_points != n_x))
    return PN_ERR_INVALID_ARG;
  if (params == nullptr) return PN_ERR_INVALID_ARG;
  c.sorted = (const void*)x == (const void*)y && n_x == n_y && points == nullptr &&
             s->full_binned;
  c.n_q = points ? n_points : n_x;
  c.a = trav_args<T>(s, x, n_x, points, c.n_q);
  c.m = MixedGeom{};
  if constexpr (kMixed) c.m = mixed_geom(s, &c.a);
  if (lists != nullptr) {
    // rows are slots (lists built with x is y) or the points of x
    if (lists->by_slot) {
      if ((const void*)x != (const void*)y || n_x != n_y) return PN_ERR_INVALID_ARG;
      if (!c.sorted) c.a.nb_row_of = lists->row_of;  // a subset of the points
    } else if (c.sorted || n_x != lists->n_rows) {
      return PN_ERR_INVALID_ARG;
    }
    c.a.nb = lists->nb;
    c.a.nb_grp = lists->grp;
    c.a.nb_len = lists->len;
  }
  // Sorted mode launches one thread per possible slot; the kernel reads the live count.
  c.n_sorted = s->ovf_active ? s->n_binned + s->cap : s->n_binned;
  c.n_launch = c.sorted ? c.n_sorted : c.n_q;
  c.fast = kMixed && c.sorted && lists == nullptr && s->d_pos32 != nullptr && !s->hashed;
  c.fast64 = false;
  if constexpr (!kMixed && std::is_same<T, double>::value) {
    c.fast64 = c.sorted && lists == nullptr && s->d_pos32 != nullptr && !s->hashed;
    if (c.fast64) {
      c.a32 = mixed_fast_args(s, c.n_q);  // Float32 coordinates, radius widened past them
      c.g64 = Exact64Geom{c.a.g, static_cast<const double*>(s->d_pos), nullptr,
                          s->periodic, 0};
    }
  }
  // the pair cache, on the Float32 traversal for a mixed search
  c.cache_on = (!kMixed || c.fast) && (!s->hashed || s->hash_dense) && lists == nullptr &&
               c.sorted && s->pc_cap > 0;
  if (c.fast) {
    c.a32 = mixed_fast_args(s, c.n_q);
    c.m.hi = s->d_pos32;
    c.m.lo = s->d_pos32lo;
    // ex - ey and the rounding of t + p + q: a few units of 2^-48 of the coordinates
    double ext = 0.0;
    for (int k = 0; k < s->ndims; ++k)
      ext = std::max(ext, std::max(std::fabs(s->min_pad[k]), std::fabs(s->max_pad[k])));
    c.m.eb = (float)(std::ldexp(1.0, -44) * (ext + s->radius));
  }
  if (c.cache_on && s->pc_valid) {
    if (c.fast) use_pair_cache(s, c.a32);
    else use_pair_cache(s, c.a);
  }
  return PN_OK;
}

// The WCSPH and adjoint pair functions; defined in pn_traverse_sph.cuh and compiled in
// translation units of their own (the kernels of one element type in two halves).
template <typename T, typename V>
int foreach_sph(pn_search* s, int32_t functor, int64_t n_x, const void* params,
                TravCall<T>& c, cudaStream_t st);

template <typename T, typename V>
static int foreach_t(pn_search* s, int32_t functor, const T* x, int64_t n_x, const T* y,
                     int64_t n_y, const int32_t* points, int64_t n_points, const void* params,
                     cudaStream_t st, const ListsRef* lists) {
  TravCall<T> c;
  const int rc0 = prepare_call<T, V>(s, x, n_x, y, n_y, points, n_points, params, lists, c);
  if (rc0 != PN_OK) return rc0;
  TravArgs<T>& a = c.a;
  const MixedGeom& m = c.m;
  const bool sorted = c.sorted;
  const int64_t n_q = c.n_q, n_launch = c.n_launch;
  switch (functor) {
    case PN_F_COUNT: {
      const auto* u = static_cast<const pn_count_params*>(params);
      CountParams<V> p{u->counts, 0};
      return launch_pair<T, V, FCount>(s, a, p, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
    }
    case PN_F_INDEX_SUM: {
      const auto* u = static_cast<const pn_index_sum_params*>(params);
      IndexSumParams<V> p{u->sums, s->d_perm};
      return launch_pair<T, V, FIndexSum>(s, a, p, m, sorted, n_launch, st,
                                           c.fast_args(), c.fast64_args(), c.geom64());
    }
    case PN_F_NEIGHBOR_LIST: {
      const auto* u = static_cast<const pn_neighbor_list_params*>(params);
      if (u->offsets == nullptr) return PN_ERR_INVALID_ARG;
      int32_t* counts = u->counts;
      if (counts == nullptr) {
        int rc = ensure_qcount(s, n_q);
        if (rc != PN_OK) return rc;
        counts = s->d_qcount;
      }
      CountParams<V> pc{counts, 1};
      int rc = launch_pair<T, V, FCount>(s, a, pc, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
      if (rc != PN_OK) return rc;
      rc = scan64(s, counts, n_q, u->offsets, st);
      if (rc != PN_OK) return rc;
      // Without an output buffer the call only counts (the caller sizes the buffer from
      // offsets[n_q]); with one, rows are written only if they all fit.
      if (u->neighbors == nullptr || u->capacity <= 0) return cuda_status(cudaGetLastError());
      k_check_capacity<<<1, 1, 0, st>>>(u->offsets + n_q, u->capacity, s->d_err); count_launch();
      EmitParams<V> pe{u->offsets, u->neighbors, s->d_perm, u->capacity, n_q};
      rc = launch_pair<T, V, FEmit>(s, a, pe, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
      if (rc != PN_OK) return rc;
      if (u->sort_rows) rc = sort_rows(s, u->offsets, n_q, u->neighbors, u->capacity, st);
      return rc;
    }
    case PN_F_NBODY_ACCEL: {
      const auto* u = static_cast<const pn_nbody_params*>(params);
      const V eps_v = std::numeric_limits<V>::epsilon();
      NBodyParams<V> p{static_cast<const V*>(u->masses), s->d_perm, (V)u->G, std::sqrt(eps_v),
                       static_cast<V*>(u->accel)};
      return launch_pair<T, V, FNBody>(s, a, p, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
    }
    case PN_F_POTENTIAL: {
      const auto* u = static_cast<const pn_potential_params*>(params);
      if ((const void*)x != (const void*)y) return PN_ERR_INVALID_ARG;
      PotentialParams<V> p{static_cast<const V*>(u->masses), s->d_perm, (V)u->cutoff,
                           (V)(1.0 / u->cutoff), static_cast<V*>(u->energy), (V)u->cutoff * (V)u->cutoff};
      return launch_pair<T, V, FPotential>(s, a, p, m, sorted, n_launch, st,
                                            c.fast_args(), c.fast64_args(), c.geom64());
    }
    default:
      return foreach_sph<T, V>(s, functor, n_x, params, c, st);
  }
}

template <typename T>
int foreach(pn_search* s, int32_t functor, const T* x, int64_t n_x, const T* y, int64_t n_y,
            const int32_t* points, int64_t n_points, const void* params, cudaStream_t st,
            const ListsRef* lists) {
  if constexpr (std::is_same<T, double>::value) {
    if (s->mixed)
      return foreach_mixed(s, functor, x, n_x, y, n_y, points, n_points, params, st, lists);
  }
  return foreach_t<T, T>(s, functor, x, n_x, y, n_y, points, n_points, params, st, lists);
}

// ------------------------------------------------------------------ precomputed lists
template <typename T, typename V>
static int lists_count_t(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y,
                         int32_t* len, int32_t* by_slot, int64_t* n_rows, cudaStream_t st) {
  if (!s->initialized || s->is_template) return PN_ERR_NOT_INITIALIZED;
  if (n_y != s->n_y || n_x < 0) return PN_ERR_INVALID_ARG;
  const bool sorted = (const void*)x == (const void*)y && n_x == n_y && s->full_binned;
  TravArgs<T> a = trav_args<T>(s, x, n_x, nullptr, n_x);
  MixedGeom m{};
  if constexpr (!std::is_same<T, V>::value) m = mixed_geom(s, &a);
  const int64_t n_sorted = s->ovf_active ? s->n_binned + s->cap : s->n_binned;
  *by_slot = sorted ? 1 : 0;
  *n_rows = sorted ? n_sorted : n_x;
  if (sorted) cudaMemsetAsync(len, 0, sizeof(int32_t) * n_sorted, st);  // vacated slots
  CountParams<V> p{len, sorted ? 2 : 1};
  return launch_pair<T, V, FCount>(s, a, p, m, sorted, *n_rows, st);
}

template <typename T, typename V>
static int lists_emit_t(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y,
                        int32_t* nb, const int64_t* grp, int32_t cap, int32_t* len,
                        cudaStream_t st) {
  if (!s->initialized || s->is_template) return PN_ERR_NOT_INITIALIZED;
  if (n_y != s->n_y || n_x < 0) return PN_ERR_INVALID_ARG;
  const bool sorted = (const void*)x == (const void*)y && n_x == n_y && s->full_binned;
  TravArgs<T> a = trav_args<T>(s, x, n_x, nullptr, n_x);
  MixedGeom m{};
  if constexpr (!std::is_same<T, V>::value) m = mixed_geom(s, &a);
  const int64_t n_sorted = s->ovf_active ? s->n_binned + s->cap : s->n_binned;
  if (len != nullptr && sorted) cudaMemsetAsync(len, 0, sizeof(int32_t) * n_sorted, st);
  EmitListParams<V> p{nb, grp, sorted ? 1 : 0, (cap + 3) & ~3, cap, len, s->d_err};
  return launch_pair<T, V, FEmitList>(s, a, p, m, sorted, sorted ? n_sorted : n_x, st);
}

template <typename T>
int lists_count(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y, int32_t* len,
                int32_t* by_slot, int64_t* n_rows, cudaStream_t st) {
  if constexpr (std::is_same<T, double>::value) {
    if (s->mixed) return lists_count_mixed(s, x, n_x, y, n_y, len, by_slot, n_rows, st);
  }
  return lists_count_t<T, T>(s, x, n_x, y, n_y, len, by_slot, n_rows, st);
}

template <typename T>
int lists_emit(pn_search* s, const T* x, int64_t n_x, const T* y, int64_t n_y, int32_t* nb,
               const int64_t* grp, int32_t cap, int32_t* len, cudaStream_t st) {
  if constexpr (std::is_same<T, double>::value) {
    if (s->mixed) return lists_emit_mixed(s, x, n_x, y, n_y, nb, grp, cap, len, st);
  }
  return lists_emit_t<T, T>(s, x, n_x, y, n_y, nb, grp, cap, len, st);
}

}  // namespace pn
