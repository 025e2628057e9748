// pn_traverse.cuh -- neighbour traversal (foreach_point_neighbor) and its pair functions.
//
// Reference: neighborhood_search.jl:183-234 launches one thread per query point, which
// loops over the 3^d cells around its own cell (nhs_grid.jl:519-583) and gathers the
// neighbours' coordinates through the cell list's Int32 index columns.
//
// Here the candidates come from the cell-sorted coordinate copy: since cells are numbered
// column-major, the three cells (x-1, x, x+1) of one row of the stencil are one contiguous
// slot range, so a query walks 3^(d-1) contiguous ranges.  Query threads are taken in
// cell-sorted order (when x is y), so the lanes of a warp share their rows and the
// candidate loads are broadcast / L1 hits.  Candidates are visited in the reference's order
// (CartesianIndices over the 3^d cells, first dimension fastest; inside a cell by point
// index), so every sum is accumulated in a fixed, reproducible order.
//
// The distance test restates the reference bit for bit: pos_diff = xi - yj in T,
// d2 = ((pd1*pd1 + pd2*pd2) + pd3*pd3) without contraction, and with a periodic box,
// when d2 > r^2, pos_diff -= size .* round.(pos_diff ./ size) and d2 is recomputed
// (neighborhood_search.jl:428-436).  The correction is skipped when every |pos_diff_k| is
// below size_k/2: round() is then 0 and the correction is exactly the identity.
#pragma once

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
  int32_t* err;
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

__device__ __forceinline__ float fsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double fsqrt(double a) { return sqrt(a); }

// ================================================================== pair functions
// A functor provides Params, Acc, init(acc, p, query), pair(acc, p, query, slot, pd, d2),
// finish(acc, p, query) and fail(p, query) (a rejected query: write the empty result where
// later passes depend on it).  `slot` indexes the cell-sorted arrays.

template <typename T> struct CountParams { int32_t* counts; int32_t by_row; };
template <typename T> struct IndexSumParams { int64_t* sums; const int32_t* perm; };
template <typename T> struct EmitParams {
  const int64_t* offsets; int32_t* nbrs; const int32_t* perm; int64_t capacity; int64_t n_rows;
};
template <typename T> struct NBodyParams { const T* masses; const int32_t* perm; T G; T sqrt_eps; T* accel; };
template <typename T> struct PotentialParams { const T* masses; const int32_t* perm; T cutoff, inv_cutoff; T* energy; };

template <typename T, int D>
struct FCount {
  using Params = CountParams<T>;
  struct Acc { int32_t n; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) { a.n = 0; }
  static __device__ __forceinline__ void pair(Acc& a, const Params&, const Query<T, D>&, int32_t,
                                              const T*, T) { ++a.n; }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    p.counts[p.by_row ? q.q : q.i] = a.n;
  }
  static __device__ __forceinline__ void fail(const Params& p, const Query<T, D>& q) {
    if (p.by_row) p.counts[q.q] = 0;
  }
};

template <typename T, int D>
struct FIndexSum {
  using Params = IndexSumParams<T>;
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { int64_t s; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) { a.s = 0; }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T*, T) { a.s += (int64_t)__ldg(&p.perm[js]) + 1; }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
    p.sums[q.i] = a.s;
  }
};

template <typename T, int D>
struct FEmit {
  using Params = EmitParams<T>;
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
                                              const T*, T) {
    if (a.o < a.end) p.nbrs[a.o++] = __ldg(&p.perm[js]);
  }
  static __device__ __forceinline__ void finish(Acc&, const Params&, const Query<T, D>&) {}
};

// benchmarks/n_body.jl:41-56
template <typename T, int D>
struct FNBody {
  using Params = NBodyParams<T>;
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T a[D]; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) {
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] = (T)0;
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T* pd, T d2) {
    const T r = fsqrt(d2);
    if (r < p.sqrt_eps) return;
    const T s = -p.G * __ldg(&p.masses[__ldg(&p.perm[js])]) / (r * r * r);
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
  using Params = PotentialParams<T>;
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T e; T mi; };
  static __device__ __forceinline__ void init(Acc& a, const Params& p, const Query<T, D>& q) {
    a.e = (T)0;
    a.mi = p.masses[q.i];
  }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T*, T d2) {
    const T r = fsqrt(d2);
    if (r > (T)0 && r < p.cutoff)
      a.e += __ldg(&p.masses[__ldg(&p.perm[js])]) * ((T)1 / r - p.inv_cutoff);
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
  using Params = DensityParams<T>;
  static __device__ __forceinline__ void fail(const Params&, const Query<T, D>&) {}
  struct Acc { T w; };
  static __device__ __forceinline__ void init(Acc& a, const Params&, const Query<T, D>&) { a.w = (T)0; }
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t,
                                              const T*, T d2) {
    const T q = fsqrt(d2) * p.c.inv_h;
    if (q < (T)2) {
      const T t = (T)1 - (T)0.5 * q;
      const T t2 = t * t;
      a.w += t2 * t2 * ((T)2 * q + (T)1);
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
};

template <typename T, int D>
struct FForce {
  using Params = ForceParams<T>;
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
  static __device__ __forceinline__ void pair(Acc& a, const Params& p, const Query<T, D>&, int32_t js,
                                              const T* pd, T d2) {
    if (d2 < p.c.r_min2) return;
    const V4<T> sa = load4(p.pa, js);
    const V4<T> sb = load4(p.pb, js);
    const T vj[3] = {sb.x, sb.y, sb.z};
    const T r = fsqrt(d2);
    const T q = r * p.c.inv_h;
    if (!(q < (T)2)) return;
    const T t = (T)1 - (T)0.5 * q;
    const T gw = p.c.dw_coef * t * t * t;  // grad W = gw * pd
    T vr = (T)0;
#pragma unroll
    for (int k = 0; k < D; ++k) vr += (a.vi[k] - vj[k]) * pd[k];
    T visc = (T)0;
    if (vr < (T)0) {
      const T mu = p.c.h * vr / (d2 + p.c.eps_h2);
      visc = -p.c.alpha * p.c.c0 * mu / ((T)0.5 * (a.rhoi + sb.w));
    }
    const T s = -p.c.mass * (a.Pi + sa.w + visc) * gw;
#pragma unroll
    for (int k = 0; k < D; ++k) a.a[k] += s * pd[k];
  }
  static __device__ __forceinline__ void finish(Acc& a, const Params& p, const Query<T, D>& q) {
#pragma unroll
    for (int k = 0; k < D; ++k) p.accel[(int64_t)q.i * D + k] = a.a[k];
  }
};

// ================================================================== traversal kernel
__device__ __forceinline__ int32_t pwrap(int32_t c, int32_t nc) {
  return c < 2 ? c + nc : (c > nc + 1 ? c - nc : c);
}

template <typename T, int D, bool PER, class F>
__device__ __forceinline__ void scan_range(const TravArgs<T>& a, const typename F::Params& p,
                                           typename F::Acc& acc, const Query<T, D>& q,
                                           int32_t beg, int32_t end) {
  const GridDev<T>& g = a.g;
  for (int32_t js = beg; js < end; ++js) {
    T yj[D];
    load_pos<T, D>(a.pos, js, yj);
    T pd[D];
    pd[0] = xsub(q.x[0], yj[0]);
    T d2 = xmul(pd[0], pd[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) {
      pd[k] = xsub(q.x[k], yj[k]);
      d2 = xadd(d2, xmul(pd[k], pd[k]));
    }
    if (PER && d2 > g.r2) {
      bool wrap = false;
#pragma unroll
      for (int k = 0; k < D; ++k) wrap |= !(fabs(pd[k]) < g.half_box[k]);
      if (wrap) {
#pragma unroll
        for (int k = 0; k < D; ++k)
          pd[k] = xsub(pd[k], xmul(g.box_size[k], xrint(xdiv(pd[k], g.box_size[k]))));
        d2 = xmul(pd[0], pd[0]);
#pragma unroll
        for (int k = 1; k < D; ++k) d2 = xadd(d2, xmul(pd[k], pd[k]));
      }
    }
    if (d2 <= g.r2) F::pair(acc, p, q, js, pd, d2);
  }
}

// The 3^d stencil around cell c (1-based coordinates), rows of three cells along x.
template <typename T, int D, bool PER, class F>
__device__ __forceinline__ void visit_stencil(const TravArgs<T>& a, const typename F::Params& p,
                                              typename F::Acc& acc, const Query<T, D>& q,
                                              const int32_t* c) {
  const GridDev<T>& g = a.g;
  constexpr int OZ = D == 3 ? 1 : 0;
  constexpr int OY = D >= 2 ? 1 : 0;
  const bool x_contig = !PER || (c[0] >= 3 && c[0] <= g.ncell[0]);
#pragma unroll 1
  for (int oz = -OZ; oz <= OZ; ++oz) {
    int32_t rowz = 0;
    if (D == 3) {
      const int32_t cz = PER ? pwrap(c[2] + oz, g.ncell[2]) : c[2] + oz;
      rowz = (cz - 1) * g.n[0] * g.n[1];
    }
#pragma unroll 1
    for (int oy = -OY; oy <= OY; ++oy) {
      int32_t row = rowz;
      if (D >= 2) {
        const int32_t cy = PER ? pwrap(c[1] + oy, g.ncell[1]) : c[1] + oy;
        row += (cy - 1) * g.n[0];
      }
      if (x_contig) {
        const int32_t l0 = row + c[0] - 2;
        scan_range<T, D, PER, F>(a, p, acc, q, __ldg(&a.start[l0]), __ldg(&a.start[l0 + 3]));
        if (a.ovf_start)
          scan_range<T, D, PER, F>(a, p, acc, q, __ldg(&a.ovf_start[l0]), __ldg(&a.ovf_start[l0 + 3]));
      } else {
#pragma unroll 1
        for (int ox = -1; ox <= 1; ++ox) {
          const int32_t l = row + pwrap(c[0] + ox, g.ncell[0]) - 1;
          scan_range<T, D, PER, F>(a, p, acc, q, __ldg(&a.start[l]), __ldg(&a.start[l + 1]));
          if (a.ovf_start)
            scan_range<T, D, PER, F>(a, p, acc, q, __ldg(&a.ovf_start[l]), __ldg(&a.ovf_start[l + 1]));
        }
      }
    }
  }
}

// Sorted mode: queries are the cell-sorted slots (x is y, every point binned).  Slots
// [0, start[n_total]) are the main structure, then the overflow slots up to
// ovf_start[n_total]; vacated slots (perm < 0) are skipped.
template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS)
k_trav_sorted(const TravArgs<T> a, const typename F::Params p) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t n_slots = a.ovf_start ? a.ovf_start[a.g.n_total] : a.start[a.g.n_total];
  if (k >= n_slots) return;
  Query<T, D> q;
  q.i = a.perm[k];
  if (q.i < 0) return;
  q.q = q.i;
  q.k = (int32_t)k;
  load_pos<T, D>(a.pos, k, q.x);
  const int32_t lin = a.cell_of_slot[k];
  int32_t c[3] = {1, 1, 1};
  c[0] = lin % a.g.n[0] + 1;
  if (D >= 2) c[1] = (lin / a.g.n[0]) % a.g.n[1] + 1;
  if (D == 3) c[2] = lin / (a.g.n[0] * a.g.n[1]) + 1;
  typename F::Acc acc;
  F::init(acc, p, q);
  visit_stencil<T, D, PER, F>(a, p, acc, q, c);
  F::finish(acc, p, q);
}

// List mode: queries are x[:, qlist[q]] (or q) in the given order.  A query whose
// neighbouring cells fall outside the grid is the reference's BoundsError.
template <typename T, int D, bool PER, class F>
__global__ void __launch_bounds__(TRAV_THREADS)
k_trav_list(const TravArgs<T> a, const typename F::Params p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n_q) return;
  Query<T, D> q;
  q.i = a.qlist ? a.qlist[t] : (int32_t)t;
  q.q = (int32_t)t;
  q.k = -1;
  if (q.i < 0 || q.i >= a.n_x) {
    set_error(a.err, PN_ERR_INVALID_ARG);
    F::fail(p, q);
    return;
  }
  bool ok = true;
  int32_t c[3] = {1, 1, 1};
#pragma unroll
  for (int k = 0; k < D; ++k) {
    q.x[k] = a.x[(int64_t)q.i * D + k];
    ok &= cell_coord_1d(a.g, PER, k, q.x[k], c[k]);
  }
  if (!ok) {
    set_error(a.err, PN_ERR_BOUNDS);
    F::fail(p, q);
    return;
  }
  typename F::Acc acc;
  F::init(acc, p, q);
  visit_stencil<T, D, PER, F>(a, p, acc, q, c);
  F::finish(acc, p, q);
}

}  // namespace pn
