/*
 * pn_oracle_body.h -- body of the CPU restatement, included twice by pn_oracle.c with
 * T = float / double and S = f32 / f64.  TEST INFRASTRUCTURE ONLY (see pn_oracle.h).
 *
 * Floating-point rules follow Julia: no contraction of a*b+c (this file is compiled with
 * -ffp-contract=off), StaticArrays `dot` as ((a1*b1 + a2*b2) + a3*b3), IEEE division and
 * sqrt, `round` = ties-to-even (rint), `floor` before the saturating Int conversion.
 * Integer arithmetic on cell coordinates wraps like Julia's Int64.
 */
#define FN(name) PNO_CAT(name, S)

/* util.jl:19-34 floor_to_int: saturating floor.  Julia compares a Float with
 * typemax(Int)/typemin(Int) exactly, which for an integer-valued float is the same as
 * comparing against +-2^63. */
int64_t FN(pno_floor_to_int_)(T x) {
  T r = (T)floor((double)x);
  if (isnan(r) || r >= (T)9223372036854775808.0) return INT64_MAX;
  if (r <= -(T)9223372036854775808.0) return INT64_MIN;
  return (int64_t)r;
}

/* full_grid.jl:48-82 (FullGridCellList ctor) + nhs_grid.jl:77-129 (Grid NHS ctor). */
int FN(pno_grid_create_)(int32_t ndims, T radius, const T* min_corner, const T* max_corner,
                         const T* periodic_min, const T* periodic_max, int32_t max_ppc,
                         pno_grid* g) {
  memset(g, 0, sizeof(*g));
  if (ndims < 1 || ndims > 3) return PNO_ERR_INVALID_ARG;
  g->ndims = ndims;
  g->dtype = (sizeof(T) == 8);
  g->max_ppc = max_ppc;
  g->radius = (double)radius;
  /* `1001 // 1000 * search_radius`: Rational -> T(1001)/T(1000), then times r, in T. */
  const T pad = (T)((T)1001 / (T)1000) * radius;
  for (int k = 0; k < ndims; ++k) {
    g->min_pad[k] = (double)(T)(min_corner[k] - pad);
    g->max_pad[k] = (double)(T)(max_corner[k] + pad);
    g->n_cells[k] = -1;
    g->cell_size[k] = (double)radius;
  }
  g->n_total = 1;
  /* `search_radius < eps()` compares against Float64 eps = 2^-52. */
  if ((double)radius < 2.220446049250313e-16) {
    g->is_template = 1;
    g->n_total = 0;
  } else {
    for (int k = 0; k < ndims; ++k) {
      T span = (T)((T)g->max_pad[k] - (T)g->min_pad[k]);
      T q = (T)(span / radius);
      g->n[k] = (int64_t)ceil((double)q);
      g->n_total *= g->n[k];
    }
  }
  if (periodic_min != NULL && !g->is_template) {
    g->periodic = 1;
    for (int k = 0; k < ndims; ++k) {
      g->box_min[k] = (double)periodic_min[k];
      g->box_max[k] = (double)periodic_max[k];
      T size = (T)(periodic_max[k] - periodic_min[k]);
      g->box_size[k] = (double)size;
      /* floor.(Int, (size .+ 10eps()) / r): Float64 arithmetic. */
      double nc = floor(((double)size + 10.0 * 2.220446049250313e-16) / (double)radius);
      g->n_cells[k] = (int64_t)nc;
      /* size ./ n_cells: Int promoted to T. */
      g->cell_size[k] = (double)(T)(size / (T)g->n_cells[k]);
      if (g->n_cells[k] < 3) return PNO_ERR_INVALID_ARG;
    }
  }
  return PNO_OK;
}

static inline void FN(periodic_wrap_)(const pno_grid* g, int64_t* c) {
  /* nhs_grid.jl:607-620: mod.(cell .- 2, n_cells) .+ 2 */
  if (!g->periodic) return;
  for (int k = 0; k < g->ndims; ++k) c[k] = pno_wadd(pno_mod(pno_wsub(c[k], 2), g->n_cells[k]), 2);
}

/* nhs_grid.jl:622-628 cell_coords with full_grid.jl:84-94 nonperiodic_cell_coords. */
void FN(pno_cell_coords_)(const pno_grid* g, const T* x, int64_t* out) {
  for (int k = 0; k < g->ndims; ++k) {
    T t = (T)(x[k] - (T)g->min_pad[k]);
    T q = (T)(t / (T)g->cell_size[k]);
    out[k] = pno_wadd(FN(pno_floor_to_int_)(q), 1);
  }
  FN(periodic_wrap_)(g, out);
}

/* nhs_grid.jl:636-638 generic nonperiodic_cell_coords (DictionaryCellList). */
void FN(pno_cell_coords_dict_)(const pno_grid* g, const T* x, int64_t* out) {
  for (int k = 0; k < g->ndims; ++k) {
    T q = (T)(x[k] / (T)g->cell_size[k]);
    out[k] = FN(pno_floor_to_int_)(q);
  }
  FN(periodic_wrap_)(g, out);
}

/* neighborhood_search.jl:439-449 periodic_coords. */
void FN(pno_periodic_coords_)(const pno_grid* g, const T* x, T* out) {
  for (int k = 0; k < g->ndims; ++k) {
    T mn = (T)g->box_min[k], mx = (T)g->box_max[k], sz = (T)g->box_size[k];
    T off = (T)floor((double)(T)((T)(x[k] - mn) / sz));
    T xp = (T)(x[k] - (T)(off * sz));
    if (xp < mn) xp = mn;
    if (xp > mx) xp = mx;
    out[k] = xp;
  }
}

/* full_grid.jl:205-212 check_cell_bounds: valid cells are 2:n-1 per dimension. */
static inline int FN(in_bounds_)(const pno_grid* g, const int64_t* c) {
  for (int k = 0; k < g->ndims; ++k)
    if (c[k] < 2 || c[k] > g->n[k] - 1) return 0;
  return 1;
}

/* full_grid.jl:157-161 cell_index: column-major LinearIndices, returned 0-based. */
static inline int64_t FN(linear_)(const pno_grid* g, const int64_t* c) {
  int64_t lin = 0, stride = 1;
  for (int k = 0; k < g->ndims; ++k) {
    lin += (c[k] - 1) * stride;
    stride *= g->n[k];
  }
  return lin;
}

/* nhs_grid.jl:255-281 initialize_grid! (ParallelUpdate semantics, executed serially in
 * `idx` order, so each cell's column is sorted by point index).  `cells` is the
 * DynamicVectorOfVectors backend (max_ppc x n_total, column-major), `lengths` its lengths
 * (vector_of_vectors.jl:93-121). */
int FN(pno_build_)(const pno_grid* g, const T* y, int64_t n_y, const int32_t* idx,
                   int64_t n_idx, int32_t* cells, int32_t* lengths) {
  for (int64_t c = 0; c < g->n_total; ++c) lengths[c] = 0;
  if (g->is_template) return PNO_OK;
  const int64_t m = idx ? n_idx : n_y;
  const int d = g->ndims;
  for (int64_t t = 0; t < m; ++t) {
    const int64_t i = idx ? idx[t] : t;
    if (i < 0 || i >= n_y) return PNO_ERR_INVALID_ARG;
  }
  for (int64_t t = 0; t < m; ++t) {
    const int64_t i = idx ? idx[t] : t;
    int64_t c[3];
    FN(pno_cell_coords_)(g, y + i * d, c);
    if (!FN(in_bounds_)(g, c)) return PNO_ERR_OUT_OF_DOMAIN;
    const int64_t lin = FN(linear_)(g, c);
    if (lengths[lin] + 1 > g->max_ppc) return PNO_ERR_CELL_FULL;
    cells[lin * g->max_ppc + lengths[lin]] = (int32_t)i;
    lengths[lin] += 1;
  }
  return PNO_OK;
}

/* Same, but threaded with an atomic push like the reference's ParallelUpdate on CPU
 * threads (cell order inside a column is then nondeterministic).  Used only to time the
 * CPU baseline. */
int FN(pno_build_parallel_)(const pno_grid* g, const T* y, int64_t n_y, int32_t* cells,
                            int32_t* lengths, int32_t n_threads) {
  int status = PNO_OK;
  const int d = g->ndims;
  if (g->is_template) return PNO_OK;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(static)
  for (int64_t c = 0; c < g->n_total; ++c) lengths[c] = 0;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(static)
  for (int64_t i = 0; i < n_y; ++i) {
    int64_t c[3];
    FN(pno_cell_coords_)(g, y + i * d, c);
    if (!FN(in_bounds_)(g, c)) {
      status = PNO_ERR_OUT_OF_DOMAIN;
      continue;
    }
    const int64_t lin = FN(linear_)(g, c);
    int32_t slot = __atomic_fetch_add(&lengths[lin], 1, __ATOMIC_RELAXED);
    if (slot >= g->max_ppc) {
      __atomic_fetch_sub(&lengths[lin], 1, __ATOMIC_RELAXED);
      status = PNO_ERR_CELL_FULL;
      continue;
    }
    cells[lin * g->max_ppc + slot] = (int32_t)i;
  }
  return status;
}

/* r^2 in the search radius' type: Float32 for a mixed grid. */
static inline T FN(r2_)(const pno_grid* g) {
  const T r = (T)g->radius;
  if (g->mixed) {
    const float rf = (float)g->radius;
    return (T)(float)(rf * rf);
  }
  return (T)(r * r);
}

/* neighborhood_search.jl:547-555 (via nhs_grid.jl:547-553) and :428-436:
 * pos_diff = xi - yj in T; d2 = dot(pos_diff, pos_diff); with a periodic box and
 * d2 > r^2, pos_diff -= size .* round.(pos_diff ./ size) and d2 is recomputed. */
static inline T FN(pair_d2_)(const pno_grid* g, const T* xi, const T* yj, T* pd) {
  const int d = g->ndims;
  if (g->mixed) {
    /* pos_diff = convert.(Float32, xi - yj): the difference in Float64, then rounded */
    float pf[3];
    for (int k = 0; k < d; ++k) pf[k] = (float)((double)xi[k] - (double)yj[k]);
    float d2f = pf[0] * pf[0];
    for (int k = 1; k < d; ++k) d2f = d2f + pf[k] * pf[k];
    const float rf = (float)g->radius;
    if (g->periodic && d2f > rf * rf) {
      for (int k = 0; k < d; ++k) {
        const float sz = (float)g->box_size[k];
        const float q = pf[k] / sz;
        const float rq = rintf(q);
        const float sh = sz * rq;
        pf[k] = pf[k] - sh;
      }
      d2f = pf[0] * pf[0];
      for (int k = 1; k < d; ++k) d2f = d2f + pf[k] * pf[k];
    }
    for (int k = 0; k < d; ++k) pd[k] = (T)pf[k];
    return (T)d2f;
  }
  for (int k = 0; k < d; ++k) pd[k] = (T)(xi[k] - yj[k]);
  T d2 = (T)(pd[0] * pd[0]);
  for (int k = 1; k < d; ++k) d2 = (T)(d2 + (T)(pd[k] * pd[k]));
  const T r2 = FN(r2_)(g);
  if (g->periodic && d2 > r2) {
    for (int k = 0; k < d; ++k) {
      T sz = (T)g->box_size[k];
      T q = (T)(pd[k] / sz);
      T rq = (T)rint((double)q);
      pd[k] = (T)(pd[k] - (T)(sz * rq));
    }
    d2 = (T)(pd[0] * pd[0]);
    for (int k = 1; k < d; ++k) d2 = (T)(d2 + (T)(pd[k] * pd[k]));
  }
  return d2;
}

/* The FP64 pair geometry handed to the pair functions: pos_diff recomputed in double from
 * the T coordinates (with the periodic image, when the T-precision test used one). */
static inline double FN(pair_geom64_)(const pno_grid* g, const T* xi, const T* yj,
                                      double* pd) {
  const int d = g->ndims;
  double d2 = 0.0;
  for (int k = 0; k < d; ++k) pd[k] = (double)xi[k] - (double)yj[k];
  if (g->periodic) {
    for (int k = 0; k < d; ++k) pd[k] -= g->box_size[k] * rint(pd[k] / g->box_size[k]);
  }
  for (int k = 0; k < d; ++k) d2 += pd[k] * pd[k];
  return d2;
}

static inline double FN(mass_)(const pno_params* p, int64_t j) {
  return p->masses ? p->masses[j] : p->mass;
}

/* One accepted pair (i, j) for functor `f`; accumulates into acc[] and |terms| into ab[]. */
static inline void FN(apply_)(const pno_grid* g, int32_t f, const pno_params* p, int64_t i,
                              int64_t j, const T* xi, const T* yj, double* acc,
                              double* ab) {
  const int d = g->ndims;
  double pd[3];
  if (f == PNO_F_COUNT) {
    acc[0] += 1.0;
    return;
  }
  if (f == PNO_F_INDEX_SUM) {
    acc[0] += (double)(j + 1);
    return;
  }
  const double r = sqrt(FN(pair_geom64_)(g, xi, yj, pd));
  if (f == PNO_F_NBODY_ACCEL) {
    /* benchmarks/n_body.jl:47-53 */
    const double eps_t = (sizeof(T) == 4) ? 1.1920928955078125e-7 : 2.220446049250313e-16;
    if (r < sqrt(eps_t)) return;
    const double s = -p->G * FN(mass_)(p, j) / (r * r * r);
    for (int k = 0; k < d; ++k) {
      acc[k] += s * pd[k];
      ab[k] += fabs(s * pd[k]);
    }
  } else if (f == PNO_F_POTENTIAL) {
    if (r > 0.0 && r < p->cutoff) {
      const double t = FN(mass_)(p, i) * FN(mass_)(p, j) * (1.0 / r - 1.0 / p->cutoff);
      acc[0] += t;
      ab[0] += fabs(t);
    }
  } else if (f == PNO_F_WCSPH_DENSITY) {
    const double t = FN(mass_)(p, j) * pno_wendland_w(d, p->h, r);
    acc[0] += t;
    ab[0] += fabs(t);
  } else if (f == PNO_F_WCSPH_FORCE) {
    if (r < p->r_min) return;
    const double ri = p->rho[i], rj = p->rho[j];
    const double Pi = p->pressure[i] / (ri * ri), Pj = p->pressure[j] / (rj * rj);
    double vr = 0.0;
    for (int k = 0; k < d; ++k) vr += (p->vel[i * d + k] - p->vel[j * d + k]) * pd[k];
    double visc = 0.0;
    if (vr < 0.0) {
      const double mu = p->h * vr / (r * r + p->eps_visc * p->h * p->h);
      visc = -p->alpha * p->c0 * mu / (0.5 * (ri + rj));
    }
    const double gw = pno_wendland_dw(d, p->h, r) / r;
    const double s = -FN(mass_)(p, j) * (Pi + Pj + visc) * gw;
    for (int k = 0; k < d; ++k) {
      acc[k] += s * pd[k];
      ab[k] += fabs(s * pd[k]);
    }
  }
}

/* Loop over the 3^d neighbouring cells of `ci` in CartesianIndices order (first dimension
 * fastest), nhs_grid.jl:519-583.  Returns 0 if a neighbouring cell is outside the grid
 * (the reference's BoundsError). */
#define PNO_FOR_NEIGHBOR_CELLS(g, ci, LIN, BODY)                                         \
  do {                                                                                   \
    const int d_ = (g)->ndims;                                                           \
    const int o3n = d_ >= 3 ? 1 : 0, o2n = d_ >= 2 ? 1 : 0;                              \
    for (int o3 = -o3n; o3 <= o3n; ++o3)                                                 \
      for (int o2 = -o2n; o2 <= o2n; ++o2)                                               \
        for (int o1 = -1; o1 <= 1; ++o1) {                                               \
          int64_t nc[3] = {pno_wadd((ci)[0], o1), d_ >= 2 ? pno_wadd((ci)[1], o2) : 0,   \
                           d_ >= 3 ? pno_wadd((ci)[2], o3) : 0};                         \
          FN(periodic_wrap_)(g, nc);                                                     \
          int ok_ = 1;                                                                   \
          for (int k_ = 0; k_ < d_; ++k_)                                                \
            if (nc[k_] < 1 || nc[k_] > (g)->n[k_]) ok_ = 0;                              \
          if (!ok_) {                                                                    \
            bad = 1;                                                                     \
            continue;                                                                    \
          }                                                                              \
          const int64_t LIN = FN(linear_)(g, nc);                                        \
          BODY                                                                           \
        }                                                                                \
  } while (0)

/* neighborhood_search.jl:183-201 foreach_point_neighbor + nhs_grid.jl:519-575, with the
 * pair function fixed to functor `f`.  Each point's accumulators are summed in the
 * reference's iteration order (cells in CartesianIndices order, points in column order). */
int FN(pno_foreach_)(const pno_grid* g, const int32_t* cells, const int32_t* lengths,
                     const T* x, int64_t n_x, const T* y, int64_t n_y,
                     const int32_t* points, int64_t n_points, int32_t f,
                     const pno_params* p, void* out, double* abs_out, int32_t n_threads) {
  const int d = g->ndims;
  const T r2 = FN(r2_)(g);
  const int64_t m = points ? n_points : n_x;
  int status = PNO_OK;
  (void)n_y;
  if (g->is_template) return PNO_ERR_INVALID_ARG;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 64)
  for (int64_t t = 0; t < m; ++t) {
    const int64_t i = points ? points[t] : t;
    if (i < 0 || i >= n_x) {
      status = PNO_ERR_INVALID_ARG;
      continue;
    }
    const T* xi = x + i * d;
    int64_t ci[3];
    FN(pno_cell_coords_)(g, xi, ci);
    double acc[3] = {0, 0, 0}, ab[3] = {0, 0, 0};
    int bad = 0;
    PNO_FOR_NEIGHBOR_CELLS(g, ci, lin, {
      const int32_t len = lengths[lin];
      const int32_t* col = cells + lin * g->max_ppc;
      for (int32_t a = 0; a < len; ++a) {
        const int64_t j = col[a];
        const T* yj = y + j * d;
        T pd[3];
        const T d2 = FN(pair_d2_)(g, xi, yj, pd);
        if (d2 <= r2) FN(apply_)(g, f, p, i, j, xi, yj, acc, ab);
      }
    });
    if (bad) {
      status = PNO_ERR_OUT_OF_DOMAIN;
      continue;
    }
    const int nout = (f == PNO_F_NBODY_ACCEL || f == PNO_F_WCSPH_FORCE) ? d : 1;
    if (f == PNO_F_COUNT) {
      ((int32_t*)out)[i] = (int32_t)acc[0];
    } else if (f == PNO_F_INDEX_SUM) {
      ((int64_t*)out)[i] = (int64_t)acc[0];
    } else {
      for (int k = 0; k < nout; ++k) {
        ((double*)out)[i * nout + k] = acc[k];
        if (abs_out) abs_out[i * nout + k] = ab[k];
      }
    }
  }
  return status;
}

/* Neighbour lists in the reference's traversal order.  With offsets == NULL only counts[]
 * is written; otherwise row i is written to nbrs[offsets[i] ...]. */
int FN(pno_neighbor_lists_)(const pno_grid* g, const int32_t* cells, const int32_t* lengths,
                            const T* x, int64_t n_x, const T* y, int64_t n_y,
                            const int64_t* offsets, int32_t* counts, int32_t* nbrs,
                            int32_t n_threads) {
  const int d = g->ndims;
  const T r2 = FN(r2_)(g);
  int status = PNO_OK;
  (void)n_y;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 64)
  for (int64_t i = 0; i < n_x; ++i) {
    const T* xi = x + i * d;
    int64_t ci[3];
    FN(pno_cell_coords_)(g, xi, ci);
    int64_t cnt = 0;
    int bad = 0;
    PNO_FOR_NEIGHBOR_CELLS(g, ci, lin, {
      const int32_t len = lengths[lin];
      const int32_t* col = cells + lin * g->max_ppc;
      for (int32_t a = 0; a < len; ++a) {
        const int64_t j = col[a];
        T pd[3];
        if (FN(pair_d2_)(g, xi, y + j * d, pd) <= r2) {
          if (offsets) nbrs[offsets[i] + cnt] = (int32_t)j;
          ++cnt;
        }
      }
    });
    if (bad) status = PNO_ERR_OUT_OF_DOMAIN;
    counts[i] = (int32_t)cnt;
  }
  return status;
}

/* nhs_trivial.jl:55 + neighborhood_search.jl:390-421: every point of y is a candidate. */
int FN(pno_trivial_lists_)(const pno_grid* g, const T* x, int64_t n_x, const T* y,
                           int64_t n_y, const int64_t* offsets, int32_t* counts,
                           int32_t* nbrs, int32_t n_threads) {
  const int d = g->ndims;
  const T r2 = FN(r2_)(g);
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 16)
  for (int64_t i = 0; i < n_x; ++i) {
    int64_t cnt = 0;
    for (int64_t j = 0; j < n_y; ++j) {
      T pd[3];
      if (FN(pair_d2_)(g, x + i * d, y + j * d, pd) <= r2) {
        if (offsets) nbrs[offsets[i] + cnt] = (int32_t)j;
        ++cnt;
      }
    }
    counts[i] = (int32_t)cnt;
  }
  return PNO_OK;
}

/* nhs_grid.jl:585-591 eachneighbor: all points in the 3^d cells around q (candidates, not
 * filtered by distance).  Returns the count, or -1 on a BoundsError. */
int64_t FN(pno_eachneighbor_)(const pno_grid* g, const int32_t* cells,
                              const int32_t* lengths, const T* q, int32_t* out,
                              int64_t cap) {
  int64_t ci[3];
  int64_t cnt = 0;
  int bad = 0;
  FN(pno_cell_coords_)(g, q, ci);
  PNO_FOR_NEIGHBOR_CELLS(g, ci, lin, {
    for (int32_t a = 0; a < lengths[lin]; ++a) {
      if (cnt < cap) out[cnt] = cells[lin * g->max_ppc + a];
      ++cnt;
    }
  });
  return bad ? -1 : cnt;
}

/* eachneighbor for a DictionaryCellList (cell = floor(x / cell_size), no offset): the
 * candidates are the points whose cell is one of the 3^d cells around q's cell. */
int64_t FN(pno_eachneighbor_dict_)(const pno_grid* g, const T* y, int64_t n_y, const T* q,
                                   int32_t* out, int64_t cap) {
  const int d = g->ndims;
  int64_t cq[3], cnt = 0;
  FN(pno_cell_coords_dict_)(g, q, cq);
  /* Walk cells in CartesianIndices order; inside a cell, points in insertion order. */
  for (int o3 = (d >= 3 ? -1 : 0); o3 <= (d >= 3 ? 1 : 0); ++o3)
    for (int o2 = (d >= 2 ? -1 : 0); o2 <= (d >= 2 ? 1 : 0); ++o2)
      for (int o1 = -1; o1 <= 1; ++o1) {
        int64_t nc[3] = {pno_wadd(cq[0], o1), d >= 2 ? pno_wadd(cq[1], o2) : 0,
                         d >= 3 ? pno_wadd(cq[2], o3) : 0};
        FN(periodic_wrap_)(g, nc);
        for (int64_t j = 0; j < n_y; ++j) {
          int64_t cj[3];
          FN(pno_cell_coords_dict_)(g, y + j * d, cj);
          int same = 1;
          for (int k = 0; k < d; ++k)
            if (cj[k] != nc[k]) same = 0;
          if (same) {
            if (cnt < cap) out[cnt] = (int32_t)j;
            ++cnt;
          }
        }
      }
  return cnt;
}

/* FP64 loss L = sum_i (rho_i - 1)^2 + lambda * E and its gradient with respect to the
 * coordinates, over the neighbour pairs that the T-precision search finds (x == y).
 * rho_i = sum_j m W(r_ij) (self included); E = 1/2 sum_i sum_{j != i, 0<r<R} phi(r_ij),
 * phi = m_i m_j (1/r - 1/R).  grad_k = sum_j [(g_k + g_j) m W'(r) + lambda phi'(r)] e_kj,
 * g = 2 (rho - 1), e_kj = (x_k - x_j) / r. */
int FN(pno_loss_grad_)(const pno_grid* g, const int32_t* cells, const int32_t* lengths,
                       const T* x, int64_t n, const pno_params* p, double* rho,
                       double* loss, double* grad, int32_t n_threads) {
  const int d = g->ndims;
  const T r2 = FN(r2_)(g);
  double lsum = 0.0, esum = 0.0;
  int status = PNO_OK;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 64) \
    reduction(+ : lsum, esum)
  for (int64_t i = 0; i < n; ++i) {
    const T* xi = x + i * d;
    int64_t ci[3];
    FN(pno_cell_coords_)(g, xi, ci);
    double rh = 0.0, e = 0.0;
    int bad = 0;
    PNO_FOR_NEIGHBOR_CELLS(g, ci, lin, {
      for (int32_t a = 0; a < lengths[lin]; ++a) {
        const int64_t j = cells[lin * g->max_ppc + a];
        T pdt[3];
        if (FN(pair_d2_)(g, xi, x + j * d, pdt) <= r2) {
          double pd[3];
          const double rr = sqrt(FN(pair_geom64_)(g, xi, x + j * d, pd));
          rh += FN(mass_)(p, j) * pno_wendland_w(d, p->h, rr);
          if (rr > 0.0 && rr < p->cutoff)
            e += FN(mass_)(p, i) * FN(mass_)(p, j) * (1.0 / rr - 1.0 / p->cutoff);
        }
      }
    });
    if (bad) status = PNO_ERR_OUT_OF_DOMAIN;
    rho[i] = rh;
    lsum += (rh - 1.0) * (rh - 1.0);
    esum += e;
  }
  *loss = lsum + p->lambda_pot * 0.5 * esum;
  if (!grad) return status;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 64)
  for (int64_t k = 0; k < n; ++k) {
    const T* xk = x + k * d;
    int64_t ci[3];
    FN(pno_cell_coords_)(g, xk, ci);
    double acc[3] = {0, 0, 0};
    const double gk = 2.0 * (rho[k] - 1.0);
    int bad = 0;
    PNO_FOR_NEIGHBOR_CELLS(g, ci, lin, {
      for (int32_t a = 0; a < lengths[lin]; ++a) {
        const int64_t j = cells[lin * g->max_ppc + a];
        T pdt[3];
        if (FN(pair_d2_)(g, xk, x + j * d, pdt) <= r2) {
          double pd[3];
          const double rr = sqrt(FN(pair_geom64_)(g, xk, x + j * d, pd));
          if (rr <= 0.0) continue;
          const double gj = 2.0 * (rho[j] - 1.0);
          double s = (gk + gj) * FN(mass_)(p, j) * pno_wendland_dw(d, p->h, rr);
          if (rr < p->cutoff)
            s += p->lambda_pot * (-FN(mass_)(p, k) * FN(mass_)(p, j) / (rr * rr));
          for (int q = 0; q < d; ++q) acc[q] += s * pd[q] / rr;
        }
      }
    });
    (void)bad;
    for (int q = 0; q < d; ++q) grad[k * d + q] = acc[q];
  }
  return status;
}

/* Central finite differences of the same loss for the coordinates listed in `which`
 * (entry = point * d + dim), with the neighbour set held fixed and the change of L
 * evaluated locally around the moved point, in FP64. */
int FN(pno_loss_fd_)(const pno_grid* g, const int32_t* cells, const int32_t* lengths,
                     const T* x, int64_t n, const pno_params* p, const double* rho,
                     const int64_t* which, int64_t n_which, double step, double* fd) {
  const int d = g->ndims;
  const T r2 = FN(r2_)(g);
  (void)n;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t w = 0; w < n_which; ++w) {
    const int64_t k = which[w] / d;
    const int dim = (int)(which[w] % d);
    const T* xk = x + k * d;
    int64_t ci[3];
    FN(pno_cell_coords_)(g, xk, ci);
    double dl[2] = {0.0, 0.0};
    for (int side = 0; side < 2; ++side) {
      const double sgn = side == 0 ? 1.0 : -1.0;
      double drho_k = 0.0, dl_nb = 0.0, de = 0.0;
      int bad = 0;
      PNO_FOR_NEIGHBOR_CELLS(g, ci, lin, {
        for (int32_t a = 0; a < lengths[lin]; ++a) {
          const int64_t j = cells[lin * g->max_ppc + a];
          if (j == k) continue;
          T pdt[3];
          if (FN(pair_d2_)(g, xk, x + j * d, pdt) <= r2) {
            double pd[3];
            const double r0 = sqrt(FN(pair_geom64_)(g, xk, x + j * d, pd));
            pd[dim] += sgn * step;
            double s2 = 0.0;
            for (int q = 0; q < d; ++q) s2 += pd[q] * pd[q];
            const double r1 = sqrt(s2);
            const double mj = FN(mass_)(p, j);
            const double dw = mj * (pno_wendland_w(d, p->h, r1) - pno_wendland_w(d, p->h, r0));
            drho_k += dw;
            dl_nb += dw * (2.0 * (rho[j] - 1.0) + dw);
            const double mm = FN(mass_)(p, k) * mj;
            const double e1 = (r1 > 0.0 && r1 < p->cutoff) ? mm * (1.0 / r1 - 1.0 / p->cutoff) : 0.0;
            const double e0 = (r0 > 0.0 && r0 < p->cutoff) ? mm * (1.0 / r0 - 1.0 / p->cutoff) : 0.0;
            de += e1 - e0;
          }
        }
      });
      (void)bad;
      dl[side] = drho_k * (2.0 * (rho[k] - 1.0) + drho_k) + dl_nb + p->lambda_pot * de;
    }
    fd[w] = (dl[0] - dl[1]) / (2.0 * step);
  }
  return PNO_OK;
}

/* ---------------------------------------------------------------- SpatialHashingCellList */

/* GridNeighborhoodSearch over SpatialHashingCellList{d}(; list_size, max_points_per_cell)
 * (spatial_hashing.jl:79-89, nhs_grid.jl:77-129): the cell size is r, or the PeriodicBox's
 * size / n_cells as for the full grid; a point's cell is floor.(x ./ cell_size)
 * (nhs_grid.jl:636-638), wrapped to 2:n_cells+1 with a periodic box. */
int FN(pno_grid_create_hash_)(int32_t ndims, T radius, const T* periodic_min,
                              const T* periodic_max, int64_t list_size, int32_t max_ppc,
                              pno_grid* g) {
  const T zero[3] = {(T)0, (T)0, (T)0};
  if (list_size < 1) return PNO_ERR_INVALID_ARG;
  const int st = FN(pno_grid_create_)(ndims, radius, periodic_min ? periodic_min : zero,
                                      periodic_max ? periodic_max : zero, periodic_min,
                                      periodic_max, max_ppc, g);
  if (st != PNO_OK) return st;
  g->list_size = list_size;
  g->n_total = list_size;
  return PNO_OK;
}

/* initialize_grid! into a SpatialHashingCellList (nhs_grid.jl:227-281), serially in point
 * order.  `cells` holds list_size lists of max_ppc entries (the DynamicVectorOfVectors
 * backend), `coords` the flattened coordinates stored for each list (4 words; all zero is
 * typemin(UInt128), unused) and `collisions` the collision flags.  atomic == 0 restates
 * push_cell! (spatial_hashing.jl:91-107, SerialUpdate): the first cell pushed into a list
 * sets its coordinates, another cell marks a collision.  atomic != 0 restates
 * push_cell_atomic! (:109-126, used by the default ParallelUpdate): there the stored
 * UInt128 is compared with a tuple, which is never equal, so the coordinates stay unused
 * and every push of a cell whose flattened coordinates are not zero marks a collision. */
int FN(pno_hash_build_)(const pno_grid* g, const T* y, int64_t n_y, int32_t* cells,
                        int32_t* lengths, uint32_t* coords, uint8_t* collisions,
                        int32_t atomic) {
  const int64_t L = g->list_size;
  const int d = g->ndims;
  for (int64_t h = 0; h < L; ++h) {
    lengths[h] = 0;
    coords[4 * h] = coords[4 * h + 1] = coords[4 * h + 2] = coords[4 * h + 3] = 0;
    collisions[h] = 0;
  }
  if (g->is_template) return PNO_OK;
  for (int64_t i = 0; i < n_y; ++i) {
    int64_t c[3] = {0, 0, 0};
    FN(pno_cell_coords_dict_)(g, y + i * d, c);
    const int64_t h = pno_spatial_hash(c, d, L);
    if (lengths[h] + 1 > g->max_ppc) return PNO_ERR_CELL_FULL;
    cells[h * g->max_ppc + lengths[h]] = (int32_t)i;
    lengths[h] += 1;
    uint32_t flat[4];
    if (pno_coordinates_flattened(c, d, flat) != PNO_OK) return PNO_ERR_OUT_OF_DOMAIN;
    uint32_t* cw = coords + 4 * h;
    const int unused = !cw[0] && !cw[1] && !cw[2] && !cw[3];
    const int same = cw[0] == flat[0] && cw[1] == flat[1] && cw[2] == flat[2] &&
                     cw[3] == flat[3];
    if (atomic) {
      if (!same) collisions[h] = 1;
    } else if (unused) {
      for (int k = 0; k < 4; ++k) cw[k] = flat[k];
    } else if (!same) {
      collisions[h] = 1;
    }
  }
  return PNO_OK;
}

/* Neighbour lists over a SpatialHashingCellList: nhs_grid.jl:519-575 with its collision
 * handling (:479-513).  For each of the 3^d cells (CartesianIndices order) the cell's list
 * is visited; when the list has a collision flag, or stored coordinates other than the
 * cell's (check_cell_collision), each accepted point's own cell is compared with the
 * visited cell (check_collision) and a point of another cell is skipped. */
int FN(pno_hash_neighbor_lists_)(const pno_grid* g, const int32_t* cells,
                                 const int32_t* lengths, const uint32_t* coords,
                                 const uint8_t* collisions, const T* x, int64_t n_x,
                                 const T* y, int64_t n_y, const int64_t* offsets,
                                 int32_t* counts, int32_t* nbrs, int32_t n_threads) {
  const int d = g->ndims;
  const T r2 = FN(r2_)(g);
  int status = PNO_OK;
  (void)n_y;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 64)
  for (int64_t i = 0; i < n_x; ++i) {
    const T* xi = x + i * d;
    int64_t ci[3] = {0, 0, 0};
    FN(pno_cell_coords_dict_)(g, xi, ci);
    int64_t cnt = 0;
    int bad = 0;
    const int o3n = d >= 3 ? 1 : 0, o2n = d >= 2 ? 1 : 0;
    for (int o3 = -o3n; o3 <= o3n; ++o3)
      for (int o2 = -o2n; o2 <= o2n; ++o2)
        for (int o1 = -1; o1 <= 1; ++o1) {
          int64_t nc[3] = {pno_wadd(ci[0], o1), d >= 2 ? pno_wadd(ci[1], o2) : 0,
                           d >= 3 ? pno_wadd(ci[2], o3) : 0};
          FN(periodic_wrap_)(g, nc);
          const int64_t h = pno_spatial_hash(nc, d, g->list_size);
          uint32_t flat[4];
          if (pno_coordinates_flattened(nc, d, flat) != PNO_OK) {
            bad = 1;
            continue;
          }
          const uint32_t* cw = coords + 4 * h;
          const int cell_collision = collisions[h] || cw[0] != flat[0] || cw[1] != flat[1] ||
                                     cw[2] != flat[2] || cw[3] != flat[3];
          for (int32_t a = 0; a < lengths[h]; ++a) {
            const int64_t j = cells[h * g->max_ppc + a];
            T pd[3];
            if (!(FN(pair_d2_)(g, xi, y + j * d, pd) <= r2)) continue;
            if (cell_collision) {
              int64_t cj[3] = {0, 0, 0};
              FN(pno_cell_coords_dict_)(g, y + j * d, cj);
              if (cj[0] != nc[0] || cj[1] != nc[1] || cj[2] != nc[2]) continue;
            }
            if (offsets) nbrs[offsets[i] + cnt] = (int32_t)j;
            ++cnt;
          }
        }
    if (bad) status = PNO_ERR_OUT_OF_DOMAIN;
    counts[i] = (int32_t)cnt;
  }
  return status;
}

#undef FN
