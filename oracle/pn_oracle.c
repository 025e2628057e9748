/*
 * pn_oracle.c -- CPU restatement of PointNeighbors.jl's GridNeighborhoodSearch +
 * FullGridCellList (ParallelUpdate), TrivialNeighborhoodSearch and the benchmark pair
 * functions.  TEST INFRASTRUCTURE ONLY: what the CUDA library is compared with, never
 * part of the product path.  Build: oracle/build_oracle.py (gcc -O2 -fopenmp -ffp-contract=off).
 *
 * Reference files followed (paths inside PointNeighbors.jl v0.6.7):
 *   src/util.jl:2-34                      extract_svector, floor_to_int
 *   src/cell_lists/full_grid.jl:48-212    FullGridCellList ctor, cell coords, bounds check
 *   src/vector_of_vectors.jl:93-121       pushat_atomic!, "cell list is full"
 *   src/nhs_grid.jl:77-129,255-281        Grid NHS ctor, initialize_grid! (ParallelUpdate)
 *   src/nhs_grid.jl:519-638               traversal, neighboring_cells, periodic_cell_index
 *   src/neighborhood_search.jl:183-453    foreach_point_neighbor, periodic distance/coords
 *   src/nhs_trivial.jl:21-55              brute-force TrivialNeighborhoodSearch
 *   benchmarks/n_body.jl:16-55            n-body pair function
 * The WCSPH pair functions (Wendland C2, Tait EOS, Monaghan viscosity) are the workload's
 * own definitions; the reference delegates them to TrixiParticles, which is not vendored.
 */
#include "pn_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PNO_CAT_(a, b) a##b
#define PNO_CAT(a, b) PNO_CAT_(a, b)

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Julia Int64 arithmetic wraps around. */
static inline int64_t pno_wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
static inline int64_t pno_wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
/* Julia `mod(x, n)` for n > 0: result in [0, n). */
static inline int64_t pno_mod(int64_t x, int64_t n) {
  int64_t r = x % n;
  if (r != 0 && ((r < 0) != (n < 0))) r += n;
  return r;
}

/* spatial_hashing.jl:142-156 spatial_hash (Ihmsen et al.): Int64 products and xor, which
 * wrap around like Julia's, then mod(h, list_size); returned 0-based. */
int64_t pno_spatial_hash(const int64_t* cell, int32_t ndims, int64_t list_size) {
  uint64_t h = (uint64_t)cell[0] * 73856093u;
  if (ndims >= 2) h ^= (uint64_t)cell[1] * 19349663u;
  if (ndims >= 3) h ^= (uint64_t)cell[2] * 83492791u;
  return pno_mod((int64_t)h, list_size);
}

/* spatial_hashing.jl:171-184 coordinates_flattened: coordinate k, reinterpreted as UInt32,
 * at bits 32k of a UInt128. */
int pno_coordinates_flattened(const int64_t* cell, int32_t ndims, uint32_t* out) {
  out[0] = out[1] = out[2] = out[3] = 0;
  for (int k = 0; k < ndims; ++k) {
    if (cell[k] < INT32_MIN || cell[k] > INT32_MAX) return PNO_ERR_OUT_OF_DOMAIN;
    out[k] = (uint32_t)(int32_t)cell[k];
  }
  return PNO_OK;
}

/* Wendland C2 kernel with support 2h: W = sigma_d (1 - q/2)^4 (2q + 1), q = r/h. */
static inline double pno_wendland_sigma(int d, double h) {
  if (d == 3) return 21.0 / (16.0 * M_PI * h * h * h);
  if (d == 2) return 7.0 / (4.0 * M_PI * h * h);
  return 5.0 / (8.0 * h);
}
static inline double pno_wendland_w(int d, double h, double r) {
  const double q = r / h;
  if (q >= 2.0) return 0.0;
  const double t = 1.0 - 0.5 * q;
  return pno_wendland_sigma(d, h) * t * t * t * t * (2.0 * q + 1.0);
}
/* dW/dr = sigma_d / h * (-5 q) (1 - q/2)^3 */
static inline double pno_wendland_dw(int d, double h, double r) {
  const double q = r / h;
  if (q >= 2.0) return 0.0;
  const double t = 1.0 - 0.5 * q;
  return pno_wendland_sigma(d, h) / h * (-5.0 * q) * t * t * t;
}

#define T float
#define S f32
#include "pn_oracle_body.h"
#undef T
#undef S

#define T double
#define S f64
#include "pn_oracle_body.h"
#undef T
#undef S

/* Float64 coordinates, Float32 search radius (pn_oracle.h). full_grid.jl:48-82: the padding
 * `1001 // 1000 * search_radius` is Float32 (the Rational converts to the radius' type),
 * subtracted from the Float64 corners in Float64; the grid size is
 * ceil((max - min) / search_radius) in Float64.  nhs_grid.jl:112-124 with a Float32
 * PeriodicBox: n_cells = floor((size + 10eps()) / r) in Float64, cell_size = size / n_cells
 * in Float32. */
int pno_grid_create_mixed(int32_t ndims, float radius, const double* min_corner,
                          const double* max_corner, const float* periodic_min,
                          const float* periodic_max, int32_t max_ppc, pno_grid* g) {
  memset(g, 0, sizeof(*g));
  if (ndims < 1 || ndims > 3) return PNO_ERR_INVALID_ARG;
  g->ndims = ndims;
  g->dtype = 1;
  g->mixed = 1;
  g->max_ppc = max_ppc;
  g->radius = (double)radius;
  const float pad = (float)((float)1001 / (float)1000) * radius;
  for (int k = 0; k < ndims; ++k) {
    g->min_pad[k] = min_corner[k] - (double)pad;
    g->max_pad[k] = max_corner[k] + (double)pad;
    g->n_cells[k] = -1;
    g->cell_size[k] = (double)radius;
  }
  g->n_total = 1;
  if ((double)radius < 2.220446049250313e-16) {
    g->is_template = 1;
    g->n_total = 0;
  } else {
    for (int k = 0; k < ndims; ++k) {
      g->n[k] = (int64_t)ceil((g->max_pad[k] - g->min_pad[k]) / (double)radius);
      g->n_total *= g->n[k];
    }
  }
  if (periodic_min != NULL && !g->is_template) {
    g->periodic = 1;
    for (int k = 0; k < ndims; ++k) {
      g->box_min[k] = (double)periodic_min[k];
      g->box_max[k] = (double)periodic_max[k];
      const float size = periodic_max[k] - periodic_min[k];
      g->box_size[k] = (double)size;
      const double nc = floor(((double)size + 10.0 * 2.220446049250313e-16) / (double)radius);
      g->n_cells[k] = (int64_t)nc;
      g->cell_size[k] = (double)(size / (float)g->n_cells[k]);
      if (g->n_cells[k] < 3) return PNO_ERR_INVALID_ARG;
    }
  }
  return PNO_OK;
}
