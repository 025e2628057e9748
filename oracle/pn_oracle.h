/*
 * pn_oracle.h -- CPU restatement of PointNeighbors.jl's GridNeighborhoodSearch over
 * FullGridCellList, of TrivialNeighborhoodSearch, and of the pair functions used by the
 * benchmarks.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links or calls this code: it is
 * what the CUDA path is compared against (tests/, __graft_entry__.smoke(), and bench.py's
 * CPU-baseline leg).
 *
 * Parity pin: the reference (Julia) cannot run in this environment, so this restatement
 * is pinned against the known-answer vectors that the reference's own test suite holds
 * (test/nhs_grid.jl, test/neighborhood_search.jl, test/cell_lists/full_grid.jl,
 * test/gpu.jl); see tests/test_oracle_golden.py.
 *
 * Every function is instantiated for float (suffix _f32) and double (suffix _f64).
 * Indices at this interface are 0-based; cell coordinates are the reference's 1-based
 * cell coordinates (int64, with Julia's wrapping integer arithmetic).
 */
#ifndef PN_ORACLE_H
#define PN_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PNO_OK = 0,
  PNO_ERR_OUT_OF_DOMAIN = 1, /* "particle coordinates are NaN or outside the domain ..." */
  PNO_ERR_INVALID_ARG = 2,   /* ArgumentError / BoundsError on construction or indices  */
  PNO_ERR_CELL_FULL = 6      /* "cell list is full. Use a larger `max_points_per_cell`." */
};

/* Functor ids (same numbering as the CUDA library's pn_functor). */
enum {
  PNO_F_COUNT = 0,        /* out: int32[n_x]  number of f calls per point (self included)   */
  PNO_F_NBODY_ACCEL = 2,  /* out: double[n_x*d]  -G m_j pos_diff / d^3, d >= sqrt(eps(T))   */
  PNO_F_POTENTIAL = 3,    /* out: double[n_x]    m_i m_j (1/d - 1/R), 0 < d < R            */
  PNO_F_WCSPH_DENSITY = 4,/* out: double[n_x]    sum_j m_j W(d)                            */
  PNO_F_WCSPH_FORCE = 5,  /* out: double[n_x*d]  pressure + Monaghan viscosity acceleration */
  PNO_F_INDEX_SUM = 7     /* out: int64[n_x]     sum of neighbour indices (1-based)         */
};

/* Grid geometry, exactly as the reference computes it (values are exact in T). */
typedef struct {
  int32_t ndims;
  int32_t periodic;
  int32_t dtype;           /* 0 = Float32, 1 = Float64 */
  int32_t max_ppc;         /* max_points_per_cell (column capacity)                  */
  int64_t n[3];            /* padded FullGridCellList size per dimension             */
  int64_t n_cells[3];      /* periodic cell count per dimension, -1 if not periodic  */
  int64_t n_total;         /* prod(n)                                                */
  double min_pad[3];       /* min_corner - 1.001 r (in T)                            */
  double max_pad[3];
  double cell_size[3];     /* r, or periodic_box.size / n_cells (in T)               */
  double box_min[3], box_max[3], box_size[3];
  double radius;
  int32_t is_template;     /* search_radius < eps(): empty template cell list        */
  int32_t mixed;           /* Float64 coordinates with a Float32 search radius        */
  int64_t list_size;       /* SpatialHashingCellList: number of hash lists (0: none)  */
} pno_grid;

/* Pair-function parameters (all in FP64; the oracle evaluates pair functions in FP64). */
typedef struct {
  double mass;          /* uniform particle mass m (used when masses == NULL)     */
  const double* masses; /* optional per-point masses (neighbour side indexed by j) */
  double G;             /* n-body gravitational constant                          */
  double cutoff;        /* potential cutoff R                                     */
  double h;             /* smoothing length                                       */
  double c0, rho0, gamma_exp;  /* Tait equation of state                          */
  double alpha;         /* Monaghan artificial viscosity alpha                    */
  double eps_visc;      /* viscosity regularisation epsilon (times h^2)           */
  double r_min;         /* pairs closer than this are skipped by force functors  */
  const double* rho;    /* per-point density (force functor)                      */
  const double* pressure;
  const double* vel;    /* per-point velocity, d components per point             */
  double lambda_pot;    /* loss weight of the n-body energy                       */
} pno_params;

/* GridNeighborhoodSearch with Float64 coordinates (and cell-list corners) and a Float32
 * search radius (docs/literate/src/tut_gpu_usage.jl:38-50): cells in Float64 with the
 * Float32 padding and cell size; pos_diff = Float32(xi - yj), d2, the periodic correction
 * and the test in Float32 (nhs_grid.jl:547-555, neighborhood_search.jl:428-436).  The
 * other functions take the Float64 (_f64) entry points with this grid. */
int pno_grid_create_mixed(int32_t ndims, float radius, const double* min_corner,
                          const double* max_corner, const float* periodic_min,
                          const float* periodic_max, int32_t max_ppc, pno_grid* g);

/* SpatialHashingCellList helpers (cell_lists/spatial_hashing.jl:142-162): the 0-based
 * hash list of a cell, and its coordinates flattened to 128 bits as four 32-bit words
 * (word k = the k-th coordinate as UInt32, word 3 = 0).  coordinates_flattened returns
 * PNO_ERR_OUT_OF_DOMAIN where the reference throws InexactError (a coordinate outside
 * Int32). */
int64_t pno_spatial_hash(const int64_t* cell, int32_t ndims, int64_t list_size);
int pno_coordinates_flattened(const int64_t* cell, int32_t ndims, uint32_t* out);

#define PNO_DECL(T, S)                                                                     \
  int64_t pno_floor_to_int_##S(T x);                                                       \
  int pno_grid_create_##S(int32_t ndims, T radius, const T* min_corner, const T* max_corner,\
                          const T* periodic_min, const T* periodic_max, int32_t max_ppc,   \
                          pno_grid* g);                                                    \
  void pno_cell_coords_##S(const pno_grid* g, const T* x, int64_t* out);                   \
  void pno_cell_coords_dict_##S(const pno_grid* g, const T* x, int64_t* out);              \
  void pno_periodic_coords_##S(const pno_grid* g, const T* x, T* out);                     \
  int pno_build_##S(const pno_grid* g, const T* y, int64_t n_y, const int32_t* idx,        \
                    int64_t n_idx, int32_t* cells, int32_t* lengths);                      \
  int pno_build_parallel_##S(const pno_grid* g, const T* y, int64_t n_y, int32_t* cells,   \
                             int32_t* lengths, int32_t n_threads);                         \
  int pno_foreach_##S(const pno_grid* g, const int32_t* cells, const int32_t* lengths,     \
                      const T* x, int64_t n_x, const T* y, int64_t n_y,                    \
                      const int32_t* points, int64_t n_points, int32_t functor,            \
                      const pno_params* p, void* out, double* abs_out, int32_t n_threads); \
  int pno_neighbor_lists_##S(const pno_grid* g, const int32_t* cells,                      \
                             const int32_t* lengths, const T* x, int64_t n_x, const T* y,  \
                             int64_t n_y, const int64_t* offsets, int32_t* counts,         \
                             int32_t* nbrs, int32_t n_threads);                            \
  int pno_trivial_lists_##S(const pno_grid* g, const T* x, int64_t n_x, const T* y,        \
                            int64_t n_y, const int64_t* offsets, int32_t* counts,          \
                            int32_t* nbrs, int32_t n_threads);                             \
  int64_t pno_eachneighbor_##S(const pno_grid* g, const int32_t* cells,                    \
                               const int32_t* lengths, const T* q, int32_t* out,           \
                               int64_t cap);                                               \
  int64_t pno_eachneighbor_dict_##S(const pno_grid* g, const T* y, int64_t n_y,            \
                                    const T* q, int32_t* out, int64_t cap);                \
  int pno_loss_grad_##S(const pno_grid* g, const int32_t* cells, const int32_t* lengths,   \
                        const T* x, int64_t n, const pno_params* p, double* rho,           \
                        double* loss, double* grad, int32_t n_threads);                    \
  int pno_loss_fd_##S(const pno_grid* g, const int32_t* cells, const int32_t* lengths,     \
                      const T* x, int64_t n, const pno_params* p, const double* rho,       \
                      const int64_t* which, int64_t n_which, double step, double* fd);    \
  int pno_grid_create_hash_##S(int32_t ndims, T radius, const T* periodic_min,             \
                               const T* periodic_max, int64_t list_size, int32_t max_ppc,  \
                               pno_grid* g);                                               \
  int pno_hash_build_##S(const pno_grid* g, const T* y, int64_t n_y, int32_t* cells,       \
                         int32_t* lengths, uint32_t* coords, uint8_t* collisions,          \
                         int32_t atomic);                                                  \
  int pno_hash_neighbor_lists_##S(const pno_grid* g, const int32_t* cells,                 \
                                  const int32_t* lengths, const uint32_t* coords,          \
                                  const uint8_t* collisions, const T* x, int64_t n_x,      \
                                  const T* y, int64_t n_y, const int64_t* offsets,         \
                                  int32_t* counts, int32_t* nbrs, int32_t n_threads);

PNO_DECL(float, f32)
PNO_DECL(double, f64)
#undef PNO_DECL

#ifdef __cplusplus
}
#endif
#endif
