"""GB300-native GridNeighborhoodSearch over a FullGridCellList.

Python host API that mirrors PointNeighbors.jl's interface for this path
(src/PointNeighbors.jl:23-35): `GridNeighborhoodSearch`, `FullGridCellList`,
`PeriodicBox`, `initialize`, `update`, `foreach_point_neighbor`, `requires_update`,
`copy_neighborhood_search`, with the reference's argument meaning and error messages.
Julia's `initialize!`/`update!` are spelled `initialize`/`update`.  Every call goes
through the C ABI of libpn_gb300.so (include/pn_gb300.h); nothing runs on the CPU.

Conventions (the reference's):
  - coordinates are `(d, N)` tensors on the GPU, column i = point i.  The memory layout
    is the reference's column-major `T[d, N]`, i.e. a tensor with strides (1, d)
    (`pts.T` for a contiguous `(N, d)` tensor `pts`); other layouts are copied.
  - the element type of `search_radius` sets the arithmetic type; Python floats and
    float64 arrays are Float64, numpy.float32 values are Float32.
  - point indices are 0-based (Python), the reference's are 1-based.
  - the pair function `f` is one of the functor classes below; an arbitrary Python
    callable cannot run inside the CUDA kernels and raises UnsupportedFunctorError.
Calls are synchronous like the reference's (each ends with a stream sync and an error
check); `check=False` leaves them asynchronous on torch's current stream.
"""
from __future__ import annotations

import ctypes as C
import math
import numbers

import numpy as np

from . import _lib, build, workloads  # noqa: F401

lib = _lib.load

__all__ = [
    "foreach_point_neighbor_unsafe", "foreach_neighbor", "foreach_neighbor_unsafe",
    "mapreduce_neighbor", "mapreduce_neighbor_unsafe", "initialize_grid", "update_grid",
    "GridNeighborhoodSearch", "FullGridCellList", "SpatialHashingCellList", "spatial_hash",
    "PeriodicBox", "ParallelUpdate", "SemiParallelUpdate", "SerialIncrementalUpdate",
    "SerialUpdate",
    "ParallelIncrementalUpdate", "initialize", "update", "foreach_point_neighbor",
    "requires_update", "copy_neighborhood_search", "cell_coords", "eachneighbor",
    "neighbor_lists", "CountNeighbors", "NeighborIndexSum", "NBodyAcceleration",
    "TruncatedPotential", "WCSPHDensity", "WCSPHForce", "WCSPHStep",
    "AdjointLossForward", "AdjointLossBackward", "adjoint_loss", "BatchedNeighborhoodSearch",
    "PrecomputedNeighborhoodSearch",
    "ArgumentError", "BoundsError", "PointNeighborsError", "UnsupportedFunctorError",
]


# ------------------------------------------------------------------------- errors

class ArgumentError(ValueError):
    """Julia's ArgumentError."""


class BoundsError(IndexError):
    """Julia's BoundsError."""


class PointNeighborsError(RuntimeError):
    """Julia's ErrorException raised by `error(...)` in the reference."""


class UnsupportedFunctorError(TypeError):
    """The pair function is not one of the compiled functors."""


def _raise(status: int, what: str = ""):
    msg = _lib.status_string(status)
    if what:
        msg = f"{msg} ({what})"
    if status in (_lib.PN_ERR_OUT_OF_DOMAIN, _lib.PN_ERR_CELL_FULL, _lib.PN_ERR_TIMEOUT,
                  _lib.PN_ERR_CUDA, _lib.PN_ERR_OUT_OF_MEMORY, _lib.PN_ERR_CAPACITY,
                  _lib.PN_ERR_NOT_INITIALIZED):
        raise PointNeighborsError(msg)
    if status == _lib.PN_ERR_BOUNDS:
        raise BoundsError(msg)
    if status == _lib.PN_ERR_UNSUPPORTED_FUNCTOR:
        raise UnsupportedFunctorError(msg)
    raise ArgumentError(msg)


# ------------------------------------------------------------------------- types

def _eltype(v):
    """Element type implied by a value, like Julia's typeof."""
    if isinstance(v, (np.floating, np.ndarray)) and np.asarray(v).dtype == np.float32:
        return np.float32
    try:
        import torch
        if isinstance(v, torch.Tensor):
            return np.float32 if v.dtype == torch.float32 else np.float64
    except ImportError:  # pragma: no cover
        pass
    if isinstance(v, (list, tuple)) and v and all(_eltype(e) == np.float32 for e in v):
        return np.float32
    return np.float64


def _vec(v, dtype):
    try:
        import torch
        if isinstance(v, torch.Tensor):
            v = v.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(v, dtype=np.float64).astype(dtype).reshape(-1)


class PeriodicBox:
    """PeriodicBox(; min_corner, max_corner) (neighborhood_search.jl:129-141)."""

    def __init__(self, *, min_corner, max_corner):
        self.eltype = _eltype(min_corner)
        self.min_corner = _vec(min_corner, self.eltype)
        self.max_corner = _vec(max_corner, self.eltype)
        self.size = (self.max_corner - self.min_corner).astype(self.eltype)


class FullGridCellList:
    """FullGridCellList(; min_corner, max_corner, search_radius, max_points_per_cell)
    (full_grid.jl:48-82).  `min_corner`/`max_corner` hold the padded corners like the
    reference; `max_points_per_cell = 0` removes the per-cell limit.

    The corners are Float32 only when they and the search radius are (Julia's promotion of
    `min_corner .- 1001 // 1000 * search_radius`); Float64 corners with a Float32 radius
    give the mixed-precision search (Float64 coordinates, Float32 distances)."""

    def __init__(self, *, min_corner, max_corner, search_radius=0.0, max_points_per_cell=100):
        mn = _vec(min_corner, np.float64)
        mx = _vec(max_corner, np.float64)
        if mn.size != mx.size:
            raise ArgumentError("min_corner and max_corner must have the same length")
        if mn.size > 100:
            raise ArgumentError("FullGridCellList only supports up to 100 dimensions, "
                                "check your `min_corner` and `max_corner`")
        if mn.size > 3:
            raise ArgumentError("this GPU FullGridCellList supports 1 to 3 dimensions")
        R = _eltype(search_radius) if not isinstance(search_radius, numbers.Integral) else np.float64
        T = np.float32 if _eltype(min_corner) == np.float32 and R == np.float32 else np.float64
        self.eltype = T
        self.ndims = mn.size
        self._min = mn.astype(T)
        self._max = mx.astype(T)
        self.search_radius = search_radius
        self.max_points_per_cell = int(max_points_per_cell)
        r = R(search_radius)
        pad = T(R(R(1001) / R(1000)) * r)
        self.min_corner = (self._min - pad).astype(T)
        self.max_corner = (self._max + pad).astype(T)
        self.grid_size = None  # computed by the search from the corners

    @classmethod
    def from_state(cls, *, min_corner, max_corner, grid_size, max_points_per_cell=100,
                   search_radius=0.0):
        """A cell list given by the fields a reference FullGridCellList stores
        (full_grid.jl:30-35): its padded `min_corner`/`max_corner`, `size(linear_indices)`
        and the backend's capacity `size(cells.backend, 1)`.  The search takes them as they
        are (pn_create_from_grid) instead of padding corners again."""
        self = cls.__new__(cls)
        mn = _vec(min_corner, np.float64)
        mx = _vec(max_corner, np.float64)
        gs = [int(v) for v in np.atleast_1d(grid_size)]
        if mn.size != mx.size or mn.size != len(gs):
            raise ArgumentError("min_corner, max_corner and grid_size must have the same length")
        if mn.size > 3:
            raise ArgumentError("this GPU FullGridCellList supports 1 to 3 dimensions")
        R = _eltype(search_radius) if not isinstance(search_radius, numbers.Integral) else np.float64
        T = np.float32 if _eltype(min_corner) == np.float32 and R == np.float32 else np.float64
        self.eltype = T
        self.ndims = mn.size
        self.min_corner = mn.astype(T)
        self.max_corner = mx.astype(T)
        self._min, self._max = self.min_corner, self.max_corner
        self.search_radius = search_radius
        self.max_points_per_cell = int(max_points_per_cell)
        self.grid_size = tuple(gs)
        return self


class SpatialHashingCellList:
    """SpatialHashingCellList{ndims}(; list_size, max_points_per_cell = 100)
    (spatial_hashing.jl:79-89): the cells of an unbounded domain hashed into `list_size`
    lists (the reference recommends about twice the number of points).
    `max_points_per_cell` limits each list; 0 removes the limit."""

    def __init__(self, ndims, *, list_size, max_points_per_cell=100):
        if isinstance(list_size, bool) or not isinstance(list_size, numbers.Integral) or \
                list_size < 1:
            raise ArgumentError("`list_size` must be a positive integer")
        if int(ndims) not in (1, 2, 3):
            raise ArgumentError("this GPU SpatialHashingCellList supports 1 to 3 dimensions")
        self.ndims = int(ndims)
        self.list_size = int(list_size)
        self.max_points_per_cell = int(max_points_per_cell)


def spatial_hash(cell, list_size: int) -> int:
    """spatial_hash(cell, list_size) - 1 (spatial_hashing.jl:142-156): the 0-based list of
    a cell, with Julia's wrapping Int64 products and xor and mod(h, list_size)."""
    h = 0
    for c, k in zip(cell, (73856093, 19349663, 83492791)):
        h ^= (int(c) * k) & 0xFFFFFFFFFFFFFFFF
    if h >= 1 << 63:
        h -= 1 << 64
    return h % int(list_size)


class ParallelUpdate:
    """Full rebuild on update (the FullGridCellList default, nhs_grid.jl:135-144)."""

    def __repr__(self):
        return "ParallelUpdate()"

    def __eq__(self, o):
        return type(o) is type(self)


class ParallelIncrementalUpdate:
    """Re-bin only the points whose cell changed (nhs_grid.jl:146-156, 408-467).

    `rebuild_fraction` (not in the reference): when more than this fraction of the points
    are outside the cell they had at the last full build, update! rebuilds the cell list
    instead of extending its overflow lists (decided on the device; same results)."""

    def __init__(self, rebuild_fraction: float = 0.01):
        if not rebuild_fraction >= 0:
            raise ArgumentError("rebuild_fraction must be >= 0")
        self.rebuild_fraction = float(rebuild_fraction)

    def __repr__(self):
        return "ParallelIncrementalUpdate()"

    def __eq__(self, o):
        return type(o) is type(self)


class SemiParallelUpdate(ParallelIncrementalUpdate):
    """SemiParallelUpdate() (nhs_grid.jl:158-168): the reference marks the changed cells in
    parallel and moves their points serially; on the GPU it is the incremental update of
    ParallelIncrementalUpdate (the same neighbour sets)."""

    def __repr__(self):
        return "SemiParallelUpdate()"


class SerialIncrementalUpdate(ParallelIncrementalUpdate):
    """SerialIncrementalUpdate() (nhs_grid.jl:170-181): a serial incremental update in the
    reference; the incremental update of ParallelIncrementalUpdate here."""

    def __repr__(self):
        return "SerialIncrementalUpdate()"


class SerialUpdate(ParallelUpdate):
    """SerialUpdate() (nhs_grid.jl:183-194): a serial rebuild in the reference; the rebuild of
    ParallelUpdate here (the same cells; the GPU's in-cell order does not depend on threads)."""

    def __repr__(self):
        return "SerialUpdate()"


_STRATEGIES = {ParallelUpdate: _lib.PN_PARALLEL_UPDATE,
               ParallelIncrementalUpdate: _lib.PN_PARALLEL_INCREMENTAL_UPDATE,
               SemiParallelUpdate: _lib.PN_PARALLEL_INCREMENTAL_UPDATE,
               SerialIncrementalUpdate: _lib.PN_PARALLEL_INCREMENTAL_UPDATE,
               SerialUpdate: _lib.PN_PARALLEL_UPDATE}
# supported_update_strategies (full_grid.jl:39-42, spatial_hashing.jl:42-45), first = default
_FULL_GRID_STRATEGIES = (ParallelUpdate, ParallelIncrementalUpdate, SemiParallelUpdate,
                         SerialIncrementalUpdate, SerialUpdate)
_HASHING_STRATEGIES = (ParallelUpdate, SerialUpdate)


def check_update_strategy(cell_list, update_strategy):
    """The strategy to use (the cell list's first supported one for None), or the reference's
    ArgumentError (nhs_grid.jl:86-93)."""
    supported = (_HASHING_STRATEGIES if isinstance(cell_list, SpatialHashingCellList)
                 else _FULL_GRID_STRATEGIES)
    if update_strategy is None:
        return supported[0]()
    if type(update_strategy) not in supported:
        options = "(" + ", ".join(t.__name__ for t in supported) + ")"
        raise ArgumentError(f"{update_strategy} is not a valid update strategy for this "
                            f"cell list. Available options are {options}")
    return update_strategy


def _periodic_argument_error(box, r, ndims, cell_list, from_state):
    """The ArgumentError for a periodic search the library rejected: the reference's message
    when a dimension has fewer than 3 periodic cells (nhs_grid.jl:113-116), else the reason
    that is this library's own (the grid must hold the periodic cells and their neighbours,
    n_cells + 2 <= cells of the padded grid, and have fewer than 2^31 cells)."""
    T = _eltype(r)
    for k in range(ndims):
        size = T(T(box.max_corner[k]) - T(box.min_corner[k]))
        if math.floor((float(size) + 10 * 2.220446049250313e-16) / float(r)) < 3:
            raise ArgumentError("the `GridNeighborhoodSearch` needs at least 3 cells in "
                                "each dimension when used with periodicity. Please use no "
                                "NHS for very small problems.")
    if cell_list is not None:
        raise ArgumentError("the cell list must cover the periodic box: it needs n_cells + 2 "
                            "cells per dimension" +
                            (" (grid_size too small for the PeriodicBox)" if from_state else
                             " (build it over the PeriodicBox's corners)") +
                            ", and fewer than 2^31 cells in total")
    raise ArgumentError("invalid PeriodicBox for this search")


class GridNeighborhoodSearch:
    """GridNeighborhoodSearch{ndims}(; search_radius, n_points, periodic_box, cell_list,
    update_strategy) over a FullGridCellList (nhs_grid.jl:67-129).

    `pair_cache` (not in the reference): when true, the first WCSPH-density or
    adjoint-forward sweep with x is y after initialize/update also records which candidates
    of each query's stencil rows are neighbours (a start and a 128-bit mask per row, 20 bytes
    x 3^(d-1) per point), and the sweeps that follow until the next initialize/update visit
    exactly those.  Queries the cache cannot describe keep the cell stencil, so results do
    not depend on it.

    A Float32 search radius over a Float64 cell list is the reference's mixed precision
    (docs/literate/src/tut_gpu_usage.jl:38-50): coordinates are Float64 (`coord_eltype`),
    pos_diff and distance Float32 (`eltype`), and so are the pair functions' arrays."""

    def __init__(self, ndims, *, search_radius=0.0, n_points=0, periodic_box=None,
                 cell_list=None, update_strategy=None, pair_cache=0):
        if cell_list is None:
            raise ArgumentError("a FullGridCellList or SpatialHashingCellList is required: "
                                "the GPU search has no DictionaryCellList")
        if not isinstance(cell_list, (FullGridCellList, SpatialHashingCellList)):
            raise ArgumentError("only FullGridCellList and SpatialHashingCellList are "
                                "supported")
        hashing = isinstance(cell_list, SpatialHashingCellList)
        if cell_list.ndims != ndims:
            raise ArgumentError(f"a {ndims}D cell list is required for a "
                                f"GridNeighborhoodSearch{{{ndims}}}")
        update_strategy = check_update_strategy(cell_list, update_strategy)
        if isinstance(search_radius, numbers.Integral) or isinstance(search_radius, bool):
            raise ArgumentError("`search_radius` cannot be an integer type, since computed "
                                "distances will be converted to this type")
        T = _eltype(search_radius)
        if periodic_box is not None and search_radius >= 2.220446049250313e-16 \
                and periodic_box.eltype != T:
            raise ArgumentError("the `search_radius` and the `PeriodicBox` must have the "
                                "same element type")
        self.ndims = int(ndims)
        self.eltype = T
        self.mixed = not hashing and T == np.float32 and cell_list.eltype == np.float64
        self.coord_eltype = np.float64 if self.mixed else T
        self.search_radius = T(search_radius)
        self.n_points = int(n_points)
        self.periodic_box = periodic_box
        self.cell_list = cell_list
        self.update_strategy = update_strategy
        cfg = _lib.pn_config()
        cfg.ndims = self.ndims
        C_ = self.coord_eltype
        cfg.dtype = _lib.PN_FLOAT32 if C_ == np.float32 else _lib.PN_FLOAT64
        cfg.flags = _lib.PN_FLAG_FLOAT32_SEARCH if self.mixed else 0
        cfg.search_radius = float(self.search_radius)
        from_state = not hashing and cell_list.grid_size is not None
        if not hashing:
            for k in range(self.ndims):
                cfg.min_corner[k] = float(C_(cell_list._min[k]))
                cfg.max_corner[k] = float(C_(cell_list._max[k]))
        if periodic_box is not None:
            cfg.periodic = 1
            for k in range(self.ndims):
                cfg.periodic_min[k] = float(T(periodic_box.min_corner[k]))
                cfg.periodic_max[k] = float(T(periodic_box.max_corner[k]))
        cfg.update_strategy = _STRATEGIES[type(update_strategy)]
        cfg.n_points = self.n_points
        cfg.max_points_per_cell = cell_list.max_points_per_cell
        self._cfg = cfg
        h = C.c_void_p()
        if hashing:
            rc = lib().pn_create_spatial_hashing(C.byref(cfg), cell_list.list_size, C.byref(h))
        elif from_state:
            grid = (C.c_int64 * 3)(*(list(cell_list.grid_size) + [0] * (3 - self.ndims)))
            rc = lib().pn_create_from_grid(C.byref(cfg), grid, C.byref(h))
        else:
            rc = lib().pn_create(C.byref(cfg), C.byref(h))
        if rc != _lib.PN_OK:
            if rc == _lib.PN_ERR_INVALID_ARG and periodic_box is not None and \
                    self.search_radius >= 2.220446049250313e-16:
                _periodic_argument_error(periodic_box, self.search_radius, self.ndims,
                                         None if hashing else cell_list, from_state)
            _raise(rc, "GridNeighborhoodSearch")
        self._h = h
        if isinstance(update_strategy, ParallelIncrementalUpdate):
            lib().pn_set_rebuild_fraction(h, update_strategy.rebuild_fraction)
        self.pair_cache = bool(pair_cache)
        if self.pair_cache:
            lib().pn_set_pair_cache(h, 1)
        self._cfg = cfg

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().pn_destroy(h)
            except Exception:  # pragma: no cover - interpreter shutdown
                pass
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def _sync(self) -> int:
        return lib().pn_sync(self._h)

    def _clear_error(self):
        lib().pn_get_error(self._h, 1)

    def grid_info(self) -> dict:
        gi = _lib.pn_grid_info()
        rc = lib().pn_get_grid_info(self._h, C.byref(gi))
        if rc != _lib.PN_OK:
            _raise(rc)
        d = self.ndims
        return {
            "grid_size": tuple(gi.grid_size[:d]), "n_cells": tuple(gi.n_cells[:d]),
            "min_corner": tuple(gi.min_corner[:d]), "max_corner": tuple(gi.max_corner[:d]),
            "cell_size": tuple(gi.cell_size[:d]), "search_radius": gi.search_radius,
            "n_binned": gi.n_binned, "n_overflow": gi.n_overflow, "list_size": gi.list_size,
            "periodic": bool(gi.periodic), "is_template": bool(gi.is_template),
        }

    @property
    def n_cells(self):
        """Periodic cells per dimension, -1 without a periodic box (nhs_grid.jl:71)."""
        return self.grid_info()["n_cells"]

    @property
    def cell_size(self):
        return self.grid_info()["cell_size"]


# ------------------------------------------------------------------------- helpers

def _torch():
    import torch
    return torch


def _stream():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _coords(nhs: GridNeighborhoodSearch, a, name: str):
    """A (d, N) CUDA tensor in the reference's column-major layout (strides (1, d))."""
    torch = _torch()
    if not isinstance(a, torch.Tensor) or not a.is_cuda:
        raise ArgumentError(f"`{name}` must be a CUDA tensor of shape (d, N)")
    if a.dim() != 2 or a.shape[0] != nhs.ndims:
        raise ArgumentError(f"`{name}` must have shape ({nhs.ndims}, N), got {tuple(a.shape)}")
    want = torch.float32 if nhs.coord_eltype == np.float32 else torch.float64
    if a.dtype != want:
        raise ArgumentError(f"`{name}` must have dtype {want} like the cell list")
    if a.shape[1] > 0 and a.stride() != (1, nhs.ndims):
        a = a.t().contiguous().t()
    return a


def _bound(nhs, a, name):
    """The tensor the search was built from when `a` is the caller's y (so that x is y is
    recognised even when the layout had to be converted), else `a` converted."""
    if a is getattr(nhs, "_y_src", None):
        return nhs._y_keep
    return _coords(nhs, a, name)


def _index_tensor(idx, n, name):
    torch = _torch()
    if idx is None:
        return None
    if isinstance(idx, range):
        t = torch.arange(idx.start, idx.stop, idx.step, dtype=torch.int32, device="cuda")
    else:
        t = torch.as_tensor(idx, device="cuda").to(torch.int32).contiguous()
    if t.numel() and (int(t.min()) < 0 or int(t.max()) >= n):
        raise BoundsError(f"attempt to access {n}-element coordinates at index "
                          f"{name} outside 0:{n - 1}")
    return t


def _ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def _finish(nhs, rc, check, what):
    if rc != _lib.PN_OK:
        nhs._clear_error()
        _raise(rc, what)
    if check:
        st = nhs._sync()
        if st != _lib.PN_OK:
            _raise(st, what)


# ------------------------------------------------------------------------- API

def requires_update(nhs):
    """(x_changed, y_changed) -> (False, True) (nhs_grid.jl:133); (True, True) for the
    precomputed search (nhs_precomputed.jl:128)."""
    if getattr(nhs, "_precomputed", False):
        return (True, True)
    return (False, True)


def copy_neighborhood_search(nhs, search_radius, n_points):
    """Same corners, periodic box, strategy and cell capacity; new radius and size
    (nhs_grid.jl:640-649, nhs_precomputed.jl:249-266)."""
    if getattr(nhs, "_precomputed", False):
        return nhs._copy(search_radius, n_points)
    cl = nhs.cell_list
    T = _eltype(search_radius)
    if isinstance(cl, SpatialHashingCellList):  # spatial_hashing.jl:133-141
        new_cl = SpatialHashingCellList(cl.ndims, list_size=cl.list_size,
                                        max_points_per_cell=cl.max_points_per_cell)
    else:
        # copy_cell_list (full_grid.jl:179-185) passes the stored corners -- padded by the
        # old radius, not at all for a template -- to the constructor, which pads them again
        CT = np.result_type(cl.eltype, T)  # a Float64 cell list stays Float64
        new_cl = FullGridCellList(min_corner=np.asarray(cl.min_corner).astype(CT),
                                  max_corner=np.asarray(cl.max_corner).astype(CT),
                                  search_radius=T(search_radius),
                                  max_points_per_cell=cl.max_points_per_cell)
    return GridNeighborhoodSearch(nhs.ndims, search_radius=T(search_radius), n_points=n_points,
                                  periodic_box=nhs.periodic_box, cell_list=new_cl,
                                  update_strategy=nhs.update_strategy)


def initialize(nhs, x, y, *, eachindex_y=None, check=True):
    """initialize!(nhs, x, y; eachindex_y) (nhs_grid.jl:220-281, nhs_precomputed.jl:130-147)."""
    if getattr(nhs, "_precomputed", False):
        return nhs._initialize(x, y, eachindex_y, check)
    y_src = y
    y = _coords(nhs, y, "y")
    idx = _index_tensor(eachindex_y, y.shape[1], "eachindex_y")
    rc = lib().pn_initialize(nhs._h, _ptr(y), y.shape[1], _ptr(idx),
                             0 if idx is None else idx.numel(), _stream())
    nhs._y_src, nhs._y_keep = y_src, y
    nhs._generation = getattr(nhs, "_generation", 0) + 1
    _finish(nhs, rc, check, "initialize!")
    return nhs


def update(nhs: GridNeighborhoodSearch, x, y, *, points_moving=(True, True), eachindex_y=None,
           check=True):
    """update!(nhs, x, y; points_moving, eachindex_y) (nhs_grid.jl:283-292,
    nhs_precomputed.jl:149-167)."""
    if getattr(nhs, "_precomputed", False):
        return nhs._update(x, y, points_moving, eachindex_y, check)
    if not points_moving[1]:
        return nhs
    y_src = y
    y = _coords(nhs, y, "y")
    if eachindex_y is not None and isinstance(nhs.update_strategy, ParallelIncrementalUpdate) \
            and not (isinstance(eachindex_y, range) and eachindex_y == range(y.shape[1])):
        raise PointNeighborsError("this neighborhood search/update strategy does not support "
                                  "inactive points")
    idx = _index_tensor(eachindex_y, y.shape[1], "eachindex_y")
    if isinstance(nhs.update_strategy, ParallelIncrementalUpdate):
        idx = None
    rc = lib().pn_update(nhs._h, _ptr(y), y.shape[1], _ptr(idx),
                         0 if idx is None else idx.numel(), 1, _stream())
    nhs._y_src, nhs._y_keep = y_src, y
    nhs._generation = getattr(nhs, "_generation", 0) + 1
    _finish(nhs, rc, check, "update!")
    return nhs


class PairFunction:
    """A pair function compiled into the library (the `f` of foreach_point_neighbor)."""

    functor: int = -1

    def params(self, nhs, x, y, n_q):  # pragma: no cover - abstract
        raise NotImplementedError


def _out(t, name, n, dtype):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != dtype or \
            not t.is_contiguous() or t.numel() < n:
        raise ArgumentError(f"`{name}` must be a contiguous CUDA {dtype} tensor with at "
                            f"least {n} elements")
    return t


def _tdtype(nhs):
    torch = _torch()
    return torch.float32 if nhs.eltype == np.float32 else torch.float64


class CountNeighbors(PairFunction):
    """counts[i] = number of neighbours of point i (itself included), the tutorial's
    `n_neighbors[i] += 1` (docs/literate/src/tut_gpu_usage.jl:83-94)."""

    functor = _lib.PN_F_COUNT

    def __init__(self, counts):
        self.counts = counts

    def params(self, nhs, x, y, n_q):
        _out(self.counts, "counts", x.shape[1], _torch().int32)
        return _lib.pn_count_params(self.counts.data_ptr())


class NeighborIndexSum(PairFunction):
    """sums[i] = sum of the 1-based indices of i's neighbours: the reference test's
    `mapreduce_neighbor(+, ...) do ... neighbor end` (test/neighborhood_search.jl:389-399)."""

    functor = _lib.PN_F_INDEX_SUM

    def __init__(self, sums):
        self.sums = sums

    def params(self, nhs, x, y, n_q):
        _out(self.sums, "sums", x.shape[1], _torch().int64)
        return _lib.pn_index_sum_params(self.sums.data_ptr())


class NBodyAcceleration(PairFunction):
    """accel[:, i] += -G m_j pos_diff / d^3 for d >= sqrt(eps(T))
    (benchmarks/n_body.jl:41-56)."""

    functor = _lib.PN_F_NBODY_ACCEL

    def __init__(self, masses, G, accel):
        self.masses, self.G, self.accel = masses, float(G), accel

    def params(self, nhs, x, y, n_q):
        _out(self.masses, "masses", y.shape[1], _tdtype(nhs))
        _out(self.accel, "accel", x.shape[1] * nhs.ndims, _tdtype(nhs))
        return _lib.pn_nbody_params(self.masses.data_ptr(), self.G, self.accel.data_ptr())


class TruncatedPotential(PairFunction):
    """energy[i] = sum_j m_i m_j (1/d - 1/R) over neighbours with 0 < d < R."""

    functor = _lib.PN_F_POTENTIAL

    def __init__(self, masses, cutoff, energy):
        self.masses, self.cutoff, self.energy = masses, float(cutoff), energy

    def params(self, nhs, x, y, n_q):
        _out(self.masses, "masses", y.shape[1], _tdtype(nhs))
        _out(self.energy, "energy", x.shape[1], _tdtype(nhs))
        return _lib.pn_potential_params(self.masses.data_ptr(), self.cutoff,
                                        self.energy.data_ptr())


class _WCSPH(PairFunction):
    def __init__(self, *, density=None, pressure=None, velocity=None, accel=None, mass=1.0,
                 h=1.5, c0=10.0, rho0=1.0, gamma_exp=7.0, alpha=0.02, eps_visc=0.01,
                 r_min=None, reuse_state=False):
        self.density, self.pressure, self.velocity, self.accel = density, pressure, velocity, accel
        self.reuse_state = bool(reuse_state)
        self.consts = dict(mass=mass, h=h, c0=c0, rho0=rho0, gamma_exp=gamma_exp, alpha=alpha,
                           eps_visc=eps_visc)
        self.r_min = r_min

    def params(self, nhs, x, y, n_q):
        T = _tdtype(nhs)
        n = x.shape[1]
        d = nhs.ndims
        r_min = self.r_min
        if r_min is None:
            r_min = float(np.sqrt(np.finfo(nhs.eltype).eps)) * self.consts["h"]
        p = _lib.pn_wcsph_params(r_min=r_min, reuse_state=int(self.reuse_state), **self.consts)
        for name, size in (("density", n), ("pressure", n), ("velocity", n * d),
                           ("accel", n * d)):
            t = getattr(self, name)
            if t is not None:
                _out(t, name, size, T)
                setattr(p, name, t.data_ptr())
        return p


class WCSPHDensity(_WCSPH):
    """density[i] = sum_j m W(d_ij) (Wendland C2, support 2h, self included) and
    pressure[i] = c0^2 rho0 / gamma ((rho/rho0)^gamma - 1)."""

    functor = _lib.PN_F_WCSPH_DENSITY


class WCSPHForce(_WCSPH):
    """accel[:, i] = -sum_j m (p_i/rho_i^2 + p_j/rho_j^2 + Pi_ij) grad W_ij with Monaghan
    viscosity; reads density, pressure and velocity (x must be y)."""

    functor = _lib.PN_F_WCSPH_FORCE


class WCSPHStep(_WCSPH):
    """WCSPHDensity followed by WCSPHForce in one call."""

    functor = _lib.PN_F_WCSPH_STEP


class _Adjoint(PairFunction):
    def __init__(self, *, density=None, terms=None, loss=None, grad=None, grad_scale=None,
                 mass=1.0, h=1.5, cutoff=3.0, lambda_pot=0.01, reuse_state=False):
        self.density, self.terms, self.loss = density, terms, loss
        self.grad, self.grad_scale = grad, grad_scale
        self.consts = dict(mass=float(mass), h=float(h), cutoff=float(cutoff),
                           lambda_pot=float(lambda_pot))
        self.reuse_state = bool(reuse_state)

    def params(self, nhs, x, y, n_q):
        torch = _torch()
        T = _tdtype(nhs)
        n = x.shape[1]
        p = _lib.pn_adjoint_params(reuse_state=int(self.reuse_state), **self.consts)
        for name, size, dt in (("density", n, T), ("terms", n, T), ("grad", n * nhs.ndims, T),
                               ("loss", 1, torch.float64), ("grad_scale", 1, torch.float64)):
            t = getattr(self, name)
            if t is not None:
                _out(t, name, size, dt)
                setattr(p, name, t.data_ptr())
        return p


class AdjointLossForward(_Adjoint):
    """L = sum_i (rho_i - 1)^2 + lambda E over the search's pairs (x must be y):
    density[i] = rho_i (Wendland C2, support 2h), terms[i] = (rho_i - 1)^2 + lambda/2 e_i
    with e_i = sum_{j != i, 0 < d < cutoff} m^2 (1/d - 1/cutoff), loss[0] = sum of the terms
    (FP64, fixed order).  Keeps (x, 2 (rho - 1)) in the search for AdjointLossBackward."""

    functor = _lib.PN_F_ADJOINT_FORWARD


class AdjointLossBackward(_Adjoint):
    """grad[i * d + k] = grad_scale * dL/dx_ik with the neighbour set fixed; reuse_state
    takes the state of the preceding AdjointLossForward call, otherwise it is rebuilt from
    `density`."""

    functor = _lib.PN_F_ADJOINT_BACKWARD


def foreach_point_neighbor(f, x, y, nhs: GridNeighborhoodSearch, *, points=None, check=True):
    """foreach_point_neighbor(f, x, y, nhs; points) (neighborhood_search.jl:183-201)."""
    if not isinstance(f, PairFunction):
        raise UnsupportedFunctorError(
            "only the compiled pair functions (CountNeighbors, NBodyAcceleration, "
            "TruncatedPotential, WCSPHDensity, WCSPHForce, WCSPHStep, NeighborIndexSum, "
            "AdjointLossForward, AdjointLossBackward) run "
            "on the GPU; an arbitrary Python callable cannot be compiled into the kernels")
    x, y = _bound(nhs, x, "x"), _bound(nhs, y, "y")
    pts = _index_tensor(points, x.shape[1], "points")
    n_q = x.shape[1] if pts is None else pts.numel()
    p = f.params(nhs, x, y, n_q)
    fn = lib().pn_pre_foreach_point_neighbor if getattr(nhs, "_precomputed", False) \
        else lib().pn_foreach_point_neighbor
    rc = fn(nhs._h, f.functor, _ptr(x), x.shape[1], _ptr(y), y.shape[1], _ptr(pts),
            0 if pts is None else pts.numel(), C.byref(p), _stream())
    _finish(nhs, rc, check, "foreach_point_neighbor")


def foreach_point_neighbor_unsafe(f, x, y, nhs, *, points=None, check=True):
    """foreach_point_neighbor_unsafe (neighborhood_search.jl:203-234): the reference skips
    its bounds checks of `points`; the device checks them anyway, so this is
    foreach_point_neighbor."""
    return foreach_point_neighbor(f, x, y, nhs, points=points, check=check)


def foreach_neighbor(f, system_coords, neighbor_coords, nhs, point, *, check=True):
    """foreach_neighbor(f, system_coords, neighbor_coords, nhs, point)
    (neighborhood_search.jl:250-267): the pair function over the neighbours of one point of
    `system_coords` (0-based here); its outputs are written at that point."""
    return foreach_point_neighbor(f, system_coords, neighbor_coords, nhs, points=[int(point)],
                                  check=check)


foreach_neighbor_unsafe = foreach_neighbor


def mapreduce_neighbor(f, op, system_coords, neighbor_coords, nhs, point, *, init):
    """mapreduce_neighbor(f, op, system_coords, neighbor_coords, nhs, point; init)
    (neighborhood_search.jl:360-421) for the reductions the library computes: `f` is
    "count" (the number of neighbours, self included) or "index" (the 1-based neighbour
    indices), `op` is `+` (operator.add or "+").  Returns init + the reduction; the empty
    neighbourhood returns init, like the reference."""
    import operator
    if op not in (operator.add, "+"):
        raise UnsupportedFunctorError("mapreduce_neighbor: only op = + is compiled")
    torch = _torch()
    x = _bound(nhs, system_coords, "system_coords")
    n = x.shape[1]
    if f == "count":
        out = torch.zeros(n, dtype=torch.int32, device="cuda")
        pf = CountNeighbors(out)
    elif f == "index":
        out = torch.zeros(n, dtype=torch.int64, device="cuda")
        pf = NeighborIndexSum(out)
    else:
        raise UnsupportedFunctorError("mapreduce_neighbor: f must be \"count\" or \"index\"")
    foreach_neighbor(pf, system_coords, neighbor_coords, nhs, point)
    return init + int(out[int(point)])


mapreduce_neighbor_unsafe = mapreduce_neighbor


def initialize_grid(nhs, y, *, eachindex_y=None, check=True):
    """initialize_grid!(nhs, y; eachindex_y) (nhs_grid.jl:227-281)."""
    return initialize(nhs, y, y, eachindex_y=eachindex_y, check=check)


def update_grid(nhs, y, *, eachindex_y=None, check=True):
    """update_grid!(nhs, y; eachindex_y) (nhs_grid.jl:292-477)."""
    return update(nhs, y, y, eachindex_y=eachindex_y, check=check)


def neighbor_lists(x, y, nhs: GridNeighborhoodSearch, *, points=None, sort=True):
    """All neighbour lists as CSR (offsets int64[n_q + 1], neighbors int32): the
    reference test's `push!(neighbors[point], neighbor)` (test/neighborhood_search.jl:
    325-336), rows sorted ascending when `sort`."""
    torch = _torch()
    if getattr(nhs, "_precomputed", False):
        if points is not None:
            raise ArgumentError("the precomputed search exports the lists of all points")
        return nhs._lists(sort)
    x, y = _bound(nhs, x, "x"), _bound(nhs, y, "y")
    pts = _index_tensor(points, x.shape[1], "points")
    n_q = x.shape[1] if pts is None else pts.numel()
    offsets = torch.empty(n_q + 1, dtype=torch.int64, device="cuda")
    p = _lib.pn_neighbor_list_params(0, offsets.data_ptr(), 0, 0, 1 if sort else 0, 0)
    args = (nhs._h, _lib.PN_F_NEIGHBOR_LIST, _ptr(x), x.shape[1], _ptr(y), y.shape[1],
            _ptr(pts), 0 if pts is None else pts.numel())
    rc = lib().pn_foreach_point_neighbor(*args, C.byref(p), _stream())
    _finish(nhs, rc, True, "neighbor lists (count)")
    total = int(offsets[-1])
    nbrs = torch.empty(max(total, 1), dtype=torch.int32, device="cuda")
    p.neighbors = nbrs.data_ptr()
    p.capacity = max(total, 1)
    rc = lib().pn_foreach_point_neighbor(*args, C.byref(p), _stream())
    _finish(nhs, rc, True, "neighbor lists")
    return offsets, nbrs[:total]


def cell_coords(coords, nhs: GridNeighborhoodSearch):
    """cell_coords(x, nhs) (nhs_grid.jl:622-638): the 1-based (periodic) cell of a point."""
    torch = _torch()
    x = torch.as_tensor(np.asarray(coords, dtype=nhs.coord_eltype).reshape(1, -1), device="cuda")
    out = torch.empty(nhs.ndims, dtype=torch.int64, device="cuda")
    rc = lib().pn_cell_coords(nhs._h, _ptr(x), 1, _ptr(out), _stream())
    _finish(nhs, rc, True, "cell_coords")
    return tuple(int(v) for v in out.cpu().tolist())


def export_cells(nhs: GridNeighborhoodSearch):
    """(counts[prod(grid_size)], points) with each cell's points ascending (0-based); for a
    SpatialHashingCellList, per hash list (counts[list_size])."""
    torch = _torch()
    gi = nhs.grid_info()
    n_total = gi["list_size"] or int(np.prod(gi["grid_size"]))
    counts = torch.empty(n_total, dtype=torch.int32, device="cuda")
    pts = torch.empty(max(int(gi["n_binned"]), 1), dtype=torch.int32, device="cuda")
    rc = lib().pn_export_cells(nhs._h, _ptr(counts), _ptr(pts), _stream())
    _finish(nhs, rc, True, "export_cells")
    c = counts.cpu().numpy()
    return c, pts.cpu().numpy()[: int(c.sum())]


def eachneighbor(coords, nhs: GridNeighborhoodSearch):
    """eachneighbor(coords, nhs) (nhs_grid.jl:585-591): the points in the 3^d cells around
    the cell of `coords` (0-based), read from the GPU cell list."""
    gi = nhs.grid_info()
    n = gi["grid_size"]
    c = cell_coords(coords, nhs)
    counts, pts = export_cells(nhs)
    starts = np.concatenate([[0], np.cumsum(counts)])
    d = nhs.ndims
    out = []
    if gi["list_size"] > 0:
        # SpatialHashingCellList: each cell's whole hash list, like points_in_cell
        rng = [range(-1, 2) if k < d else range(0, 1) for k in range(3)]
        for o3 in rng[2]:
            for o2 in rng[1]:
                for o1 in rng[0]:
                    cc = [c[0] + o1, c[1] + o2 if d > 1 else 0, c[2] + o3 if d > 2 else 0]
                    if nhs.periodic_box is not None:
                        for k in range(d):
                            cc[k] = (cc[k] - 2) % gi["n_cells"][k] + 2
                    h = spatial_hash(cc[:d], gi["list_size"])
                    out.extend(pts[starts[h]:starts[h + 1]].tolist())
        return np.asarray(out, dtype=np.int64)
    rng = [range(-1, 2) if k < d else range(0, 1) for k in range(3)]
    for o3 in rng[2]:
        for o2 in rng[1]:
            for o1 in rng[0]:
                cc = [c[0] + o1, (c[1] + o2) if d > 1 else 1, (c[2] + o3) if d > 2 else 1]
                if nhs.periodic_box is not None:
                    for k in range(d):
                        nc = gi["n_cells"][k]
                        cc[k] = (cc[k] - 2) % nc + 2
                if any(cc[k] < 1 or cc[k] > n[k] for k in range(d)):
                    raise BoundsError(f"cell {tuple(cc[:d])} is outside the grid")
                lin = (cc[0] - 1) + ((cc[1] - 1) * n[0] if d > 1 else 0) + \
                      ((cc[2] - 1) * n[0] * n[1] if d > 2 else 0)
                out.extend(pts[starts[lin]:starts[lin + 1]].tolist())
    return np.asarray(out, dtype=np.int64)


from .adjoint import adjoint_loss  # noqa: E402  (uses the API above)
from .batch import BatchedNeighborhoodSearch  # noqa: E402
from .precomputed import PrecomputedNeighborhoodSearch  # noqa: E402
