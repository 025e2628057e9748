"""PrecomputedNeighborhoodSearch (nhs_precomputed.jl): neighbour lists computed by a
GridNeighborhoodSearch over a FullGridCellList at initialize!/update!, walked by every
foreach_point_neighbor.  The lists live in libpn_gb300 (pn_pre_* entry points): per query,
slots of the grid search's cell-sorted arrays, in groups of 32 rows stored transposed."""
from __future__ import annotations

import ctypes as C

from . import (ArgumentError, GridNeighborhoodSearch, PointNeighborsError,
               SpatialHashingCellList, _coords, _finish, _lib, _ptr, _raise, _stream, _torch,
               lib)

# nhs_precomputed.jl:113-124
_MAX_NEIGHBORS = {1: 32, 2: 64, 3: 320}


class PrecomputedNeighborhoodSearch:
    """PrecomputedNeighborhoodSearch{ndims}(; search_radius, n_points, periodic_box,
    update_strategy, update_neighborhood_search, max_neighbors, sort_neighbor_lists,
    transpose_backend) (nhs_precomputed.jl:89-111).

    The lists are computed by a GridNeighborhoodSearch: pass it as
    `update_neighborhood_search`, or pass `cell_list` (a FullGridCellList) and the search is
    built from the other arguments.  `max_neighbors` is the reference's capacity per point
    (a point with more neighbours is the "cell list is full" error; 0 = no limit).  The
    lists are always stored transposed in groups of 32 rows (the layout the reference's
    transpose_backend = true selects for GPUs); `transpose_backend` is accepted for
    compatibility."""

    _precomputed = True

    def __init__(self, ndims, *, search_radius=0.0, n_points=0, periodic_box=None,
                 update_strategy=None, update_neighborhood_search=None, cell_list=None,
                 max_neighbors=None, sort_neighbor_lists=True, transpose_backend=False):
        if update_neighborhood_search is None:
            update_neighborhood_search = GridNeighborhoodSearch(
                ndims, search_radius=search_radius, n_points=0, periodic_box=periodic_box,
                cell_list=cell_list, update_strategy=update_strategy)
        grid = update_neighborhood_search
        if not isinstance(grid, GridNeighborhoodSearch) or grid.ndims != ndims:
            raise ArgumentError("the lists are computed by a GridNeighborhoodSearch of the "
                                "same dimension")
        if max_neighbors is None:
            max_neighbors = _MAX_NEIGHBORS.get(int(ndims))
            if max_neighbors is None:
                raise ArgumentError("`NDIMS` must be 1, 2, or 3")
        self.ndims = int(ndims)
        self.eltype = grid.eltype
        self.coord_eltype = grid.coord_eltype
        self.mixed = grid.mixed
        self.search_radius = grid.search_radius
        self.n_points = int(n_points)
        self.periodic_box = grid.periodic_box
        self.cell_list = grid.cell_list
        self.update_strategy = grid.update_strategy
        self.max_neighbors = int(max_neighbors)
        self.sort_neighbor_lists = bool(sort_neighbor_lists)
        self.transpose_backend = bool(transpose_backend)
        self.neighborhood_search = grid
        cfg = _lib.pn_config()
        C.pointer(cfg)[0] = grid._cfg
        cfg.n_points = self.n_points
        h = C.c_void_p()
        if isinstance(grid.cell_list, SpatialHashingCellList):
            rc = lib().pn_pre_create_spatial_hashing(C.byref(cfg), grid.cell_list.list_size,
                                                     self.max_neighbors, C.byref(h))
        else:
            rc = lib().pn_pre_create(C.byref(cfg), self.max_neighbors, C.byref(h))
        if rc != _lib.PN_OK:
            _raise(rc, "PrecomputedNeighborhoodSearch")
        self._h = h
        self._cfg = cfg

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().pn_pre_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def _sync(self) -> int:
        return lib().pn_pre_sync(self._h)

    def _clear_error(self):
        lib().pn_pre_sync(self._h)

    def _points(self, x, y):
        y_src = y
        y = _coords(self, y, "y")
        x = y if x is y_src else _coords(self, x, "x")
        return x, y, y_src

    def _check_eachindex(self, eachindex_y, n_y):
        if eachindex_y is not None and not (isinstance(eachindex_y, range) and
                                            eachindex_y == range(n_y)):
            raise PointNeighborsError("this neighborhood search does not support inactive "
                                      "points")

    def _initialize(self, x, y, eachindex_y, check):
        x, y, y_src = self._points(x, y)
        self._check_eachindex(eachindex_y, y.shape[1])
        rc = lib().pn_pre_initialize(self._h, _ptr(x), x.shape[1], _ptr(y), y.shape[1], None,
                                     0, _stream())
        self._y_src, self._y_keep, self._x_keep = y_src, y, x
        _finish(self, rc, check, "initialize!")
        return self

    def _update(self, x, y, points_moving, eachindex_y, check):
        x, y, y_src = self._points(x, y)
        self._check_eachindex(eachindex_y, y.shape[1])
        rc = lib().pn_pre_update(self._h, _ptr(x), x.shape[1], _ptr(y), y.shape[1], None, 0,
                                 int(bool(points_moving[0])), int(bool(points_moving[1])),
                                 _stream())
        self._y_src, self._y_keep, self._x_keep = y_src, y, x
        _finish(self, rc, check, "update!")
        return self

    def _lists(self, sort):
        """CSR (offsets int64[n_x + 1], neighbors int32) of the stored lists, point indices
        (0-based), rows sorted ascending when `sort` (the reference's sorteach!)."""
        torch = _torch()
        n = self._x_keep.shape[1]
        offsets = torch.empty(n + 1, dtype=torch.int64, device="cuda")
        rc = lib().pn_pre_neighbor_lists(self._h, int(sort), _ptr(offsets), None, 0, _stream())
        _finish(self, rc, True, "neighbor lists (count)")
        total = int(offsets[-1])
        nbrs = torch.empty(max(total, 1), dtype=torch.int32, device="cuda")
        rc = lib().pn_pre_neighbor_lists(self._h, int(sort), _ptr(offsets), _ptr(nbrs),
                                         max(total, 1), _stream())
        _finish(self, rc, True, "neighbor lists")
        return offsets, nbrs[:total]

    def _copy(self, search_radius, n_points):
        from . import copy_neighborhood_search
        grid = copy_neighborhood_search(self.neighborhood_search, search_radius, n_points)
        return PrecomputedNeighborhoodSearch(
            self.ndims, n_points=n_points, update_neighborhood_search=grid,
            max_neighbors=self.max_neighbors, sort_neighbor_lists=self.sort_neighbor_lists,
            transpose_backend=self.transpose_backend)
