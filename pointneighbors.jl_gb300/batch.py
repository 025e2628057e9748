"""The batched form: many independent 3D Float32 clouds, each described by its own
GridNeighborhoodSearch (corners, search radius, n_points), searched together through
libpn_gb300's pn_batch_* entry points.

The reference has no batched search; with it each cloud is a separate search whose
update!/foreach_point_neighbor launches its own kernels.  Here all clouds share one set of
device arrays: coordinates are one (3, N) tensor with the clouds' points concatenated in
order (global point index = cloud offset + local index), and outputs are indexed the same
way.  A step is a few launches whatever the number of clouds, and update! + the WCSPH step
can be captured once in a CUDA graph and replayed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import (ArgumentError, CountNeighbors, GridNeighborhoodSearch, PairFunction,
               WCSPHDensity, WCSPHForce, WCSPHStep, _coords, _lib, _out, _raise, _stream,
               _tdtype, lib)


def _batch_params(f: PairFunction, nhs_list, x, n_total):
    """One C parameter struct per cloud.  WCSPH constants may be scalars or sequences with
    one value per cloud; output arrays are global (indexed by global point index)."""
    n = len(nhs_list)
    if isinstance(f, CountNeighbors):
        arr = (_lib.pn_count_params * n)()
        _out(f.counts, "counts", n_total, f.counts.dtype)
        for k in range(n):
            arr[k] = _lib.pn_count_params(f.counts.data_ptr())
        return arr
    if isinstance(f, (WCSPHDensity, WCSPHForce, WCSPHStep)):
        arr = (_lib.pn_wcsph_params * n)()
        T = _tdtype(nhs_list[0])
        ptrs = {}
        for name, size in (("density", n_total), ("pressure", n_total),
                           ("velocity", 3 * n_total), ("accel", 3 * n_total)):
            t = getattr(f, name)
            if t is not None:
                _out(t, name, size, T)
                ptrs[name] = t.data_ptr()
        for k in range(n):
            consts = {key: float(np.broadcast_to(v, (n,))[k]) for key, v in f.consts.items()}
            r_min = f.r_min
            if r_min is None:
                r_min = float(np.sqrt(np.finfo(np.float32).eps)) * consts["h"]
            arr[k] = _lib.pn_wcsph_params(r_min=float(np.broadcast_to(r_min, (n,))[k]),
                                          reuse_state=int(f.reuse_state), **consts, **ptrs)
        return arr
    raise ArgumentError(f"{type(f).__name__} is not available in the batched form "
                        "(CountNeighbors, WCSPHDensity, WCSPHForce, WCSPHStep are)")


class BatchedNeighborhoodSearch:
    """Many `GridNeighborhoodSearch(3, ...)` (Float32, no periodic box) searched together.

    `searches`: one search per cloud; each gives its cloud's FullGridCellList corners,
    search radius and `n_points`.  The batch owns its own device arrays (the searches are
    only read for their configuration)."""

    def __init__(self, searches):
        searches = list(searches)
        if not searches:
            raise ArgumentError("a batch needs at least one search")
        for s in searches:
            if not isinstance(s, GridNeighborhoodSearch) or s.ndims != 3 or \
                    s.coord_eltype != np.float32 or s.periodic_box is not None:
                raise ArgumentError("the batched form takes 3D Float32 searches without a "
                                    "periodic box")
        n = len(searches)
        cfgs = (_lib.pn_config * n)(*[s._cfg for s in searches])
        counts = (C.c_int64 * n)(*[int(s.n_points) for s in searches])
        h = C.c_void_p()
        rc = lib().pn_batch_create(cfgs, counts, n, C.byref(h))
        if rc != _lib.PN_OK:
            _raise(rc, "BatchedNeighborhoodSearch")
        self._h = h
        self.searches = searches
        self.n_points = np.asarray([s.n_points for s in searches], dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.n_points)])
        self.n_total = int(self.offsets[-1])
        self._keep = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().pn_batch_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    def _coords(self, x):
        x = _coords(self.searches[0], x, "x")
        if x.shape[1] != self.n_total:
            raise ArgumentError(f"the batch has {self.n_total} points, got {x.shape[1]}")
        return x

    def _check(self, rc, check, what):
        if rc != _lib.PN_OK:
            lib().pn_batch_sync(self._h)
            _raise(rc, what)
        if check:
            st = lib().pn_batch_sync(self._h)
            if st != _lib.PN_OK:
                _raise(st, what)

    def initialize(self, x, *, check=True):
        x = self._coords(x)
        self._x = x
        self._check(lib().pn_batch_initialize(self._h, C.c_void_p(x.data_ptr()), _stream()),
                    check, "initialize!")
        return self

    def update(self, x, *, check=True):
        x = self._coords(x)
        self._x = x
        self._check(lib().pn_batch_update(self._h, C.c_void_p(x.data_ptr()), _stream()),
                    check, "update!")
        return self

    def foreach_point_neighbor(self, f, x, *, check=True):
        x = self._coords(x)
        p = _batch_params(f, self.searches, x, self.n_total)
        self._keep = p
        self._check(lib().pn_batch_foreach_point_neighbor(self._h, f.functor,
                                                           C.c_void_p(x.data_ptr()), p,
                                                           _stream()), check,
                    "foreach_point_neighbor")

    def autotune(self, f, x, reps=3, cache=None):
        """Time the 24 tile schedules for `f`'s sweep and keep the fastest; returns it.  With
        `cache` (a file path) a schedule stored there for this batch's key is taken untimed,
        and a newly timed winner is stored."""
        x = self._coords(x)
        p = _batch_params(f, self.searches, x, self.n_total)
        functor = f.functor
        if cache is None:
            rc = lib().pn_batch_autotune(self._h, functor, C.c_void_p(x.data_ptr()), p,
                                         int(reps), _stream())
        else:
            rc = lib().pn_batch_autotune_cached(self._h, functor, C.c_void_p(x.data_ptr()), p,
                                                int(reps), str(cache).encode(), _stream())
        self._check(rc, True, "autotune")
        return self.schedule(functor)

    def tune_key(self, functor):
        buf = C.create_string_buffer(256)
        rc = lib().pn_batch_tune_key(self._h, int(functor), buf, 256)
        if rc != _lib.PN_OK:
            _raise(rc, "tune_key")
        return buf.value.decode()

    def schedule(self, functor):
        s = _lib.pn_batch_schedule()
        rc = lib().pn_batch_get_schedule(self._h, int(functor), C.byref(s))
        if rc != _lib.PN_OK:
            _raise(rc, "schedule")
        return {"block": s.block, "order": s.order, "persistent": s.persistent,
                "points_per_thread": max(1, s.points_per_thread)}

    def set_schedule(self, functor, block, order, persistent, points_per_thread=1):
        s = _lib.pn_batch_schedule(int(block), int(order), int(persistent),
                                   int(points_per_thread))
        rc = lib().pn_batch_set_schedule(self._h, int(functor), C.byref(s))
        if rc != _lib.PN_OK:
            _raise(rc, "set_schedule")

    def capture_step(self, x, f: WCSPHStep):
        """Capture update!(x) + the WCSPH density and force sweeps of every cloud into a
        CUDA graph; `x` and `f`'s arrays must stay at their addresses for the replays."""
        x = self._coords(x)
        p = _batch_params(f, self.searches, x, self.n_total)
        self._graph_keep = (x, p, f)
        rc = lib().pn_batch_capture_step(self._h, C.c_void_p(x.data_ptr()), p)
        if rc != _lib.PN_OK:
            _raise(rc, "capture_step")

    def launch_step(self, *, check=False):
        self._check(lib().pn_batch_launch_step(self._h, _stream()), check, "launch_step")

    def sync(self):
        st = lib().pn_batch_sync(self._h)
        if st != _lib.PN_OK:
            _raise(st, "batch")
