"""ctypes binding of libpn_gb300.so (the C ABI declared in include/pn_gb300.h).

This is the same binding a Julia `ccall` layer makes; the Python host API in __init__.py
is built on it.  Loading fails loudly if the library has not been built: there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# PN_GB300_LIB names another build of the library (the bounds-checked
# _build/libpn_gb300_bc.so, for instance); by default the in-tree libpn_gb300.so.
LIB_PATH = os.environ.get("PN_GB300_LIB") or os.path.join(HERE, "_build", "libpn_gb300.so")

PN_OK = 0
PN_ERR_OUT_OF_DOMAIN = 1
PN_ERR_INVALID_ARG = 2
PN_ERR_CUDA = 3
PN_ERR_TIMEOUT = 4
PN_ERR_UNSUPPORTED_FUNCTOR = 5
PN_ERR_CELL_FULL = 6
PN_ERR_NOT_INITIALIZED = 7
PN_ERR_OUT_OF_MEMORY = 8
PN_ERR_BOUNDS = 9
PN_ERR_CAPACITY = 10
PN_ERR_SCRATCH_LIMIT = 11
PN_ERR_INDEX = 12
PN_NOALLOC_SCRATCH_BYTES = 4 * 1024 * 1024
PN_FMA_PROBE_THREADS = 152 * 8 * 256

PN_FLOAT32, PN_FLOAT64 = 0, 1
PN_FLAG_FLOAT32_SEARCH = 1
PN_PARALLEL_UPDATE, PN_PARALLEL_INCREMENTAL_UPDATE = 0, 1

PN_F_COUNT = 0
PN_F_NEIGHBOR_LIST = 1
PN_F_NBODY_ACCEL = 2
PN_F_POTENTIAL = 3
PN_F_WCSPH_DENSITY = 4
PN_F_WCSPH_FORCE = 5
PN_F_WCSPH_STEP = 6
PN_F_INDEX_SUM = 7
PN_F_ADJOINT_FORWARD = 8
PN_F_ADJOINT_BACKWARD = 9

D3 = C.c_double * 3
I3 = C.c_int64 * 3


class pn_config(C.Structure):
    _fields_ = [
        ("ndims", C.c_int32), ("dtype", C.c_int32), ("search_radius", C.c_double),
        ("min_corner", D3), ("max_corner", D3), ("periodic", C.c_int32),
        ("update_strategy", C.c_int32), ("periodic_min", D3), ("periodic_max", D3),
        ("n_points", C.c_int64), ("max_points_per_cell", C.c_int32), ("flags", C.c_int32),
    ]


class pn_grid_info(C.Structure):
    _fields_ = [
        ("ndims", C.c_int32), ("dtype", C.c_int32), ("periodic", C.c_int32),
        ("is_template", C.c_int32), ("grid_size", I3), ("n_cells", I3),
        ("min_corner", D3), ("max_corner", D3), ("cell_size", D3),
        ("search_radius", C.c_double), ("n_binned", C.c_int64), ("n_overflow", C.c_int64),
        ("list_size", C.c_int64),
    ]


class pn_count_params(C.Structure):
    _fields_ = [("counts", C.c_void_p)]


class pn_index_sum_params(C.Structure):
    _fields_ = [("sums", C.c_void_p)]


class pn_neighbor_list_params(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("offsets", C.c_void_p), ("neighbors", C.c_void_p),
                ("capacity", C.c_int64), ("sort_rows", C.c_int32), ("pad_", C.c_int32)]


class pn_nbody_params(C.Structure):
    _fields_ = [("masses", C.c_void_p), ("G", C.c_double), ("accel", C.c_void_p)]


class pn_potential_params(C.Structure):
    _fields_ = [("masses", C.c_void_p), ("cutoff", C.c_double), ("energy", C.c_void_p)]


class pn_wcsph_params(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("h", C.c_double), ("c0", C.c_double), ("rho0", C.c_double),
        ("gamma_exp", C.c_double), ("alpha", C.c_double), ("eps_visc", C.c_double),
        ("r_min", C.c_double), ("density", C.c_void_p), ("pressure", C.c_void_p),
        ("velocity", C.c_void_p), ("accel", C.c_void_p), ("reuse_state", C.c_int32),
        ("pad_", C.c_int32),
    ]


class pn_adjoint_params(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("h", C.c_double), ("cutoff", C.c_double),
        ("lambda_pot", C.c_double), ("density", C.c_void_p), ("terms", C.c_void_p),
        ("loss", C.c_void_p), ("grad", C.c_void_p), ("grad_scale", C.c_void_p),
        ("reuse_state", C.c_int32), ("pad_", C.c_int32),
    ]


class pn_batch_schedule(C.Structure):
    _fields_ = [("block", C.c_int32), ("order", C.c_int32), ("persistent", C.c_int32),
                ("points_per_thread", C.c_int32)]


_P = C.c_void_p
_SIGNATURES = {
    "pn_abi_version": (C.c_int, []),
    "pn_launch_count": (C.c_ulonglong, []),
    "pn_build_flags": (C.c_int32, []),
    "pn_bounds_failure": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "pn_fma_probe": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "pn_selftest_bounded_wait": (C.c_int, [C.c_void_p]),
    "pn_create": (C.c_int, [C.POINTER(pn_config), C.POINTER(_P)]),
    "pn_create_from_grid": (C.c_int, [C.POINTER(pn_config), C.POINTER(C.c_int64), C.POINTER(_P)]),
    "pn_create_spatial_hashing": (C.c_int, [C.POINTER(pn_config), C.c_int64, C.POINTER(_P)]),
    "pn_copy_search": (C.c_int, [_P, C.c_double, C.c_int64, C.POINTER(_P)]),
    "pn_destroy": (C.c_int, [_P]),
    "pn_set_rebuild_fraction": (C.c_int, [_P, C.c_double]),
    "pn_set_pair_cache": (C.c_int, [_P, C.c_int32]),
    "pn_initialize": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int64, _P]),
    "pn_update": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int64, C.c_int32, _P]),
    "pn_foreach_point_neighbor": (C.c_int, [_P, C.c_int32, _P, C.c_int64, _P, C.c_int64,
                                            _P, C.c_int64, _P, _P]),
    "pn_sync": (C.c_int, [_P]),
    "pn_get_error": (C.c_int, [_P, C.c_int32]),
    "pn_status_string": (C.c_char_p, [C.c_int32]),
    "pn_requires_update": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "pn_get_grid_info": (C.c_int, [_P, C.POINTER(pn_grid_info)]),
    "pn_compute_geometry": (C.c_int, [C.POINTER(pn_config), C.POINTER(pn_grid_info)]),
    "pn_compute_geometry_from_grid": (C.c_int, [C.POINTER(pn_config), C.POINTER(C.c_int64),
                                                C.POINTER(pn_grid_info)]),
    "pn_cell_coords": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
    "pn_export_cells": (C.c_int, [_P, _P, _P, _P]),
    "pn_count_neighbors_noalloc": (C.c_int, [C.POINTER(pn_config), _P, C.c_int64, _P, _P]),
    "pn_pre_create": (C.c_int, [C.POINTER(pn_config), C.c_int32, C.POINTER(_P)]),
    "pn_pre_create_spatial_hashing": (C.c_int, [C.POINTER(pn_config), C.c_int64, C.c_int32,
                                                C.POINTER(_P)]),
    "pn_pre_destroy": (C.c_int, [_P]),
    "pn_pre_initialize": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int64, _P, C.c_int64, _P]),
    "pn_pre_update": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int64, _P, C.c_int64, C.c_int32,
                                C.c_int32, _P]),
    "pn_pre_foreach_point_neighbor": (C.c_int, [_P, C.c_int32, _P, C.c_int64, _P, C.c_int64,
                                                _P, C.c_int64, _P, _P]),
    "pn_pre_neighbor_lists": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, _P]),
    "pn_pre_sync": (C.c_int, [_P]),
    "pn_pre_requires_update": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "pn_batch_create": (C.c_int, [C.POINTER(pn_config), C.POINTER(C.c_int64), C.c_int32,
                                  C.POINTER(_P)]),
    "pn_batch_destroy": (C.c_int, [_P]),
    "pn_batch_initialize": (C.c_int, [_P, _P, _P]),
    "pn_batch_update": (C.c_int, [_P, _P, _P]),
    "pn_batch_foreach_point_neighbor": (C.c_int, [_P, C.c_int32, _P, _P, _P]),
    "pn_batch_autotune": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int32, _P]),
    "pn_batch_autotune_cached": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int32, C.c_char_p, _P]),
    "pn_batch_tune_key": (C.c_int, [_P, C.c_int32, C.c_char_p, C.c_int32]),
    "pn_tune_cache_lookup": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(pn_batch_schedule),
                                       C.POINTER(C.c_int32)]),
    "pn_tune_cache_store": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(pn_batch_schedule),
                                      C.c_double]),
    "pn_batch_get_schedule": (C.c_int, [_P, C.c_int32, C.POINTER(pn_batch_schedule)]),
    "pn_batch_set_schedule": (C.c_int, [_P, C.c_int32, C.POINTER(pn_batch_schedule)]),
    "pn_batch_capture_step": (C.c_int, [_P, _P, _P]),
    "pn_batch_launch_step": (C.c_int, [_P, _P]),
    "pn_batch_sync": (C.c_int, [_P]),
}

_lib = None


def load() -> C.CDLL:
    """Load libpn_gb300.so (built by build.py).  Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libpn_gb300.so is not built ({LIB_PATH}); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def status_string(status: int) -> str:
    return load().pn_status_string(int(status)).decode()
