"""C ABI checks that need no GPU: the library loads, exports every entry point that
include/pn_gb300.h declares, its structs have the layout the ctypes binding assumes, and the
host-side geometry (pn_compute_geometry) equals the oracle's restatement of the reference
constructors.  The Python host API's argument checks that run before any device call are
covered too."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "pn_gb300.h")


@pytest.fixture(scope="module")
def L(pkg):
    pkg.build.build()
    return pkg._lib


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|unsigned long long)\s+(pn_\w+)\s*\(",
                                 src, flags=re.M)))


def test_library_exports_every_declared_symbol(L):
    lib = L.load()
    names = declared_functions()
    assert len(names) >= 14
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (pn_\w+)$", out, flags=re.M))
    for n in names:
        assert n in exported, n
        getattr(lib, n)
    assert lib.pn_abi_version() == 1


def test_struct_layout_matches_header(L, tmp_path):
    structs = {"pn_config": L.pn_config, "pn_grid_info": L.pn_grid_info,
               "pn_count_params": L.pn_count_params,
               "pn_index_sum_params": L.pn_index_sum_params,
               "pn_neighbor_list_params": L.pn_neighbor_list_params,
               "pn_nbody_params": L.pn_nbody_params,
               "pn_potential_params": L.pn_potential_params,
               "pn_wcsph_params": L.pn_wcsph_params,
               "pn_adjoint_params": L.pn_adjoint_params,
               "pn_batch_schedule": L.pn_batch_schedule}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(){"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True,
                                                         text=True, check=True).stdout.split("\n") if l)
    for name, cls in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(got[f"{name}.{f}"]) == getattr(cls, f).offset, f"{name}.{f}"


def _geometry(L, ndims, dtype, r, mn, mx, box=None):
    cfg = L.pn_config()
    cfg.ndims = ndims
    cfg.dtype = L.PN_FLOAT32 if dtype == np.float32 else L.PN_FLOAT64
    cfg.search_radius = float(dtype(r))
    for k in range(ndims):
        cfg.min_corner[k] = float(dtype(mn[k]))
        cfg.max_corner[k] = float(dtype(mx[k]))
    if box is not None:
        cfg.periodic = 1
        for k in range(ndims):
            cfg.periodic_min[k] = float(dtype(box[0][k]))
            cfg.periodic_max[k] = float(dtype(box[1][k]))
    gi = L.pn_grid_info()
    rc = L.load().pn_compute_geometry(C.byref(cfg), C.byref(gi))
    return rc, gi


GEOMS = [
    (3, np.float64, 3.0, [-1.0] * 3, [51.0] * 3, None),           # 50^3 lattice, r = 3
    (3, np.float32, 3.0, [-1.0] * 3, [201.0] * 3, None),          # 200^3 lattice, r = 3
    (2, np.float32, 2.5, [0.0, 0.0], [4096.0, 4096.0], ([0.0, 0.0], [4096.0, 4096.0])),
    (2, np.float64, 0.1, [-0.1, -0.2], [0.2, 0.4], ([-0.1, -0.2], [0.2, 0.4])),
    (2, np.float64, 0.1, [-0.1, -0.2], [0.205, 0.43], ([-0.1, -0.2], [0.205, 0.43])),
    (3, np.float64, 0.1, [-0.1, -0.2, 0.05], [0.2, 0.4, 0.35], ([-0.1, -0.2, 0.05], [0.2, 0.4, 0.35])),
    (1, np.float64, 1.0, [0.0], [10.0], None),
    (2, np.float32, 3.0, [1.0, 1.0], [100.0, 100.0], None),
    (2, np.float32, 0.1, [0.0, 0.0], [1.0, 1.0], ([0.0, 0.0], [1.0, 1.0])),
]


@pytest.mark.parametrize("g", GEOMS)
def test_geometry_equals_oracle(L, O, g):
    ndims, dt, r, mn, mx, box = g
    rc, gi = _geometry(L, ndims, dt, r, mn, mx, box)
    assert rc == 0
    og = O.grid_create(ndims, dt(r), np.array(mn, dt), np.array(mx, dt),
                       periodic_box=None if box is None else (np.array(box[0], dt), np.array(box[1], dt)),
                       dtype=dt)
    for k in range(ndims):
        assert gi.grid_size[k] == og.n[k]
        assert gi.min_corner[k] == og.min_pad[k]
        assert gi.max_corner[k] == og.max_pad[k]
        assert gi.cell_size[k] == og.cell_size[k]
        assert gi.n_cells[k] == og.n_cells[k]


MIXED_GEOMS = [
    (3, 0.9, [0.0, 0.0, 0.0], [6.0, 5.0, 7.3], None),
    (3, 0.9, [0.0, 0.0, 0.0], [6.0, 5.0, 7.3], ([0.0, 0.0, 0.0], [6.0, 5.0, 7.3])),
    (2, 0.1, [-0.1, -0.2], [0.205, 0.43], ([-0.1, -0.2], [0.205, 0.43])),
    (2, 1.7, [-3.0, -3.0], [5.0, 3.0], None),
]


@pytest.mark.parametrize("g", MIXED_GEOMS)
def test_mixed_geometry_equals_oracle(L, O, g):
    """Float64 corners with a Float32 radius and PeriodicBox (PN_FLAG_FLOAT32_SEARCH)."""
    ndims, r, mn, mx, box = g
    r32 = np.float32(r)
    cfg = L.pn_config()
    cfg.ndims = ndims
    cfg.dtype = L.PN_FLOAT64
    cfg.flags = L.PN_FLAG_FLOAT32_SEARCH
    cfg.search_radius = float(r32)
    lo, hi = (np.array(mn) - r, np.array(mx) + r) if box is None else (np.array(mn), np.array(mx))
    for k in range(ndims):
        cfg.min_corner[k], cfg.max_corner[k] = lo[k], hi[k]
    if box is not None:
        cfg.periodic = 1
        for k in range(ndims):
            cfg.periodic_min[k] = float(np.float32(box[0][k]))
            cfg.periodic_max[k] = float(np.float32(box[1][k]))
    gi = L.pn_grid_info()
    assert L.load().pn_compute_geometry(C.byref(cfg), C.byref(gi)) == 0
    pb = None if box is None else (np.array(box[0]), np.array(box[1]))
    og = O.grid_create_mixed(ndims, r32, lo, hi, periodic_box=pb)
    for k in range(ndims):
        assert gi.grid_size[k] == og.n[k]
        assert gi.min_corner[k] == og.min_pad[k]
        assert gi.max_corner[k] == og.max_pad[k]
        assert gi.cell_size[k] == og.cell_size[k]
        assert gi.n_cells[k] == og.n_cells[k]
    assert gi.search_radius == float(r32)
    # the flag needs Float64 coordinates; unknown flags are rejected
    cfg.dtype = L.PN_FLOAT32
    assert L.load().pn_compute_geometry(C.byref(cfg), C.byref(gi)) == L.PN_ERR_INVALID_ARG
    cfg.dtype = L.PN_FLOAT64
    cfg.flags = 2
    assert L.load().pn_compute_geometry(C.byref(cfg), C.byref(gi)) == L.PN_ERR_INVALID_ARG


def test_mixed_cell_list_corners(pkg):
    """FullGridCellList(Float64 corners, Float32 radius): Float64 corners padded by the
    Float32 value Float32(1001 // 1000) * r (full_grid.jl:65-67); the search is mixed."""
    P = pkg
    r = np.float32(0.3)
    cl = P.FullGridCellList(min_corner=[0.1, 0.2], max_corner=[1.0, 2.0], search_radius=r)
    pad = float(np.float32(np.float32(1001) / np.float32(1000)) * r)
    assert cl.eltype == np.float64
    assert list(cl.min_corner) == [0.1 - pad, 0.2 - pad]
    assert list(cl.max_corner) == [1.0 + pad, 2.0 + pad]
    cl32 = P.FullGridCellList(min_corner=np.zeros(2, np.float32), max_corner=np.ones(2, np.float32),
                              search_radius=r)
    assert cl32.eltype == np.float32


def test_geometry_known_values(L):
    # test/cell_lists/full_grid.jl:28-29
    rc, gi = _geometry(L, 3, np.float64, 1.0, [0.0] * 3, [10.0] * 3)
    assert rc == 0 and list(gi.min_corner) == [-1.001] * 3 and list(gi.max_corner) == [11.001] * 3
    # the 2D periodic n-body workload: 1638 periodic cells of 4096/1638, 1641 grid cells
    rc, gi = _geometry(L, 2, np.float32, 2.5, [0.0, 0.0], [4096.0, 4096.0],
                       ([0.0, 0.0], [4096.0, 4096.0]))
    assert rc == 0 and gi.n_cells[0] == 1638 and gi.grid_size[0] == 1641
    assert gi.cell_size[0] == float(np.float32(4096.0) / np.float32(1638))
    # fewer than 3 periodic cells is an ArgumentError (nhs_grid.jl:120-124)
    rc, _ = _geometry(L, 2, np.float64, 1.0, [0.0, 0.0], [2.5, 2.5], ([0.0, 0.0], [2.5, 2.5]))
    assert rc == L.PN_ERR_INVALID_ARG


def test_normal_build_is_not_bounds_checked(L):
    """The in-tree library is the normal build; the checked one (PN_BOUNDS_CHECK) is a
    separate file with bit 0 of pn_build_flags set."""
    assert L.load().pn_build_flags() == 0
    assert L.status_string(L.PN_ERR_INDEX) == "a device index out of range (bounds-checked build)"


def test_status_strings_are_the_references(L):
    assert L.status_string(L.PN_ERR_OUT_OF_DOMAIN) == \
        "particle coordinates are NaN or outside the domain bounds of the cell list"
    assert L.status_string(L.PN_ERR_CELL_FULL) == \
        "cell list is full. Use a larger `max_points_per_cell`."


def test_host_api_argument_errors(pkg):
    P = pkg
    with pytest.raises(P.ArgumentError, match="same length"):
        P.FullGridCellList(min_corner=[0.0, 0.0, 0.0], max_corner=[1.0, 1.0])
    with pytest.raises(P.ArgumentError, match="up to 100 dimensions"):
        P.FullGridCellList(min_corner=np.zeros(101), max_corner=np.ones(101))
    cl3 = P.FullGridCellList(min_corner=[0.0] * 3, max_corner=[1.0] * 3, search_radius=1.0)
    assert list(cl3.min_corner) == [-1.001] * 3 and list(cl3.max_corner) == [2.001] * 3
    with pytest.raises(P.ArgumentError, match="a 2D cell list is required for a GridNeighborhoodSearch"):
        P.GridNeighborhoodSearch(2, search_radius=1.0, cell_list=cl3)
    with pytest.raises(P.ArgumentError, match="is not a valid update strategy"):
        P.GridNeighborhoodSearch(3, search_radius=1.0, cell_list=cl3, update_strategy="test")
    # the reference's five strategies for a FullGridCellList, two for spatial hashing
    for strat in (P.ParallelUpdate(), P.ParallelIncrementalUpdate(), P.SemiParallelUpdate(),
                  P.SerialIncrementalUpdate(), P.SerialUpdate()):
        assert P.check_update_strategy(cl3, strat) is strat
    assert P.check_update_strategy(cl3, None) == P.ParallelUpdate()
    hl = P.SpatialHashingCellList(3, list_size=10)
    assert P.check_update_strategy(hl, P.SerialUpdate()) == P.SerialUpdate()
    with pytest.raises(P.ArgumentError, match=r"Available options are \(ParallelUpdate, "
                                              r"SerialUpdate\)"):
        P.check_update_strategy(hl, P.SemiParallelUpdate())
    with pytest.raises(P.ArgumentError, match="cannot be an integer type"):
        P.GridNeighborhoodSearch(3, search_radius=1, cell_list=cl3)
    box32 = P.PeriodicBox(min_corner=np.zeros(3, np.float32), max_corner=np.ones(3, np.float32))
    with pytest.raises(P.ArgumentError, match="same element type"):
        P.GridNeighborhoodSearch(3, search_radius=1.0, cell_list=cl3, periodic_box=box32)
    assert P.requires_update(None) == (False, True)
    with pytest.raises(P.UnsupportedFunctorError):
        P.foreach_point_neighbor(lambda i, j, pd, d: None, None, None, None)


def _cfg_from_grid(L, ndims, dtype, r, corners_lo, corners_hi, box=None):
    cfg = L.pn_config()
    cfg.ndims = ndims
    cfg.dtype = L.PN_FLOAT32 if dtype == np.float32 else L.PN_FLOAT64
    cfg.search_radius = float(dtype(r))
    for k in range(ndims):
        cfg.min_corner[k] = corners_lo[k]
        cfg.max_corner[k] = corners_hi[k]
    if box is not None:
        cfg.periodic = 1
        for k in range(ndims):
            cfg.periodic_min[k] = float(dtype(box[0][k]))
            cfg.periodic_max[k] = float(dtype(box[1][k]))
    return cfg


@pytest.mark.parametrize("g", GEOMS + [(3, np.float64, 3.0, [-1.0] * 3, [101.0] * 3, None),
                                       (3, np.float64, 1.0, [0.0] * 3, [10.0] * 3, None)])
def test_geometry_from_grid_state(L, g):
    """pn_compute_geometry_from_grid takes a reference FullGridCellList's stored state -- its
    padded corners and size(linear_indices) -- as it is and gives the geometry the
    constructor computed from the unpadded corners, bit for bit.  (Removing the padding
    from the stored corners and padding again is not an identity in floating point; the
    cases where that round trip moves a corner are listed by this test's second half.)"""
    ndims, dt, r, mn, mx, box = g
    rc, gi = _geometry(L, ndims, dt, r, mn, mx, box)
    assert rc == 0
    grid = (C.c_int64 * 3)(*[gi.grid_size[k] if k < ndims else 0 for k in range(3)])
    cfg = _cfg_from_grid(L, ndims, dt, r, list(gi.min_corner), list(gi.max_corner), box)
    g2 = L.pn_grid_info()
    assert L.load().pn_compute_geometry_from_grid(C.byref(cfg), grid, C.byref(g2)) == 0
    for k in range(ndims):
        assert g2.grid_size[k] == gi.grid_size[k]
        assert g2.min_corner[k] == gi.min_corner[k] and g2.max_corner[k] == gi.max_corner[k]
        assert g2.cell_size[k] == gi.cell_size[k] and g2.n_cells[k] == gi.n_cells[k]
    # the naive route: unpad the stored corners in T, then construct as usual
    pad = dt(dt(1001) / dt(1000)) * dt(r)
    lo = [float(dt(dt(gi.min_corner[k]) + pad)) for k in range(ndims)]
    hi = [float(dt(dt(gi.max_corner[k]) - pad)) for k in range(ndims)]
    rc3, g3 = _geometry(L, ndims, dt, r, lo, hi, box)
    moved = rc3 != 0 or any(g3.min_corner[k] != gi.min_corner[k] or
                            g3.max_corner[k] != gi.max_corner[k] or
                            g3.grid_size[k] != gi.grid_size[k] for k in range(ndims))
    exact_inputs = all(float(dt(mn[k])) == lo[k] and float(dt(mx[k])) == hi[k]
                       for k in range(ndims))
    # where unpadding recovers the constructor's corners the naive route agrees; only
    # where it does not can the geometry move (hence the stored state is taken as it is)
    assert not (moved and exact_inputs)


def test_geometry_from_grid_golden_corners(L, golden):
    """test/cell_lists/full_grid.jl:28-29: corners 0 and 10 with radius 1 are stored as
    -1.001 and 11.001; from that stored state the search has the same 13 cells."""
    c = golden["full_grid_bounds"]
    rc, gi = _geometry(L, 3, np.float64, c["radius"], [c["min_corner"]] * 3,
                       [c["max_corner"]] * 3)
    assert rc == 0 and gi.min_corner[0] == c["expected_min_pad"]
    assert gi.max_corner[0] == c["expected_max_pad"]
    cfg = _cfg_from_grid(L, 3, np.float64, c["radius"], [c["expected_min_pad"]] * 3,
                         [c["expected_max_pad"]] * 3)
    g2 = L.pn_grid_info()
    grid = (C.c_int64 * 3)(*gi.grid_size)
    assert L.load().pn_compute_geometry_from_grid(C.byref(cfg), grid, C.byref(g2)) == 0
    assert list(g2.grid_size) == list(gi.grid_size) == [13, 13, 13]
    # a template (radius 0) stores no cells; a non-template needs at least one per dimension
    cfg0 = _cfg_from_grid(L, 3, np.float64, 0.0, [0.0] * 3, [10.0] * 3)
    assert L.load().pn_compute_geometry_from_grid(C.byref(cfg0), (C.c_int64 * 3)(0, 0, 0),
                                                  C.byref(g2)) == 0 and g2.is_template
    bad = (C.c_int64 * 3)(13, 0, 13)
    assert L.load().pn_compute_geometry_from_grid(C.byref(cfg), bad, C.byref(g2)) == L.PN_ERR_INVALID_ARG


def test_periodic_argument_errors(pkg):
    """The reference's message only for fewer than 3 periodic cells (nhs_grid.jl:113-116);
    a cell list that does not cover the periodic box gets its own reason.  Both are
    rejected by the host-side geometry, before any device call."""
    P = pkg
    box = P.PeriodicBox(min_corner=np.zeros(2), max_corner=np.full(2, 5.0))
    cl = P.FullGridCellList(min_corner=np.zeros(2), max_corner=np.full(2, 5.0),
                            search_radius=2.0)
    with pytest.raises(P.ArgumentError, match="needs at least 3 cells"):
        P.GridNeighborhoodSearch(2, search_radius=2.0, periodic_box=box, cell_list=cl)
    box = P.PeriodicBox(min_corner=np.zeros(2), max_corner=np.full(2, 30.0))
    small = P.FullGridCellList(min_corner=np.zeros(2), max_corner=np.full(2, 10.0),
                               search_radius=1.0)
    with pytest.raises(P.ArgumentError, match="must cover the periodic box"):
        P.GridNeighborhoodSearch(2, search_radius=1.0, periodic_box=box, cell_list=small)


def test_tune_cache_round_trip(L, tmp_path):
    """The batched autotuner's schedule cache (pn_tune_cache_store / _lookup) on the host:
    stored schedules come back by key, a store replaces the key's entry, unreadable lines
    and invalid schedules are ignored or rejected."""
    lib = L.load()
    path = str(tmp_path / "schedules.txt").encode()
    s = L.pn_batch_schedule(256, 1, 0, 2)
    found = C.c_int32(-1)
    out = L.pn_batch_schedule()
    assert lib.pn_tune_cache_lookup(path, b"batch/force/f32/d3/r2.75/n2^24/c2^9", C.byref(out),
                                    C.byref(found)) == 0 and found.value == 0
    assert lib.pn_tune_cache_store(path, b"batch/force/f32/d3/r2.75/n2^24/c2^9", C.byref(s),
                                   3.25) == 0
    assert lib.pn_tune_cache_store(path, b"batch/density/f32/d3/r2.75/n2^24/c2^9",
                                   C.byref(L.pn_batch_schedule(64, 0, 1, 1)), 2.5) == 0
    assert lib.pn_tune_cache_lookup(path, b"batch/force/f32/d3/r2.75/n2^24/c2^9", C.byref(out),
                                    C.byref(found)) == 0 and found.value == 1
    assert (out.block, out.order, out.persistent, out.points_per_thread) == (256, 1, 0, 2)
    # a store replaces the entry of its key and keeps the others
    assert lib.pn_tune_cache_store(path, b"batch/force/f32/d3/r2.75/n2^24/c2^9",
                                   C.byref(L.pn_batch_schedule(128, 0, 0, 1)), 1.0) == 0
    lines = open(path.decode()).read().splitlines()
    assert len(lines) == 2 and lines[0].startswith("batch/force/") and " 128 0 0 1 " in lines[0]
    lib.pn_tune_cache_lookup(path, b"batch/density/f32/d3/r2.75/n2^24/c2^9", C.byref(out),
                             C.byref(found))
    assert found.value == 1 and (out.block, out.persistent) == (64, 1)
    # unreadable lines are skipped; invalid schedules and keys are rejected
    with open(path.decode(), "a") as f:
        f.write("garbage\nbatch/count 7 0 0 1 1.0\n")
    lib.pn_tune_cache_lookup(path, b"batch/count", C.byref(out), C.byref(found))
    assert found.value == 0
    assert lib.pn_tune_cache_store(path, b"k", C.byref(L.pn_batch_schedule(96, 0, 0, 1)),
                                   1.0) == L.PN_ERR_INVALID_ARG
    assert lib.pn_tune_cache_store(path, b"bad key", C.byref(s), 1.0) == L.PN_ERR_INVALID_ARG
