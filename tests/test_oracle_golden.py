"""Pin the CPU oracle against the known answers of the reference's own test suite.

The reference (Julia) cannot run here, so these vectors -- transcribed from its tests in
tests/golden/make_golden.py -- are what makes the oracle trustworthy as the answer the
CUDA path is compared with.  CPU only.
"""
import numpy as np
import pytest

from conftest import jfloat


def test_floor_to_int_saturates(O):
    # src/util.jl:19-34
    t63 = 2**63 - 1
    for dt in (np.float32, np.float64):
        assert O.floor_to_int(float("inf"), dt) == t63
        assert O.floor_to_int(float("nan"), dt) == t63
        assert O.floor_to_int(-float("inf"), dt) == -t63 - 1
        assert O.floor_to_int(2.0**63, dt) == t63
        assert O.floor_to_int(-(2.0**63), dt) == -t63 - 1
        assert O.floor_to_int(-1.5, dt) == -2
        assert O.floor_to_int(2.9999, dt) == 2


def test_cell_coords_limits(O, golden):
    c = golden["cell_coords_limits"]
    gd = O.grid_create(2, c["radius"], [0.0, 0.0], [1.0, 1.0])  # geometry only
    gf = O.grid_create(2, c["radius"], c["full_grid"]["min_corner"], c["full_grid"]["max_corner"])
    for x, ed, ef in zip(c["coords"], c["dict_expected"], c["full_expected"]):
        xv = np.array([jfloat(v) for v in x])
        assert O.cell_coords_dict(gd, xv) == tuple(ed)
        assert O.cell_coords(gf, xv) == tuple(ef)


def _dict_grid(O, ndims, r, box=None):
    mn = [0.0] * ndims
    mx = [1.0] * ndims
    return O.grid_create(ndims, r, mn, mx, periodic_box=box)


@pytest.mark.parametrize("case", ["rect_2d", "rect_3d"])
def test_rectangular_candidates_dictionary(O, golden, case):
    c = golden[case]
    base = np.array(c["coords"])
    d = base.shape[1]
    for chk in c["checks"]:
        y = base + np.array(chk["shift"])
        q = np.array(chk["query"])
        if chk.get("query_shifted"):
            q = q + np.array(chk["shift"])
        g = _dict_grid(O, d, chk["radius"])
        got = sorted((O.eachneighbor_dict(g, y, q) + 1).tolist())
        assert got == chk["expected"]


def test_eachindex_y_full_grid(O, golden):
    c = golden["eachindex_y_3d"]
    c1 = np.array(c["coords"])
    shift = np.array(c["shift"])
    c2 = c1 + shift
    mn = np.minimum(c1.min(axis=0), c2.min(axis=0))
    mx = np.maximum(c1.max(axis=0), c2.max(axis=0))
    g = O.grid_create(3, c["radius"], mn, mx)
    O.build(g, c1)  # initialize! with all points
    lo, hi = c["eachindex_y"]
    cl = O.build(g, c2, idx=np.arange(lo - 1, hi))  # update! (full rebuild) with a subset
    q1 = np.array(c["query1"])
    assert sorted((O.eachneighbor(g, cl, q1) + 1).tolist()) == c["expected1"]
    q2 = q1 + shift
    assert sorted((O.eachneighbor(g, cl, q2) + 1).tolist()) == c["expected2"]


def _periodic_setup(s):
    y = np.array(s["coords"], dtype=np.float64)
    bmin = np.array(s["box_min"])
    bmax = np.array(s["box_max"])
    if "offset" in s:
        off = np.array(s["offset"])
        y = y - off
        bmin = bmin - off
        bmax = bmax - off
    return y, bmin, bmax


def test_periodic_candidates(O, golden):
    c = golden["periodic_candidates"]
    for s in c["setups"]:
        y, bmin, bmax = _periodic_setup(s)
        d = y.shape[1]
        # FullGridCellList over the periodic box
        g = O.grid_create(d, c["radius"], bmin, bmax, periodic_box=(bmin, bmax))
        cl = O.build(g, y)
        # DictionaryCellList
        gd = O.grid_create(d, c["radius"], bmin, bmax, periodic_box=(bmin, bmax))
        for i, exp in enumerate(c["expected"]):
            assert sorted((O.eachneighbor(g, cl, y[i]) + 1).tolist()) == exp, s["name"]
            assert sorted((O.eachneighbor_dict(gd, y, y[i]) + 1).tolist()) == exp, s["name"]


def test_periodic_neighbors_grid_and_trivial(O, golden):
    c = golden["periodic_neighbors"]
    for s in c["setups"]:
        y, bmin, bmax = _periodic_setup(s)
        d = y.shape[1]
        g = O.grid_create(d, c["radius"], bmin, bmax, periodic_box=(bmin, bmax))
        cl = O.build(g, y)
        off, nb = O.neighbor_lists(g, cl, y, y)
        toff, tnb = O.trivial_lists(g, y, y)
        for i, exp in enumerate(c["expected"]):
            assert sorted((nb[off[i]:off[i + 1]] + 1).tolist()) == exp, s["name"]
            assert sorted((tnb[toff[i]:toff[i + 1]] + 1).tolist()) == exp, s["name"]


def test_split_cells(O, golden):
    c = golden["split_cells"]
    y = np.array(c["coords"])
    bmin, bmax = np.array(c["box_min"]), np.array(c["box_max"])
    g = O.grid_create(2, c["radius"], bmin, bmax, periodic_box=(bmin, bmax))
    for i, exp in enumerate(c["expected"]):
        got = sorted(set((O.eachneighbor_dict(g, y, y[i]) + 1).tolist()))
        assert got == exp


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_periodic_rounding(O, golden, dt):
    c = golden["periodic_rounding"]
    bmin = np.array(c["box_min"], dtype=dt)
    bmax = np.array(c["box_max"], dtype=dt)
    g = O.grid_create(2, dt(c["radius"]), bmin, bmax, periodic_box=(bmin, bmax), dtype=dt)
    size = bmax - bmin
    for x in c["coords"]:
        xv = np.array([jfloat(v, dt) for v in x], dtype=dt)
        xp = O.periodic_coords(g, xv)
        assert np.all(bmin <= xp) and np.all(xp <= bmax)
        for k in range(2):
            assert xp[k] in (xv[k], dt(xv[k] - size[k]), dt(xv[k] + size[k]))
        cell = O.cell_coords(g, xv)
        assert cell == O.cell_coords(g, xp)
        assert all(2 <= cell[k] <= g.n_cells[k] + 1 for k in range(2))


@pytest.mark.parametrize("ndims", [1, 2, 3])
def test_full_grid_bounds(O, golden, ndims):
    c = golden["full_grid_bounds"]
    mn = [c["min_corner"]] * ndims
    mx = [c["max_corner"]] * ndims
    g = O.grid_create(ndims, c["radius"], mn, mx)
    assert list(g.min_pad)[:ndims] == [c["expected_min_pad"]] * ndims
    assert list(g.max_pad)[:ndims] == [c["expected_max_pad"]] * ndims
    rng = np.random.default_rng(0)
    y = rng.random((10, ndims))
    for phase in ("initialize", "update"):
        for val, fails in c[phase]:
            y[6, 0] = jfloat(val)  # y[1, 7] in the reference's 1-based (d, N) indexing
            if fails:
                with pytest.raises(O.OracleError) as e:
                    O.build(g, y)
                assert e.value.status == O.PNO_ERR_OUT_OF_DOMAIN
            else:
                O.build(g, y)


def test_gpu_tutorial_extrema(O, golden):
    c = golden["gpu_tutorial"]
    from __graft_entry__ import package
    W = package().workloads
    y = W.lattice(c["n_per_dim"], dtype=np.float32)
    g = O.grid_create(2, np.float32(c["radius"]), y.min(axis=0), y.max(axis=0),
                      dtype=np.float32)
    cl = O.build(g, y)
    cnt = O.foreach(g, cl, y, y, O.F_COUNT)
    assert (int(cnt.min()), int(cnt.max())) == tuple(c["expected_extrema"])


def test_cell_full(O):
    y = np.array([[0.5, 0.5]] * 5)
    g = O.grid_create(2, 1.0, [0.0, 0.0], [1.0, 1.0], max_ppc=4)
    with pytest.raises(O.OracleError) as e:
        O.build(g, y)
    assert e.value.status == O.PNO_ERR_CELL_FULL


CLOUDS = [(10, 11), (100, 90), (9, 10, 7), (39, 40, 41)]


@pytest.mark.parametrize("shape", CLOUDS)
@pytest.mark.parametrize("seed", [1, 2])
def test_grid_equals_trivial(O, pkg, shape, seed):
    """test/neighborhood_search.jl:186-469: Grid + FullGrid neighbour lists equal brute
    force, initialize! with seed 1 then (seed 2) update! with other coordinates."""
    W = pkg.workloads
    r = 2.5
    coords = W.reference_test_cloud(shape, r, seed=seed)
    coords_init = W.reference_test_cloud(shape, r, seed=1)
    d = len(shape)
    mn = coords.min(axis=0) - r
    mx = coords.max(axis=0) + r
    g = O.grid_create(d, r, mn, mx)
    cl = O.build(g, coords_init)
    if seed != 1:
        # update! after an initialize! with other coordinates (full rebuild semantics)
        cl = O.build(g, coords)
    toff, tnb = O.trivial_lists(g, coords, coords)
    off, nb = O.neighbor_lists(g, cl, coords, coords)
    assert np.array_equal(off, toff)
    for i in range(coords.shape[0]):
        assert np.array_equal(np.sort(nb[off[i]:off[i + 1]]), tnb[toff[i]:toff[i + 1]])
    # mapreduce_neighbor(+, ...) of the neighbour index (1-based)
    isum = O.foreach(g, cl, coords, coords, O.F_INDEX_SUM)
    expect = np.array([int((tnb[toff[i]:toff[i + 1]] + 1).sum()) for i in range(coords.shape[0])])
    assert np.array_equal(isum, expect)


@pytest.mark.parametrize("periodic", [False, True])
def test_mixed_precision_grid_equals_trivial(O, periodic):
    """Float64 coordinates with a Float32 search radius (docs/literate/src/tut_gpu_usage.jl:45-50):
    the grid's lists equal brute force under the same Float32 distance test, plain and periodic."""
    rng = np.random.default_rng(11)
    r = np.float32(0.9)
    lo, hi = np.zeros(3), np.array([6.0, 5.0, 7.3])
    y = rng.uniform(lo, hi, size=(3000, 3))
    if periodic:
        g = O.grid_create_mixed(3, r, lo, hi, periodic_box=(lo, hi))
    else:
        g = O.grid_create_mixed(3, r, lo - r, hi + r)
    assert g.mixed == 1 and g.dtype == 1
    cl = O.build(g, y)
    toff, tnb = O.trivial_lists(g, y, y)
    off, nb = O.neighbor_lists(g, cl, y, y)
    assert np.array_equal(off, toff)
    for i in range(len(y)):
        assert np.array_equal(np.sort(nb[off[i]:off[i + 1]]), tnb[toff[i]:toff[i + 1]])


def test_mixed_precision_distance_in_float32(O):
    """The distance test of a mixed search rounds the Float64 difference to Float32 first:
    a pair 1e-12 beyond the radius in Float64 is a neighbour, one Float32 step beyond is not."""
    r = np.float32(1.7)
    rd = float(r)
    step = float(np.nextafter(r, np.float32(np.inf)))
    y = np.array([[0.0, 0.0], [rd + 1e-12, 0.0], [step, 0.0]])
    g = O.grid_create_mixed(2, r, [-3.0, -3.0], [5.0, 3.0])
    cl = O.build(g, y)
    off, nb = O.neighbor_lists(g, cl, y, y)
    rows = [sorted(nb[off[i]:off[i + 1]].tolist()) for i in range(3)]
    assert rows == [[0, 1], [0, 1, 2], [1, 2]]
    # the same points with the Float64 radius: the first pair is outside
    g64 = O.grid_create(2, rd, [-3.0, -3.0], [5.0, 3.0])
    off, nb = O.neighbor_lists(g64, O.build(g64, y), y, y)
    assert sorted(nb[off[0]:off[1]].tolist()) == [0]


def test_spatial_hashing_collisions(O, golden):
    """test/cell_lists/spatial_hashing.jl:2-67: colliding cells share a list, and the
    traversal's collision checks keep each point to its own cell."""
    c = golden["spatial_hashing_collisions"]
    for case in c["cases"]:
        y = np.array(case["coords"])
        ls = case["list_size"]
        g = O.grid_create_hash(2, c["radius"], ls)
        for atomic in (True, False):
            hl = O.hash_build(g, y, atomic=atomic)
            a, b = case["colliding_cells"]
            assert O.spatial_hash(a, ls) == O.spatial_hash(b, ls)
            assert sorted((hl[tuple(a)] + 1).tolist()) == case["cell_points"]
            assert sorted((hl[tuple(b)] + 1).tolist()) == case["cell_points"]
            off, nb = O.hash_neighbor_lists(g, hl, y, y)
            rows = [(nb[off[i]:off[i + 1]] + 1).tolist() for i in range(len(y))]
            assert rows == case["neighbors"]


def test_host_spatial_hash_equals_oracle(O, pkg):
    """The host API's spatial_hash (the list a user sees through export_cells/eachneighbor)
    equals the oracle's restatement of spatial_hashing.jl:142-156, for negative and large
    cells (the Int64 products and xor wrap) and list sizes from 1 to above 2^31."""
    rng = np.random.default_rng(11)
    for d in (1, 2, 3):
        for _ in range(300):
            scale = int(rng.choice([4, 1000, 2**20, 2**31 - 2]))
            cell = [int(v) for v in rng.integers(-scale, scale, d)]
            ls = int(rng.choice([1, 7, 1000, 2**20 + 3, 2**31 + 5]))
            assert pkg.spatial_hash(cell, ls) == O.spatial_hash(cell, ls), (cell, ls)


def test_coordinates_flattened(O, golden):
    c = golden["coordinates_flattened"]
    for v in c["values"]:
        assert O.coordinates_flattened(v["cell"]) == int(v["flat"])
    for cell in c["inexact"]:
        with pytest.raises(O.OracleError):
            O.coordinates_flattened(cell)


@pytest.mark.parametrize("shape", CLOUDS)
def test_spatial_hashing_equals_trivial(O, pkg, shape):
    """test/neighborhood_search.jl:186-469 with SpatialHashingCellList(list_size = 2n): the
    lists equal brute force, for both push semantics and, on the smaller clouds, for a
    list_size of 7 (every list shared by many cells)."""
    W = pkg.workloads
    r = 2.5
    coords = W.reference_test_cloud(shape, r, seed=2)
    d = len(shape)
    mn = coords.min(axis=0) - r
    mx = coords.max(axis=0) + r
    toff, tnb = O.trivial_lists(O.grid_create(d, r, mn, mx), coords, coords)
    for ls in ((2 * len(coords), 7) if len(coords) < 10000 else (2 * len(coords),)):
        g = O.grid_create_hash(d, r, ls, max_ppc=len(coords))
        for atomic in (True, False):
            off, nb = O.hash_neighbor_lists(g, O.hash_build(g, coords, atomic=atomic),
                                            coords, coords)
            assert np.array_equal(off, toff)
            for i in range(coords.shape[0]):
                assert np.array_equal(np.sort(nb[off[i]:off[i + 1]]), tnb[toff[i]:toff[i + 1]])


def test_spatial_hashing_periodic_neighbors(O, golden):
    """test/neighborhood_search.jl:72-160 with SpatialHashingCellList(list_size = 2n)."""
    c = golden["periodic_neighbors"]
    for s in c["setups"]:
        y = np.array(s["coords"])
        g = O.grid_create_hash(y.shape[1], c["radius"], 2 * len(y),
                               periodic_box=(np.array(s["box_min"]), np.array(s["box_max"])))
        off, nb = O.hash_neighbor_lists(g, O.hash_build(g, y), y, y)
        for i, exp in enumerate(c["expected"]):
            assert sorted((nb[off[i]:off[i + 1]] + 1).tolist()) == exp, s["name"]
