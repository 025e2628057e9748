"""The cell-list build's worst case: very full cells.

The reference keeps each cell in a fixed-capacity column and raises "cell list is full"
(vector_of_vectors.jl:114-121) when a cell exceeds `max_points_per_cell`.  Here the cell
list has no capacity when `max_points_per_cell = 0`, so a clustered cloud can put tens of
thousands of points into one cell; the in-cell sort must then stay fast (cells above 256
points are ranked through shared memory), and with a limit the build must fail without
sorting.  Cells are compared with the oracle's, neighbour counts with its grid search.
"""
import numpy as np
import pytest

from test_gpu_parity import dcoords

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _one_cell_cloud(d, n, dtype, seed=5):
    """n points uniform in [4.1, 4.9]^d: all in one cell of a radius-1 grid over [3, 6]^d."""
    rng = np.random.default_rng(seed)
    return rng.uniform(4.1, 4.9, (n, d)).astype(dtype)


def _grid(P, d, n, dtype, max_ppc, strategy=None):
    T = dtype
    cl = P.FullGridCellList(min_corner=np.full(d, 3.0, T), max_corner=np.full(d, 6.0, T),
                            search_radius=T(1.0), max_points_per_cell=max_ppc)
    return P.GridNeighborhoodSearch(d, search_radius=T(1.0), n_points=n, cell_list=cl,
                                    update_strategy=strategy)


def _timed(fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


@pytest.mark.parametrize("d,dtype", [(3, np.float32), (3, np.float64), (2, np.float32)])
def test_crowded_cell_builds_fast_and_exact(P, O, d, dtype):
    n = 20000
    y = _one_cell_cloud(d, n, dtype)
    nhs = _grid(P, d, n, dtype, 0)
    yd = dcoords(y)
    P.initialize(nhs, yd, yd)  # first call: module loading, allocations
    ms = _timed(lambda: P.initialize(nhs, yd, yd))
    # one thread per slot reading its whole cell from global memory would make 4e8
    # dependent loads here; through shared memory the rank is 4e8 cheap comparisons
    assert ms < 50.0, f"build of one 20,000-point cell took {ms:.1f} ms"
    g = O.grid_create(d, dtype(1.0), np.full(d, 3.0, dtype), np.full(d, 6.0, dtype),
                      max_ppc=n, dtype=dtype)
    cl = O.build(g, y)
    counts, pts = P.export_cells(nhs)
    ocounts, opts = cl.as_csr()
    assert counts.max() == n
    assert np.array_equal(counts, ocounts)
    ends = np.cumsum(ocounts)
    assert np.array_equal(pts, np.concatenate([np.sort(opts[e - c:e])
                                               for c, e in zip(ocounts, ends)]))
    # the traversal clips stencil rows by the in-cell x order: counts test that order
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), yd, yd, nhs)
    assert np.array_equal(cnt.cpu().numpy(), O.foreach(g, cl, y, y, O.F_COUNT))


def test_crowded_cell_with_limit_fails_without_sorting(P):
    n = 20000
    y = _one_cell_cloud(3, n, np.float32)
    nhs = _grid(P, 3, n, np.float32, 100)
    yd = dcoords(y)
    with pytest.raises(P.PointNeighborsError, match="cell list is full"):
        P.initialize(nhs, yd, yd)

    def failing():
        with pytest.raises(P.PointNeighborsError, match="cell list is full"):
            P.initialize(nhs, yd, yd)
    assert _timed(failing) < 50.0
    # a cloud within the limit builds on the same search afterwards
    ok = dcoords(np.random.default_rng(1).uniform(3.0, 6.0, (500, 3)).astype(np.float32))
    P.initialize(nhs, ok, ok)


def test_crowded_hash_lists(P, O):
    """SpatialHashingCellList in the hash-list layout with lists of about 2,900 points
    (the in-list order by cell, then x, ranked through shared memory)."""
    rng = np.random.default_rng(9)
    n = 20000
    y = rng.uniform(0.0, 40.0, (n, 2))
    cl = P.SpatialHashingCellList(2, list_size=7, max_points_per_cell=0)
    nhs = P.GridNeighborhoodSearch(2, search_radius=1.0, n_points=n, cell_list=cl)
    yd = dcoords(y)
    P.initialize(nhs, yd, yd)
    assert nhs.grid_info()["grid_size"][0] == 1  # the hash-list layout, not the dense grid
    counts, pts = P.export_cells(nhs)
    assert counts.min() > 256
    toff, tnb = O.trivial_lists(O.grid_create(2, 1.0, np.full(2, -1.0), np.full(2, 41.0)), y, y)
    off, nb = P.neighbor_lists(yd, yd, nhs)
    assert np.array_equal(off.cpu().numpy(), toff)
    assert np.array_equal(nb.cpu().numpy(), tnb)


def test_incremental_update_into_one_cell(P, O):
    """Movers that all land in one cell: the overflow list of that cell would exceed 256
    points, so update! rebuilds instead; the result equals a rebuild and the oracle."""
    rng = np.random.default_rng(2)
    n = 60000
    x0 = rng.uniform(3.0, 33.0, (n, 3)).astype(np.float32)
    x1 = x0.copy()
    movers = rng.choice(n, 400, replace=False)  # 0.7 % of the points
    x1[movers] = rng.uniform(10.1, 10.9, (400, 3)).astype(np.float32)
    T = np.float32

    def grid(strategy):
        c = P.FullGridCellList(min_corner=np.full(3, 3.0, T), max_corner=np.full(3, 33.0, T),
                               search_radius=T(1.0), max_points_per_cell=0)
        return P.GridNeighborhoodSearch(3, search_radius=T(1.0), n_points=n, cell_list=c,
                                        update_strategy=strategy)
    inc = grid(P.ParallelIncrementalUpdate(1.0))  # never rebuilds for the mover count alone
    ref = grid(P.ParallelUpdate())
    a, b = dcoords(x0), dcoords(x1)
    P.initialize(inc, a, a)
    P.initialize(ref, a, a)
    P.update(inc, b, b)
    P.update(ref, b, b)
    ci, pi = P.export_cells(inc)
    cr, pr = P.export_cells(ref)
    assert np.array_equal(ci, cr) and np.array_equal(pi, pr)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), b, b, inc)
    g = O.grid_create(3, T(1.0), np.full(3, 3.0, T), np.full(3, 33.0, T), max_ppc=1000,
                      dtype=T)
    assert np.array_equal(cnt.cpu().numpy(), O.foreach(g, O.build(g, x1), x1, x1, O.F_COUNT))
