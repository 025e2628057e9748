"""GridNeighborhoodSearch over a SpatialHashingCellList (pn_create_spatial_hashing) against
the reference's known answers (test/cell_lists/spatial_hashing.jl, the periodic cases of
test/neighborhood_search.jl) and the oracle's restatement of the reference's hash lists and
collision checks.

Bars: neighbour lists and counts bit-exact (sets; rows sorted); WCSPH sums within 1e-5
(FP32) / 1e-12 (FP64) of the FP64 oracle relative to sum |terms| (the hashed traversal
visits the cells one by one, so sums run in another order than the full grid's)."""
import numpy as np
import pytest
import torch

from test_gpu_parity import TOL_F32, TOL_F64, _periodic_setup, _rel_err, csr_rows, dcoords

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def hashed(P, d, r, n, list_size=None, dtype=np.float64, box=None, max_ppc=0):
    T = dtype
    cl = P.SpatialHashingCellList(d, list_size=list_size or 2 * max(n, 1),
                                  max_points_per_cell=max_ppc)
    pb = None if box is None else P.PeriodicBox(min_corner=np.asarray(box[0], T),
                                                max_corner=np.asarray(box[1], T))
    return P.GridNeighborhoodSearch(d, search_radius=T(r), n_points=n, cell_list=cl,
                                    periodic_box=pb)


def test_golden_collisions(P, golden):
    """test/cell_lists/spatial_hashing.jl:2-67: colliding cells, empty and non-empty."""
    c = golden["spatial_hashing_collisions"]
    for case in c["cases"]:
        y = np.array(case["coords"])
        nhs = hashed(P, 2, c["radius"], len(y), list_size=case["list_size"])
        a, b = case["colliding_cells"]
        assert P.spatial_hash(a, case["list_size"]) == P.spatial_hash(b, case["list_size"])
        yd = dcoords(y)
        P.initialize(nhs, yd, yd)
        rows = [(r + 1).tolist() for r in csr_rows(*P.neighbor_lists(yd, yd, nhs))]
        assert rows == case["neighbors"]
        # eachneighbor returns the whole hash list of each cell (points_in_cell)
        assert sorted(set((P.eachneighbor(y[0], nhs) + 1).tolist())) == case["cell_points"]


def test_golden_periodic_neighbors(P, golden):
    """test/neighborhood_search.jl:59-184 with SpatialHashingCellList(list_size = 2n), and a
    copied template (copy_neighborhood_search)."""
    c = golden["periodic_neighbors"]
    for s in c["setups"]:
        y, bmin, bmax = _periodic_setup(s)
        d = y.shape[1]
        nhs = hashed(P, d, c["radius"], len(y), box=(bmin, bmax))
        tmpl = hashed(P, d, 0.0, len(y), box=(bmin, bmax))
        for search in (nhs, P.copy_neighborhood_search(tmpl, c["radius"], len(y))):
            x = dcoords(y)
            P.initialize(search, x, x)
            rows = csr_rows(*P.neighbor_lists(x, x, search))
            for i, exp in enumerate(c["expected"]):
                assert (rows[i] + 1).tolist() == exp, s["name"]


CLOUDS = [(10, 11), (100, 90), (9, 10, 7), (39, 40, 41)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", CLOUDS)
def test_hashing_equals_oracle_and_trivial(P, O, shape, dt):
    """test/neighborhood_search.jl:186-469: initialize! with seed 1, update! with seed 2;
    the lists equal the oracle's hash lists (with their collision checks) and brute force,
    for list_size = 2n and for 7 lists (every list shared by many cells)."""
    W = P.workloads
    r = 2.5
    c1 = W.reference_test_cloud(shape, r, seed=1).astype(dt)
    c2 = W.reference_test_cloud(shape, r, seed=2).astype(dt)
    d = len(shape)
    n = len(c1)
    toff, tnb = O.trivial_lists(O.grid_create(d, dt(r), c2.min(0) - r, c2.max(0) + r, dtype=dt),
                                c2, c2)
    for ls in ((2 * n, 7) if n < 10000 else (2 * n,)):
        nhs = hashed(P, d, r, n, list_size=ls, dtype=dt)
        P.initialize(nhs, dcoords(c1), dcoords(c1))
        x = dcoords(c2)
        P.update(nhs, x, x)
        off, nb = P.neighbor_lists(x, x, nhs)
        assert np.array_equal(off.cpu().numpy(), toff)
        assert np.array_equal(nb.cpu().numpy(), tnb)
        if n < 10000:
            g = O.grid_create_hash(d, dt(r), ls, max_ppc=n if ls == 7 else 64, dtype=dt)
            hoff, hnb = O.hash_neighbor_lists(g, O.hash_build(g, c2), c2, c2)
            assert np.array_equal(off.cpu().numpy(), hoff)
            assert np.array_equal(nb.cpu().numpy(),
                                  np.concatenate([np.sort(hnb[hoff[i]:hoff[i + 1]])
                                                  for i in range(n)]))
        # the grid's cell export lists each hash list's points
        counts, pts = P.export_cells(nhs)
        assert len(counts) == ls and counts.sum() == n
        assert np.array_equal(np.sort(pts), np.arange(n))


def test_hashing_unbounded_and_queries(P, O):
    """Points far from the origin and on both sides of it (no domain bounds), queries x
    not y, a subset of query points, and eachindex_y."""
    rng = np.random.default_rng(3)
    y = np.concatenate([rng.uniform(-40, 40, (20000, 3)),
                        rng.uniform(1e5, 1e5 + 30, (5000, 3)),
                        rng.uniform(-2e6, -2e6 + 30, (5000, 3))])
    xq = np.concatenate([rng.uniform(-40, 40, (2000, 3)), rng.uniform(1e5, 1e5 + 30, (500, 3))])
    r = 1.5
    nhs = hashed(P, 3, r, len(y))
    yd, xd = dcoords(y), dcoords(xq)
    P.initialize(nhs, xd, yd)
    g = O.grid_create_hash(3, r, 2 * len(y), max_ppc=64)
    hl = O.hash_build(g, y)
    off, nb = P.neighbor_lists(xd, yd, nhs)
    hoff, hnb = O.hash_neighbor_lists(g, hl, xq, y)
    assert np.array_equal(off.cpu().numpy(), hoff)
    assert np.array_equal(nb.cpu().numpy(),
                          np.concatenate([np.sort(hnb[hoff[i]:hoff[i + 1]])
                                          for i in range(len(xq))]))
    cnt = torch.zeros(len(xq), dtype=torch.int32, device="cuda")
    pts = np.arange(0, len(xq), 3)
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, yd, nhs, points=pts)
    assert np.array_equal(cnt.cpu().numpy()[pts], np.diff(hoff)[pts])
    # eachindex_y: only the listed points are binned
    sub = np.arange(0, len(y), 2)
    P.initialize(nhs, yd, yd, eachindex_y=sub)
    off, nb = P.neighbor_lists(xd, yd, nhs)
    hoff, hnb = O.hash_neighbor_lists(g, O.hash_build(g, y[sub]), xq, y[sub])
    assert np.array_equal(off.cpu().numpy(), hoff)
    assert np.array_equal(nb.cpu().numpy(),
                          np.concatenate([np.sort(sub[hnb[hoff[i]:hoff[i + 1]]])
                                          for i in range(len(xq))]))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_hashing_wcsph_vs_oracle(P, O, dt):
    W = P.workloads
    x, v, _ = W.wcsph_cloud(24, seed=5, dtype=dt)
    n = len(x)
    r = 3.0
    nhs = hashed(P, 3, r, n, dtype=dt)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    T = torch.float32 if dt == np.float32 else torch.float64
    rho = torch.zeros(n, dtype=T, device="cuda")
    prs = torch.zeros(n, dtype=T, device="cuda")
    acc = torch.zeros(3 * n, dtype=T, device="cuda")
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd, accel=acc,
                                         **W.WCSPH), xd, xd, nhs)
    g = O.grid_create(3, dt(r), np.full(3, -1.0, dt), np.full(3, 25.0, dt), dtype=dt)
    cl = O.build(g, x)
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl, x, x, O.F_WCSPH_DENSITY, prm, want_abs=True)
    tol = TOL_F32 if dt == np.float32 else TOL_F64
    assert _rel_err(rho.cpu().numpy().astype(np.float64), orho, oab) < tol
    c = W.WCSPH
    prm2, keep2 = O.make_params(rho=rho.cpu().numpy().astype(np.float64),
                                pressure=prs.cpu().numpy().astype(np.float64),
                                vel=v.astype(np.float64),
                                r_min=float(np.sqrt(np.finfo(dt).eps)) * c["h"], **c)
    oacc, oabs = O.foreach(g, cl, x, x, O.F_WCSPH_FORCE, prm2, want_abs=True)
    assert _rel_err(acc.cpu().numpy().astype(np.float64).reshape(n, 3), oacc, oabs) < tol


def test_hashing_periodic_large(P, O):
    """A periodic box whose faces are not multiples of the cell size (so the hashed cells
    do not line up with them), against brute force."""
    rng = np.random.default_rng(8)
    lo, hi = np.array([0.37, -1.3, 2.1]), np.array([17.0, 14.2, 19.9])
    y = rng.uniform(lo, hi, size=(30000, 3))
    r = 1.1
    nhs = hashed(P, 3, r, len(y), box=(lo, hi))
    yd = dcoords(y)
    P.initialize(nhs, yd, yd)
    off, nb = P.neighbor_lists(yd, yd, nhs)
    g = O.grid_create(3, r, lo, hi, periodic_box=(lo, hi), max_ppc=1000)
    toff, tnb = O.trivial_lists(g, y, y)
    assert np.array_equal(off.cpu().numpy(), toff)
    assert np.array_equal(nb.cpu().numpy(), tnb)


def test_hashing_errors(P):
    y = np.zeros((200, 2))
    nhs = hashed(P, 2, 1.0, 200, max_ppc=100)
    yd = dcoords(y)
    with pytest.raises(P.PointNeighborsError, match="cell list is full"):
        P.initialize(nhs, yd, yd)
    far = dcoords(np.array([[0.0, 0.0], [3e9, 0.0]]))
    nhs2 = hashed(P, 2, 1.0, 2)
    with pytest.raises(P.PointNeighborsError, match="outside the domain"):
        P.initialize(nhs2, far, far)
    with pytest.raises(P.ArgumentError, match="not a valid update strategy"):
        P.GridNeighborhoodSearch(2, search_radius=1.0,
                                 cell_list=P.SpatialHashingCellList(2, list_size=10),
                                 update_strategy=P.ParallelIncrementalUpdate())


def test_hashing_dense_and_list_layouts_agree(P, O):
    """The same points in the dense grid layout (list_size above the occupied box's cell
    count) and in the hash-list layout (below it): identical lists, WCSPH sums within the
    FP32 bar, and the pair cache (dense layout only) bit-identical to no cache."""
    W = P.workloads
    x, v, _ = W.wcsph_cloud(20, seed=12, dtype=np.float32)
    n = len(x)
    r = np.float32(3.0)
    xd = dcoords(x)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    outs = {}
    for name, ls, cache in (("dense", 2 * n, False), ("lists", 97, False),
                            ("dense_cache", 2 * n, True)):
        cl = P.SpatialHashingCellList(3, list_size=ls, max_points_per_cell=0)
        nhs = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl,
                                       pair_cache=cache)
        P.initialize(nhs, xd, xd)
        assert (nhs.grid_info()["grid_size"][0] > 1) == (name != "lists")
        off, nb = P.neighbor_lists(xd, xd, nhs)
        rho = torch.zeros(n, device="cuda")
        prs = torch.zeros(n, device="cuda")
        acc = torch.zeros(3 * n, device="cuda")
        for _ in range(2):  # with the cache: the second step walks it
            P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd,
                                                 accel=acc, **W.WCSPH), xd, xd, nhs)
        outs[name] = (off.cpu().numpy(), nb.cpu().numpy(), rho.cpu().numpy(),
                      acc.cpu().numpy())
    for k in range(2):
        assert np.array_equal(outs["dense"][k], outs["lists"][k])
        assert np.array_equal(outs["dense"][k], outs["dense_cache"][k])
    # density: the same sweep with or without recording the cache; the force over the
    # cache and the sums of the other layout run in another order
    assert np.array_equal(outs["dense"][2], outs["dense_cache"][2])
    for k in (2, 3):
        ref = outs["dense"][k].astype(np.float64)
        scale = np.abs(ref).max()
        assert np.max(np.abs(outs["lists"][k] - ref)) <= 1e-5 * scale
        assert np.max(np.abs(outs["dense_cache"][k] - ref)) <= 1e-5 * scale


@pytest.mark.parametrize("list_size", [None, 97])
def test_precomputed_over_hashing(P, O, list_size):
    """PrecomputedNeighborhoodSearch whose lists a SpatialHashingCellList grid search
    computes (dense layout and hash lists): its lists equal brute force after update!."""
    W = P.workloads
    r = 2.5
    c1 = W.reference_test_cloud((21, 20, 19), r, seed=1)
    c2 = W.reference_test_cloud((21, 20, 19), r, seed=2)
    n = len(c1)
    grid = hashed(P, 3, r, n, list_size=list_size)
    pre = P.PrecomputedNeighborhoodSearch(3, n_points=n, update_neighborhood_search=grid)
    P.initialize(pre, dcoords(c1), dcoords(c1))
    x = dcoords(c2)
    P.update(pre, x, x)
    off, nb = P.neighbor_lists(x, x, pre)
    toff, tnb = O.trivial_lists(O.grid_create(3, r, c2.min(0) - r, c2.max(0) + r), c2, c2)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), x, x, pre)
    assert np.array_equal(cnt.cpu().numpy(), np.diff(toff))


@pytest.mark.parametrize("periodic", [False, True])
def test_hashing_dense_layout_queries(P, O, periodic):
    """Queries x not y over the dense layout: inside the occupied box, just outside it (their
    3^d cells still reach it) and far away (no neighbours, not a BoundsError), and a subset
    of the points of y."""
    rng = np.random.default_rng(29)
    lo, hi = np.array([1.3, -2.0, 0.5]), np.array([13.0, 9.0, 10.2])
    y = rng.uniform(lo, hi, size=(12000, 3))
    r = 1.2
    if periodic:
        xq = rng.uniform(lo, hi, size=(3000, 3))
    else:
        xq = np.concatenate([rng.uniform(lo - 1.5 * r, hi + 1.5 * r, size=(3000, 3)),
                             rng.uniform(100.0, 120.0, size=(50, 3))])
    nhs = hashed(P, 3, r, len(y), box=(lo, hi) if periodic else None)
    yd, xd = dcoords(y), dcoords(xq)
    P.initialize(nhs, xd, yd)
    assert nhs.grid_info()["grid_size"][0] > 1  # the dense layout
    off, nb = P.neighbor_lists(xd, yd, nhs)
    g = (O.grid_create(3, r, lo, hi, periodic_box=(lo, hi), max_ppc=1000) if periodic
         else O.grid_create(3, r, lo - 3 * r, hi + 3 * r, max_ppc=1000))
    toff, tnb = O.trivial_lists(g, xq, y)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)
    pts = np.arange(0, len(xq), 5)
    cnt = torch.full((len(xq),), -1, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, yd, nhs, points=pts)
    assert np.array_equal(cnt.cpu().numpy()[pts], np.diff(toff)[pts])
