"""Parity of the CUDA path with the oracle and with the reference's known answers.

Every call goes through the Python host API onto the C ABI of libpn_gb300.so.  Neighbour
sets, cell assignments and counts must be bit-exact; floating-point sums are compared
with an FP64 oracle run within the tolerances stated in each test, relative to the sum of
the absolute values of the summed terms (the condition of the sum).
"""
import numpy as np
import pytest

from conftest import jfloat

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5   # FP32 sums vs the FP64 oracle, relative to sum |terms|
TOL_F64 = 1e-12  # FP64 sums vs the FP64 oracle


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    assert torch.cuda.is_available()
    return pkg


def dcoords(pts, dtype=None):
    """(N, d) points -> (d, N) CUDA tensor with the reference's column-major layout."""
    a = np.ascontiguousarray(pts if dtype is None else np.asarray(pts, dtype=dtype))
    return torch.as_tensor(a, device="cuda").T


def make_nhs(P, d, r, mn, mx, n, dtype=np.float64, box=None, strategy=None, max_ppc=100):
    T = dtype
    cl = P.FullGridCellList(min_corner=np.asarray(mn, T), max_corner=np.asarray(mx, T),
                            search_radius=T(r), max_points_per_cell=max_ppc)
    pb = None if box is None else P.PeriodicBox(min_corner=np.asarray(box[0], T),
                                                max_corner=np.asarray(box[1], T))
    return P.GridNeighborhoodSearch(d, search_radius=T(r), n_points=n, cell_list=cl,
                                    periodic_box=pb, update_strategy=strategy)


def csr_rows(off, nb):
    off = off.cpu().numpy()
    nb = nb.cpu().numpy()
    return [nb[off[i]:off[i + 1]] for i in range(len(off) - 1)]


# ----------------------------------------------------------------- known answers

@pytest.mark.parametrize("strategy", ["serial_or_parallel", "incremental_full"])
def test_golden_eachindex_y(P, golden, strategy):
    c = golden["eachindex_y_3d"]
    c1 = np.array(c["coords"])
    c2 = c1 + np.array(c["shift"])
    mn = np.minimum(c1.min(0), c2.min(0))
    mx = np.maximum(c1.max(0), c2.max(0))
    nhs = make_nhs(P, 3, c["radius"], mn, mx, len(c1))
    x1, x2 = dcoords(c1), dcoords(c2)
    P.initialize(nhs, x1, x1)
    lo, hi = c["eachindex_y"]
    P.update(nhs, x2, x2, eachindex_y=range(lo - 1, hi))
    q1 = np.array(c["query1"])
    assert sorted((P.eachneighbor(q1, nhs) + 1).tolist()) == c["expected1"]
    assert sorted((P.eachneighbor(q1 + np.array(c["shift"]), nhs) + 1).tolist()) == c["expected2"]


def _periodic_setup(s):
    y = np.array(s["coords"], dtype=np.float64)
    bmin, bmax = np.array(s["box_min"]), np.array(s["box_max"])
    if "offset" in s:
        off = np.array(s["offset"])
        y, bmin, bmax = y - off, bmin - off, bmax - off
    return y, bmin, bmax


def test_golden_periodic_candidates(P, golden):
    c = golden["periodic_candidates"]
    for s in c["setups"]:
        y, bmin, bmax = _periodic_setup(s)
        d = y.shape[1]
        nhs = make_nhs(P, d, c["radius"], bmin, bmax, len(y), box=(bmin, bmax))
        x = dcoords(y)
        P.initialize(nhs, x, x)
        for i, exp in enumerate(c["expected"]):
            assert sorted((P.eachneighbor(y[i], nhs) + 1).tolist()) == exp, s["name"]


def test_golden_periodic_neighbors(P, golden):
    c = golden["periodic_neighbors"]
    for s in c["setups"]:
        y, bmin, bmax = _periodic_setup(s)
        d = y.shape[1]
        nhs = make_nhs(P, d, c["radius"], bmin, bmax, len(y), box=(bmin, bmax))
        x = dcoords(y)
        P.initialize(nhs, x, x)
        rows = csr_rows(*P.neighbor_lists(x, x, nhs))
        for i, exp in enumerate(c["expected"]):
            assert (rows[i] + 1).tolist() == exp, s["name"]
        # the same search copied from a template (copy_neighborhood_search)
        tmpl = make_nhs(P, d, 0.0, bmin, bmax, 0, box=(bmin, bmax))
        nhs2 = P.copy_neighborhood_search(tmpl, c["radius"], len(y))
        P.initialize(nhs2, x, x)
        rows2 = csr_rows(*P.neighbor_lists(x, x, nhs2))
        assert [r.tolist() for r in rows2] == [r.tolist() for r in rows]


def test_golden_cell_coords_limits(P, golden):
    c = golden["cell_coords_limits"]
    g = c["full_grid"]
    nhs = make_nhs(P, 2, c["radius"], g["min_corner"], g["max_corner"], 1)
    for x, ef in zip(c["coords"], c["full_expected"]):
        assert P.cell_coords([jfloat(v) for v in x], nhs) == tuple(ef)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_golden_periodic_rounding(P, O, golden, dt):
    c = golden["periodic_rounding"]
    bmin, bmax = np.array(c["box_min"], dt), np.array(c["box_max"], dt)
    nhs = make_nhs(P, 2, c["radius"], bmin, bmax, 12, dtype=dt, box=(bmin, bmax))
    og = O.grid_create(2, dt(c["radius"]), bmin, bmax, periodic_box=(bmin, bmax), dtype=dt)
    nc = nhs.n_cells
    for x in c["coords"]:
        xv = np.array([jfloat(v, dt) for v in x], dtype=dt)
        cell = P.cell_coords(xv, nhs)
        assert cell == P.cell_coords(O.periodic_coords(og, xv), nhs)
        assert all(2 <= cell[k] <= nc[k] + 1 for k in range(2))
        assert cell == O.cell_coords(og, xv)


@pytest.mark.parametrize("ndims", [1, 2, 3])
def test_golden_full_grid_bounds(P, golden, ndims):
    c = golden["full_grid_bounds"]
    nhs = make_nhs(P, ndims, c["radius"], [c["min_corner"]] * ndims, [c["max_corner"]] * ndims, 10)
    assert list(nhs.cell_list.min_corner) == [c["expected_min_pad"]] * ndims
    assert nhs.grid_info()["min_corner"] == (c["expected_min_pad"],) * ndims
    y = np.random.default_rng(0).random((10, ndims))
    for phase in ("initialize", "update"):
        for val, fails in c[phase]:
            y[6, 0] = jfloat(val)
            x = dcoords(y)
            fn = P.initialize if phase == "initialize" else P.update
            if fails:
                with pytest.raises(P.PointNeighborsError, match=c["message"]):
                    fn(nhs, x, x)
            else:
                fn(nhs, x, x)


def test_golden_gpu_tutorial(P, golden):
    c = golden["gpu_tutorial"]
    pts = P.workloads.lattice(c["n_per_dim"], dtype=np.float32)
    nhs = make_nhs(P, 2, c["radius"], pts.min(0), pts.max(0), len(pts), dtype=np.float32)
    x = dcoords(pts)
    P.initialize(nhs, x, x)
    n = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(n), x, x, nhs)
    assert (int(n.min()), int(n.max())) == tuple(c["expected_extrema"])


def test_golden_cell_full(P, golden):
    y = np.array([[0.5, 0.5]] * 5)
    nhs = make_nhs(P, 2, 1.0, [0.0, 0.0], [1.0, 1.0], 5, max_ppc=4)
    x = dcoords(y)
    with pytest.raises(P.PointNeighborsError, match="cell list is full"):
        P.initialize(nhs, x, x)
    nhs_unlimited = make_nhs(P, 2, 1.0, [0.0, 0.0], [1.0, 1.0], 5, max_ppc=0)
    P.initialize(nhs_unlimited, x, x)


# ----------------------------------------------------------------- differential test

CLOUDS = [(10, 11), (100, 90), (9, 10, 7), (39, 40, 41)]


@pytest.mark.parametrize("shape", CLOUDS)
@pytest.mark.parametrize("seed", [1, 2])
@pytest.mark.parametrize("incremental", [None, 1.0, 0.0])
def test_grid_equals_trivial(P, O, shape, seed, incremental):
    """test/neighborhood_search.jl:186-469: neighbour lists equal brute force after
    initialize! (seed 1) or initialize! + update! (seed 2), for ParallelUpdate and for
    ParallelIncrementalUpdate both keeping overflow lists (rebuild_fraction 1) and
    rebuilding on the device (rebuild_fraction 0)."""
    W = P.workloads
    r = 2.5
    coords = W.reference_test_cloud(shape, r, seed=seed)
    coords_init = W.reference_test_cloud(shape, r, seed=1)
    d = len(shape)
    mn, mx = coords.min(0) - r, coords.max(0) + r
    strat = P.ParallelUpdate() if incremental is None else P.ParallelIncrementalUpdate(incremental)
    nhs = make_nhs(P, d, r, mn, mx, len(coords), strategy=strat)
    xi, x = dcoords(coords_init), dcoords(coords)
    P.initialize(nhs, xi, xi)
    if seed != 1:
        P.update(nhs, x, x)
    else:
        x = xi
    g = O.grid_create(d, r, mn, mx)
    toff, tnb = O.trivial_lists(g, coords, coords)
    off, nb = P.neighbor_lists(x, x, nhs)
    assert np.array_equal(off.cpu().numpy(), toff)
    assert np.array_equal(nb.cpu().numpy(), tnb)
    sums = torch.zeros(len(coords), dtype=torch.int64, device="cuda")
    P.foreach_point_neighbor(P.NeighborIndexSum(sums), x, x, nhs)
    expect = np.add.reduceat(tnb.astype(np.int64) + 1, toff[:-1]) if len(tnb) else 0
    expect = np.where(np.diff(toff) > 0, expect, 0)
    assert np.array_equal(sums.cpu().numpy(), expect)
    # the cell list itself equals the reference's, cell by cell
    counts, pts = P.export_cells(nhs)
    cl = O.build(g, coords)
    ocounts, opts = cl.as_csr()
    assert np.array_equal(counts, ocounts)
    assert np.array_equal(pts, opts)


def test_points_subset_and_x_not_y(P, O):
    """`points` keyword and a query set x different from y (neighborhood_search.jl:183-201)."""
    W = P.workloads
    r = 2.5
    y = W.reference_test_cloud((20, 21, 9), r, seed=3)
    xq = y[::3] + 0.37
    mn, mx = y.min(0) - r, y.max(0) + r
    nhs = make_nhs(P, 3, r, mn, mx, len(y))
    yd, xd = dcoords(y), dcoords(xq)
    P.initialize(nhs, yd, yd)
    g = O.grid_create(3, r, mn, mx)
    toff, tnb = O.trivial_lists(g, xq, y)
    off, nb = P.neighbor_lists(xd, yd, nhs)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)
    pts = np.arange(5, len(y), 7)
    cnt = torch.full((len(y),), -7, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), yd, yd, nhs, points=pts)
    full = O.foreach(g, O.build(g, y), y, y, O.F_COUNT)
    c = cnt.cpu().numpy()
    assert np.array_equal(c[pts], full[pts])
    mask = np.ones(len(y), bool)
    mask[pts] = False
    assert np.all(c[mask] == -7)


def test_empty_neighborhood(P):
    """Initialized with no neighbour points: every reduction returns its init
    (test/neighborhood_search.jl:445-466)."""
    coords = P.workloads.reference_test_cloud((9, 10, 7), 2.5, seed=1)
    mn, mx = coords.min(0) - 2.5, coords.max(0) + 2.5
    nhs = make_nhs(P, 3, 2.5, mn, mx, 0)
    x = dcoords(coords)
    empty = torch.empty((3, 0), dtype=torch.float64, device="cuda")
    P.initialize(nhs, x, empty)
    sums = torch.full((len(coords),), 123, dtype=torch.int64, device="cuda")
    P.foreach_point_neighbor(P.NeighborIndexSum(sums), x, empty, nhs)
    assert int(sums.abs().max()) == 0


def test_query_outside_grid_is_bounds_error(P):
    y = np.random.default_rng(1).random((50, 2)) * 10
    nhs = make_nhs(P, 2, 1.0, [0.0, 0.0], [10.0, 10.0], 50)
    yd = dcoords(y)
    P.initialize(nhs, yd, yd)
    xq = dcoords(np.array([[5.0, 5.0], [50.0, 5.0]]))
    cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(P.BoundsError):
        P.foreach_point_neighbor(P.CountNeighbors(cnt), xq, yd, nhs)


# ----------------------------------------------------------------- workload configs

def test_plain_count_config_125k_fp64(P, O):
    """50^3 lattice, U[-0.25, 0.25] noise, Float64, r = 3, box [-1, 51]^3: neighbour counts
    (self excluded) and the sorted pair list, bit-exact against the oracle's Grid search and
    against brute force on a sample of query points."""
    pts = P.workloads.perturbed_lattice((50, 50, 50), 0.25, seed=1, dtype=np.float64)
    r = 3.0
    nhs = make_nhs(P, 3, r, [-1.0] * 3, [51.0] * 3, len(pts))
    x = dcoords(pts)
    P.initialize(nhs, x, x)
    cnt = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), x, x, nhs)
    off, nb = P.neighbor_lists(x, x, nhs)
    g = O.grid_create(3, r, [-1.0] * 3, [51.0] * 3)
    cl = O.build(g, pts)
    ooff, onb = O.neighbor_lists(g, cl, pts, pts)
    onb_sorted = np.concatenate([np.sort(onb[ooff[i]:ooff[i + 1]]) for i in range(len(pts))])
    assert np.array_equal(cnt.cpu().numpy() - 1, np.diff(ooff) - 1)
    assert np.array_equal(off.cpu().numpy(), ooff)
    assert np.array_equal(nb.cpu().numpy(), onb_sorted)
    sample = np.arange(0, len(pts), 61)
    toff, tnb = O.trivial_lists(g, pts[sample], pts)
    offn = off.cpu().numpy()
    nbn = nb.cpu().numpy()
    for q, i in enumerate(sample):
        assert np.array_equal(nbn[offn[i]:offn[i + 1]], tnb[toff[q]:toff[q + 1]])


def _rel_err(gpu, ref, absum):
    return float(np.max(np.abs(gpu - ref) / np.maximum(absum, 1e-300)))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_wcsph_vs_oracle(P, O, dt):
    W = P.workloads
    x, v, _ = W.wcsph_cloud(30, seed=2, dtype=dt)
    n = len(x)
    r = 3.0
    nhs = make_nhs(P, 3, r, [-1.0] * 3, [31.0] * 3, n, dtype=dt)
    xd = dcoords(x)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    P.initialize(nhs, xd, xd)
    T = torch.float32 if dt == np.float32 else torch.float64
    rho = torch.zeros(n, dtype=T, device="cuda")
    p = torch.zeros(n, dtype=T, device="cuda")
    acc = torch.zeros(n * 3, dtype=T, device="cuda")
    P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=p, velocity=vd, accel=acc,
                                         **W.WCSPH), xd, xd, nhs)
    g = O.grid_create(3, dt(r), np.array([-1.0] * 3, dt), np.array([31.0] * 3, dt), dtype=dt)
    cl = O.build(g, x)
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl, x, x, O.F_WCSPH_DENSITY, prm, want_abs=True)
    tol = TOL_F32 if dt == np.float32 else TOL_F64
    assert _rel_err(rho.cpu().numpy().astype(np.float64), orho, oab) < tol
    # force: the oracle sums the same inputs (the GPU's density and pressure) in FP64
    rho_h = rho.cpu().numpy().astype(np.float64)
    p_h = p.cpu().numpy().astype(np.float64)
    prm, keep = O.make_params(rho=rho_h, pressure=p_h, vel=v.astype(np.float64),
                              r_min=float(np.sqrt(np.finfo(dt).eps)) * W.WCSPH["h"], **W.WCSPH)
    oacc, oab = O.foreach(g, cl, x, x, O.F_WCSPH_FORCE, prm, want_abs=True)
    assert _rel_err(acc.cpu().numpy().reshape(n, 3).astype(np.float64), oacc, oab) < tol
    # standalone FORCE (gathering the state) equals the fused step
    acc2 = torch.zeros_like(acc)
    P.foreach_point_neighbor(P.WCSPHForce(density=rho, pressure=p, velocity=vd, accel=acc2,
                                          **W.WCSPH), xd, xd, nhs)
    assert torch.equal(acc, acc2)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_nbody_vs_oracle(P, O, dt):
    W = P.workloads
    x = W.perturbed_lattice((25, 26, 27), 0.25, seed=4, dtype=dt)
    n = len(x)
    m = np.random.default_rng(5).uniform(1e10, 2e10, n).astype(dt)
    r = 3.0
    mn, mx = x.min(0) - r, x.max(0) + r
    nhs = make_nhs(P, 3, r, mn, mx, n, dtype=dt)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    T = torch.float32 if dt == np.float32 else torch.float64
    acc = torch.zeros(n * 3, dtype=T, device="cuda")
    G = 6.6743e-11
    P.foreach_point_neighbor(P.NBodyAcceleration(torch.as_tensor(m, device="cuda"), G, acc),
                             xd, xd, nhs)
    g = O.grid_create(3, dt(r), mn.astype(dt), mx.astype(dt), dtype=dt)
    prm, keep = O.make_params(G=G, masses=m.astype(np.float64))
    oacc, oab = O.foreach(g, O.build(g, x), x, x, O.F_NBODY_ACCEL, prm, want_abs=True)
    tol = TOL_F32 if dt == np.float32 else TOL_F64
    assert _rel_err(acc.cpu().numpy().reshape(n, 3).astype(np.float64), oacc, oab) < tol


def test_periodic_potential_2d_vs_oracle(P, O):
    """The 2D periodic n-body workload at 256^2 points: neighbour sets including periodic
    images bit-exact against the oracle's Grid search and brute force, FP32 potential sums
    within 1e-5 of FP64."""
    W = P.workloads
    x, m = W.periodic_nbody_cloud(256, seed=6, dtype=np.float32)
    n = len(x)
    r = np.float32(2.5)
    box = (np.zeros(2, np.float32), np.full(2, 256.0, np.float32))
    nhs = make_nhs(P, 2, r, box[0], box[1], n, dtype=np.float32, box=box)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    g = O.grid_create(2, r, box[0], box[1], periodic_box=box, dtype=np.float32)
    cl = O.build(g, x)
    off, nb = P.neighbor_lists(xd, xd, nhs)
    ooff, onb = O.neighbor_lists(g, cl, x, x)
    onb_sorted = np.concatenate([np.sort(onb[ooff[i]:ooff[i + 1]]) for i in range(n)])
    assert np.array_equal(off.cpu().numpy(), ooff)
    assert np.array_equal(nb.cpu().numpy(), onb_sorted)
    sample = np.arange(0, n, 97)
    toff, tnb = O.trivial_lists(g, x[sample], x)
    offn, nbn = off.cpu().numpy(), nb.cpu().numpy()
    for q, i in enumerate(sample):
        assert np.array_equal(nbn[offn[i]:offn[i + 1]], tnb[toff[q]:toff[q + 1]])
    e = torch.zeros(n, dtype=torch.float32, device="cuda")
    P.foreach_point_neighbor(P.TruncatedPotential(torch.as_tensor(m, device="cuda"), 2.5, e),
                             xd, xd, nhs)
    prm, keep = O.make_params(masses=m.astype(np.float64), cutoff=2.5)
    oe, oab = O.foreach(g, cl, x, x, O.F_POTENTIAL, prm, want_abs=True)
    assert _rel_err(e.cpu().numpy().astype(np.float64), oe, oab) < TOL_F32


@pytest.mark.parametrize("fraction", [1.0, 0.0])
def test_incremental_update_matches_rebuild(P, O, fraction):
    """ParallelIncrementalUpdate after an N(0, 0.05^2) displacement, with overflow lists
    (fraction 1) or a device-side rebuild (fraction 0): the same cell list and neighbour
    sets as a full rebuild, sums within tolerance (summation order differs with overflow
    lists; identical after a rebuild)."""
    W = P.workloads
    x, v, dx = W.wcsph_cloud(40, seed=7, dtype=np.float32)
    x1 = (x + dx).astype(np.float32)
    n = len(x)
    nhs_i = make_nhs(P, 3, np.float32(3.0), [-1.0] * 3, [41.0] * 3, n, dtype=np.float32,
                     strategy=P.ParallelIncrementalUpdate(fraction))
    nhs_f = make_nhs(P, 3, np.float32(3.0), [-1.0] * 3, [41.0] * 3, n, dtype=np.float32)
    x0d, x1d = dcoords(x), dcoords(x1)
    P.initialize(nhs_i, x0d, x0d)
    P.update(nhs_i, x1d, x1d)
    P.initialize(nhs_f, x1d, x1d)
    assert nhs_i.grid_info()["n_binned"] == n
    ci, pi = P.export_cells(nhs_i)
    cf, pf = P.export_cells(nhs_f)
    assert np.array_equal(ci, cf) and np.array_equal(pi, pf)
    oi, ni = P.neighbor_lists(x1d, x1d, nhs_i)
    of, nf = P.neighbor_lists(x1d, x1d, nhs_f)
    assert torch.equal(oi, of) and torch.equal(ni, nf)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    outs = []
    for nhs in (nhs_i, nhs_f):
        rho = torch.zeros(n, device="cuda")
        p = torch.zeros(n, device="cuda")
        acc = torch.zeros(3 * n, device="cuda")
        P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=p, velocity=vd, accel=acc,
                                             **W.WCSPH), x1d, x1d, nhs)
        outs.append((rho, acc))
    assert torch.allclose(outs[0][0], outs[1][0], rtol=1e-6, atol=0)
    scale = outs[1][1].abs().max()
    assert float((outs[0][1] - outs[1][1]).abs().max() / scale) < 1e-4
    if fraction == 0.0:  # rebuilt: the same layout, hence the same sums bit for bit
        assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
        assert nhs_i.grid_info()["n_overflow"] == 0
    # the standalone force call (state gathered from the arrays) after the incremental
    # update gives the fused step's result bit for bit
    rho_i = torch.zeros(n, device="cuda")
    p_i = torch.zeros(n, device="cuda")
    P.foreach_point_neighbor(P.WCSPHDensity(density=rho_i, pressure=p_i, **W.WCSPH),
                             x1d, x1d, nhs_i)
    acc2 = torch.zeros(3 * n, device="cuda")
    P.foreach_point_neighbor(P.WCSPHForce(density=rho_i, pressure=p_i, velocity=vd, accel=acc2,
                                          **W.WCSPH), x1d, x1d, nhs_i)
    assert torch.equal(rho_i, outs[0][0]) and torch.equal(acc2, outs[0][1])
    # a second update back to the original positions empties the overflow
    P.update(nhs_i, x0d, x0d)
    P.initialize(nhs_f, x0d, x0d)
    ci, pi = P.export_cells(nhs_i)
    cf, pf = P.export_cells(nhs_f)
    assert np.array_equal(ci, cf) and np.array_equal(pi, pf)


def test_incremental_random_walk(P):
    """Ten update! calls along a random walk (N(0, 0.05^2) per step, ~8 % of the points
    change cell per step) with rebuild_fraction 0.1: the device switches between overflow
    lists and rebuilds; after every step the cell list and the neighbour lists equal a
    fresh ParallelUpdate build."""
    W = P.workloads
    x, _, _ = W.wcsph_cloud(30, seed=5, dtype=np.float32)
    n = len(x)
    nhs_i = make_nhs(P, 3, np.float32(3.0), [-1.0] * 3, [31.0] * 3, n, dtype=np.float32,
                     strategy=P.ParallelIncrementalUpdate(0.1))
    nhs_f = make_nhs(P, 3, np.float32(3.0), [-1.0] * 3, [31.0] * 3, n, dtype=np.float32)
    rng = np.random.default_rng(11)
    xs = x.astype(np.float64)
    xd = dcoords(x)
    P.initialize(nhs_i, xd, xd)
    seen = set()
    for _ in range(10):
        xs = xs + rng.normal(0, 0.05, size=xs.shape)
        xd = dcoords(xs.astype(np.float32))
        P.update(nhs_i, xd, xd)
        P.initialize(nhs_f, xd, xd)
        ci, pi = P.export_cells(nhs_i)
        cf, pf = P.export_cells(nhs_f)
        assert np.array_equal(ci, cf) and np.array_equal(pi, pf)
        oi, ni = P.neighbor_lists(xd, xd, nhs_i)
        of, nf = P.neighbor_lists(xd, xd, nhs_f)
        assert torch.equal(oi, of) and torch.equal(ni, nf)
        torch.cuda.synchronize()
        n_ovf = nhs_i.grid_info()["n_overflow"]
        assert n_ovf <= 0.1 * n
        seen.add(n_ovf == 0)
    assert seen == {True, False}  # both paths were taken


def test_determinism(P):
    """Cell-sorted order is a function of the input (not of atomic timing): repeated
    builds and sweeps give bit-identical results."""
    W = P.workloads
    x, v, _ = W.wcsph_cloud(32, seed=8, dtype=np.float32)
    n = len(x)
    nhs = make_nhs(P, 3, np.float32(3.0), [-1.0] * 3, [33.0] * 3, n, dtype=np.float32)
    xd = dcoords(x)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    res = []
    for _ in range(3):
        P.initialize(nhs, xd, xd)
        rho = torch.zeros(n, device="cuda")
        p = torch.zeros(n, device="cuda")
        acc = torch.zeros(3 * n, device="cuda")
        P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=p, velocity=vd, accel=acc,
                                             **W.WCSPH), xd, xd, nhs)
        res.append((rho, acc))
    for r in res[1:]:
        assert torch.equal(r[0], res[0][0]) and torch.equal(r[1], res[0][1])


# ----------------------------------------------------------------- full-size properties

def test_wcsph_8m_sample_vs_oracle(P, O):
    """The 200^3 FP32 WCSPH workload at full size: density and force of a sample of query
    points against the FP64 oracle (which bins all 8M points), neighbour counts exact."""
    W = P.workloads
    x, v, dx = W.wcsph_cloud(200, seed=1, dtype=np.float32)
    n = len(x)
    nhs = make_nhs(P, 3, np.float32(3.0), [-1.0] * 3, [201.0] * 3, n, dtype=np.float32,
                   strategy=P.ParallelIncrementalUpdate())
    xd = dcoords(x)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    P.initialize(nhs, xd, xd)
    x1 = (x + dx).astype(np.float32)
    x1d = dcoords(x1)
    P.update(nhs, x1d, x1d)
    rho = torch.zeros(n, device="cuda")
    p = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=p, velocity=vd, accel=acc,
                                         **W.WCSPH), x1d, x1d, nhs)
    P.foreach_point_neighbor(P.CountNeighbors(cnt), x1d, x1d, nhs)
    g = O.grid_create(3, np.float32(3.0), np.full(3, -1.0, np.float32),
                      np.full(3, 201.0, np.float32), dtype=np.float32)
    cl = O.build(g, x1)
    sample = np.random.default_rng(0).choice(n, 20000, replace=False).astype(np.int32)
    ocnt = O.foreach(g, cl, x1, x1, O.F_COUNT, points=sample)
    assert np.array_equal(cnt.cpu().numpy()[sample], ocnt[sample])
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl, x1, x1, O.F_WCSPH_DENSITY, prm, points=sample, want_abs=True)
    rho_h = rho.cpu().numpy().astype(np.float64)
    assert _rel_err(rho_h[sample], orho[sample], oab[sample]) < TOL_F32
    prm, keep = O.make_params(rho=rho_h, pressure=p.cpu().numpy().astype(np.float64),
                              vel=v.astype(np.float64),
                              r_min=float(np.sqrt(np.finfo(np.float32).eps)) * 1.5, **W.WCSPH)
    oacc, oab = O.foreach(g, cl, x1, x1, O.F_WCSPH_FORCE, prm, points=sample, want_abs=True)
    a = acc.cpu().numpy().reshape(n, 3).astype(np.float64)
    assert _rel_err(a[sample], oacc[sample], oab[sample]) < TOL_F32


def test_periodic_16m_properties(P, O):
    """The 4096^2 periodic FP32 workload at full size: counts of a sample equal the
    oracle's, and the neighbour relation is symmetric (sum of counts over all points equals
    the number of ordered pairs found from the other side)."""
    W = P.workloads
    x, m = W.periodic_nbody_cloud(4096, seed=1, dtype=np.float32)
    n = len(x)
    box = (np.zeros(2, np.float32), np.full(2, 4096.0, np.float32))
    nhs = make_nhs(P, 2, np.float32(2.5), box[0], box[1], n, dtype=np.float32, box=box)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, xd, nhs)
    sums = torch.zeros(n, dtype=torch.int64, device="cuda")
    P.foreach_point_neighbor(P.NeighborIndexSum(sums), xd, xd, nhs)
    g = O.grid_create(2, np.float32(2.5), box[0], box[1], periodic_box=box, dtype=np.float32)
    cl = O.build(g, x)
    sample = np.random.default_rng(1).choice(n, 50000, replace=False).astype(np.int32)
    ocnt = O.foreach(g, cl, x, x, O.F_COUNT, points=sample)
    osum = O.foreach(g, cl, x, x, O.F_INDEX_SUM, points=sample)
    assert np.array_equal(cnt.cpu().numpy()[sample], ocnt[sample])
    assert np.array_equal(sums.cpu().numpy()[sample], osum[sample])
    # symmetry: sum_i sum_{j in N(i)} (j+1) == sum_j count_j * (j+1)
    idx1 = torch.arange(1, n + 1, dtype=torch.int64, device="cuda")
    assert int(sums.sum()) == int((cnt.to(torch.int64) * idx1).sum())


# ----------------------------------------------------------------- 1D and rectangular boxes

RECT_CASES = [
    # (ndims, radius, box min, box max, periodic)
    (1, 1.3, [0.0], [50.0], False),
    (1, 1.3, [0.0], [50.0], True),
    (2, 1.5, [0.0, 0.0], [20.0, 7.0], True),
    (3, 2.2, [0.0, 0.0, 0.0], [12.0, 15.0, 9.0], True),
    (3, 2.2, [-3.0, 1.0, 0.5], [9.0, 16.0, 9.5], False),
]


@pytest.mark.parametrize("case", RECT_CASES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_grid_equals_trivial_1d_and_rectangular_boxes(P, O, case, dt):
    """PeriodicBox with different sizes per dimension and 1D searches (nhs_grid.jl:117-124):
    neighbour lists (periodic images included) equal brute force; sums over the same pairs
    agree with the oracle."""
    d, r, lo, hi, per = case
    lo, hi = np.asarray(lo), np.asarray(hi)
    rng = np.random.default_rng(d * 10 + int(per))
    n = 600 if d == 1 else 1500
    x = (lo + rng.uniform(0, 1, size=(n, d)) * (hi - lo)).astype(dt)
    box = (lo, hi) if per else None
    nhs = make_nhs(P, d, r, lo, hi, n, dtype=dt, box=box)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    g = O.grid_create(d, dt(r), lo.astype(dt), hi.astype(dt), dtype=dt,
                      periodic_box=(lo.astype(dt), hi.astype(dt)) if per else None)
    toff, tnb = O.trivial_lists(g, x, x)
    off, nb = P.neighbor_lists(xd, xd, nhs)
    assert np.array_equal(off.cpu().numpy(), toff)
    assert np.array_equal(nb.cpu().numpy(), tnb)
    # the truncated potential over the same pairs (periodic images included)
    m = rng.uniform(0.5, 1.5, size=n).astype(dt)
    e = torch.zeros(n, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    P.foreach_point_neighbor(P.TruncatedPotential(torch.as_tensor(m, device="cuda"), r, e),
                             xd, xd, nhs)
    cl = O.build(g, x)
    prm, keep = O.make_params(masses=m.astype(np.float64), cutoff=r)
    oe, oab = O.foreach(g, cl, x, x, O.F_POTENTIAL, prm, want_abs=True)
    tol = TOL_F32 if dt == np.float32 else TOL_F64
    assert _rel_err(e.cpu().numpy().astype(np.float64), oe, oab) < tol


def test_every_update_strategy_gives_the_same_lists(P, O):
    """The reference's five strategies for a FullGridCellList (full_grid.jl:39-42): on the GPU
    the serial and semi-parallel ones are the parallel rebuild and incremental update, and
    all give the brute-force lists after initialize! and update!."""
    W = P.workloads
    r = 2.5
    c1 = W.reference_test_cloud((30, 31, 29), r, seed=1)
    c2 = W.reference_test_cloud((30, 31, 29), r, seed=2)
    mn = np.minimum(c1.min(0), c2.min(0)) - r
    mx = np.maximum(c1.max(0), c2.max(0)) + r
    toff, tnb = O.trivial_lists(O.grid_create(3, r, mn, mx), c2, c2)
    for strat in (P.ParallelUpdate(), P.ParallelIncrementalUpdate(), P.SemiParallelUpdate(),
                  P.SerialIncrementalUpdate(), P.SerialUpdate()):
        nhs = make_nhs(P, 3, r, mn, mx, len(c1), strategy=strat)
        P.initialize(nhs, dcoords(c1), dcoords(c1))
        x = dcoords(c2)
        P.update(nhs, x, x)
        off, nb = P.neighbor_lists(x, x, nhs)
        assert np.array_equal(off.cpu().numpy(), toff), strat
        assert np.array_equal(nb.cpu().numpy(), tnb), strat


def test_fma_probe(P):
    """The measurement aid behind bench.py's Float32 roofline: every thread's value is
    finite (nothing elided) and a launch takes a plausible time."""
    out = torch.zeros(P._lib.PN_FMA_PROBE_THREADS, dtype=torch.float32, device="cuda")
    assert P.lib().pn_fma_probe(out.data_ptr(), 64, P._stream()) == 0
    torch.cuda.synchronize()
    assert bool(torch.isfinite(out).all()) and float(out.min()) > 0


def test_bounded_wait_gives_up(P):
    """The library's one device-side wait (the cell-list scan's look-back) is bounded: with
    a predecessor tile that never publishes, the scan records PN_ERR_TIMEOUT and returns
    (after about a second), and the context stays usable for the next search."""
    import time
    t0 = time.perf_counter()
    assert P.lib().pn_selftest_bounded_wait(P._stream()) == P._lib.PN_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 60
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [5.0, 5.0]])
    nhs = make_nhs(P, 2, 1.5, [-2.0, -2.0], [7.0, 7.0], 3)
    x = dcoords(pts)
    P.initialize(nhs, x, x)
    cnt = torch.zeros(3, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), x, x, nhs)
    assert cnt.tolist() == [2, 2, 1]


def test_per_point_api(P, O):
    """foreach_neighbor / mapreduce_neighbor for one point (neighborhood_search.jl:250-421)
    and the initialize_grid! / update_grid! spellings, against brute force."""
    W = P.workloads
    r = 2.5
    c = W.reference_test_cloud((12, 13, 11), r, seed=3)
    mn, mx = c.min(0) - r, c.max(0) + r
    nhs = make_nhs(P, 3, r, mn, mx, len(c))
    x = dcoords(c)
    P.initialize_grid(nhs, x)
    toff, tnb = O.trivial_lists(O.grid_create(3, r, mn, mx), c, c)
    for i in (0, 77, len(c) - 1):
        row = tnb[toff[i]:toff[i + 1]]
        assert P.mapreduce_neighbor("count", "+", x, x, nhs, i, init=0) == len(row)
        assert P.mapreduce_neighbor("index", "+", x, x, nhs, i, init=5) == 5 + int((row + 1).sum())
        cnt = torch.full((len(c),), -7, dtype=torch.int32, device="cuda")
        P.foreach_neighbor(P.CountNeighbors(cnt), x, x, nhs, i)
        got = cnt.cpu().numpy()
        assert got[i] == len(row) and (np.delete(got, i) == -7).all()
    c2 = c + 0.1
    x2 = dcoords(c2)
    P.update_grid(nhs, x2)
    off, nb = P.neighbor_lists(x2, x2, nhs)
    toff, tnb = O.trivial_lists(O.grid_create(3, r, mn, mx), c2, c2)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)
