"""Mixed precision (Float64 coordinates, Float32 search radius; PN_FLAG_FLOAT32_SEARCH)
against the oracle's restatement (pno_grid_create_mixed) of the reference's rule
(neighborhood_search.jl:402-410, docs/literate/src/tut_gpu_usage.jl:38-50): cells in Float64,
pos_diff converted to Float32, d^2, the periodic correction and the test in Float32.

Bars: neighbour lists and counts bit-exact against the oracle (grid and brute force),
including pairs placed within Float32 rounding of the radius; WCSPH sums within 1e-5 of
the FP64 oracle relative to sum |terms| (the pair functions compute in Float32)."""
import numpy as np
import pytest
import torch

from test_gpu_parity import TOL_F32, _rel_err, csr_rows, dcoords

pytestmark = pytest.mark.gpu

R = np.float32(0.9)


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _mixed(P, d, lo, hi, n, periodic=False, strategy=None, r=R):
    """A mixed search over [lo, hi] (the periodic box itself when periodic)."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    box = None
    if periodic:
        box = P.PeriodicBox(min_corner=lo.astype(np.float32), max_corner=hi.astype(np.float32))
        cl = P.FullGridCellList(min_corner=lo, max_corner=hi, search_radius=r,
                                max_points_per_cell=0)
    else:
        cl = P.FullGridCellList(min_corner=lo - r, max_corner=hi + r, search_radius=r,
                                max_points_per_cell=0)
    nhs = P.GridNeighborhoodSearch(d, search_radius=r, n_points=n, cell_list=cl,
                                   periodic_box=box, update_strategy=strategy)
    assert nhs.mixed and nhs.eltype == np.float32 and nhs.coord_eltype == np.float64
    return nhs


def _oracle(O, d, lo, hi, periodic=False, r=R):
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    if periodic:
        return O.grid_create_mixed(d, r, lo, hi, periodic_box=(lo, hi))
    return O.grid_create_mixed(d, r, lo - r, hi + r)


def _near_radius_cloud(d, side, seed):
    """A lattice of spacing exactly R (as Float64) with offsets of 1e-9: many pairs lie
    within Float32 rounding of the radius, on both sides in Float64."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(side)] * d, indexing="ij"), -1).reshape(-1, d)
    return g * float(R) + 0.05 + rng.uniform(-1e-9, 1e-9, g.shape)


CASES = [(2, False), (2, True), (3, False), (3, True)]


@pytest.mark.parametrize("d,periodic", CASES)
def test_mixed_lists_equal_oracle(P, O, d, periodic):
    rng = np.random.default_rng(3 + d)
    hi = np.array([9.0, 8.1, 7.3][:d])
    y = rng.uniform(0.0, hi, size=(6000 if d == 3 else 4000, d))
    y = np.concatenate([y, _near_radius_cloud(d, 8, seed=d)])
    n = len(y)
    nhs = _mixed(P, d, np.zeros(d), hi, n, periodic)
    yd = dcoords(y)
    P.initialize(nhs, yd, yd)
    off, nb = P.neighbor_lists(yd, yd, nhs)
    g = _oracle(O, d, np.zeros(d), hi, periodic)
    toff, tnb = O.trivial_lists(g, y, y)
    assert np.array_equal(off.cpu().numpy(), toff)
    assert np.array_equal(nb.cpu().numpy(), tnb)
    # the Float32 test decides: a Float64 search over the same points differs
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), yd, yd, nhs)
    assert np.array_equal(cnt.cpu().numpy(), np.diff(toff))
    g64 = O.grid_create(d, float(R), (np.zeros(d) if periodic else -float(R) * np.ones(d)),
                        hi + (0 if periodic else float(R)),
                        periodic_box=(np.zeros(d), hi) if periodic else None)
    c64, _ = O.trivial_lists(g64, y, y)
    assert not np.array_equal(c64, toff)


def test_mixed_boundary_pairs(P, O):
    """A pair 1e-12 beyond the radius in Float64 is a neighbour (its Float32 pos_diff is
    r), one Float32 step beyond is not."""
    r = np.float32(1.7)
    step = float(np.nextafter(r, np.float32(np.inf)))
    y = np.array([[0.0, 0.0], [float(r) + 1e-12, 0.0], [step, 0.0]])
    cl = P.FullGridCellList(min_corner=[-3.0, -3.0], max_corner=[5.0, 3.0], search_radius=r)
    nhs = P.GridNeighborhoodSearch(2, search_radius=r, n_points=3, cell_list=cl)
    yd = dcoords(y)
    P.initialize(nhs, yd, yd)
    rows = [sorted(v.tolist()) for v in csr_rows(*P.neighbor_lists(yd, yd, nhs))]
    assert rows == [[0, 1], [0, 1, 2], [1, 2]]


@pytest.mark.parametrize("periodic", [False, True])
def test_mixed_queries_not_y_and_incremental_update(P, O, periodic):
    rng = np.random.default_rng(17)
    hi = np.array([10.0, 9.0, 8.0])
    y = rng.uniform(0.0, hi, size=(20000, 3))
    xq = rng.uniform(0.0, hi, size=(3000, 3))
    nhs = _mixed(P, 3, np.zeros(3), hi, len(y), periodic,
                 strategy=P.ParallelIncrementalUpdate(rebuild_fraction=1.0))
    g = _oracle(O, 3, np.zeros(3), hi, periodic)
    yd, xd = dcoords(y), dcoords(xq)
    P.initialize(nhs, xd, yd)
    off, nb = P.neighbor_lists(xd, yd, nhs)
    toff, tnb = O.trivial_lists(g, xq, y)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)
    # an incremental update (overflow lists) keeps the exact Float32 decisions
    y2 = np.clip(y + rng.normal(0, 0.2, y.shape), 0.0, np.nextafter(hi, 0))
    y2d = dcoords(y2)
    P.update(nhs, y2d, y2d)
    assert nhs.grid_info()["n_overflow"] > 0
    off, nb = P.neighbor_lists(y2d, y2d, nhs)
    toff, tnb = O.trivial_lists(g, y2, y2)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)


def test_mixed_wcsph_vs_oracle(P, O):
    W = P.workloads
    x, v, _ = W.wcsph_cloud(24, seed=9, dtype=np.float64)
    n = len(x)
    r = np.float32(3.0)
    lo, hi = np.full(3, -1.0), np.full(3, 25.0)
    cl = P.FullGridCellList(min_corner=lo, max_corner=hi, search_radius=r)
    nhs = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    rho = torch.zeros(n, device="cuda")
    prs = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    vd = torch.as_tensor(v.astype(np.float32), device="cuda").reshape(-1)
    P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd, accel=acc,
                                         **W.WCSPH), xd, xd, nhs)
    g = O.grid_create_mixed(3, r, lo, hi)
    cl_o = O.build(g, x)
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl_o, x, x, O.F_WCSPH_DENSITY, prm, want_abs=True)
    assert _rel_err(rho.cpu().numpy().astype(np.float64), orho, oab) < TOL_F32
    c = W.WCSPH
    prm2, keep2 = O.make_params(rho=rho.cpu().numpy().astype(np.float64),
                                pressure=prs.cpu().numpy().astype(np.float64),
                                vel=v.astype(np.float32).astype(np.float64),
                                r_min=float(np.sqrt(np.finfo(np.float32).eps)) * c["h"], **c)
    oacc, oabs = O.foreach(g, cl_o, x, x, O.F_WCSPH_FORCE, prm2, want_abs=True)
    got = acc.cpu().numpy().astype(np.float64).reshape(n, 3)
    assert _rel_err(got, oacc, oabs) < TOL_F32
    # the standalone force (state gathered from the user's arrays) equals the fused step
    acc2 = torch.zeros_like(acc)
    P.foreach_point_neighbor(P.WCSPHForce(density=rho, pressure=prs, velocity=vd, accel=acc2,
                                          **W.WCSPH), xd, xd, nhs)
    assert torch.equal(acc, acc2)


def test_mixed_precomputed_lists(P, O):
    rng = np.random.default_rng(23)
    hi = np.array([8.0, 8.0, 8.0])
    y = np.concatenate([rng.uniform(0.0, hi, size=(8000, 3)), _near_radius_cloud(3, 8, 5)])
    n = len(y)
    grid = _mixed(P, 3, np.zeros(3), hi, n)
    pre = P.PrecomputedNeighborhoodSearch(3, n_points=n, update_neighborhood_search=grid)
    yd = dcoords(y)
    P.initialize(pre, yd, yd)
    off, nb = P.neighbor_lists(yd, yd, pre)
    toff, tnb = O.trivial_lists(_oracle(O, 3, np.zeros(3), hi), y, y)
    assert np.array_equal(off.cpu().numpy(), toff) and np.array_equal(nb.cpu().numpy(), tnb)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), yd, yd, pre)
    assert np.array_equal(cnt.cpu().numpy(), np.diff(toff))


def test_mixed_adjoint_matches_float64_search(P):
    """The adjoint over a mixed search: Float32 arithmetic, gradients returned in the
    coordinates' Float64, close to the same loss over a Float64 search."""
    W = P.workloads
    x, _, _ = W.wcsph_cloud(12, seed=4, dtype=np.float64)
    n = len(x)
    lo, hi = np.full(3, -1.0), np.full(3, 13.0)
    nm = P.GridNeighborhoodSearch(3, search_radius=np.float32(3.0), n_points=n,
                                  cell_list=P.FullGridCellList(min_corner=lo, max_corner=hi,
                                                               search_radius=np.float32(3.0)))
    n64 = P.GridNeighborhoodSearch(3, search_radius=3.0, n_points=n,
                                   cell_list=P.FullGridCellList(min_corner=lo, max_corner=hi,
                                                                search_radius=3.0))
    xm = dcoords(x).clone().requires_grad_(True)
    x64 = dcoords(x).clone().requires_grad_(True)
    lm = P.adjoint_loss(xm, nm)
    l64 = P.adjoint_loss(x64, n64)
    lm.backward()
    l64.backward()
    assert xm.grad.dtype == torch.float64
    assert abs(float(lm.detach()) - float(l64.detach())) <= 1e-5 * abs(float(l64.detach()))
    gm, g64 = xm.grad.cpu().numpy(), x64.grad.cpu().numpy()
    assert np.max(np.abs(gm - g64)) <= 1e-3 * np.max(np.abs(g64))


def test_golden_gpu_tutorial_mixed(P, golden):
    """docs/literate/src/tut_gpu_usage.jl:38-50 with Float64 coordinates and the tutorial's
    Float32 radius 3.0f0 (the tutorial's mixed-precision variant): the neighbour counts'
    extrema of test/gpu.jl:35."""
    c = golden["gpu_tutorial"]
    pts = P.workloads.lattice(c["n_per_dim"], dtype=np.float64)
    r = np.float32(c["radius"])
    cl = P.FullGridCellList(min_corner=pts.min(0), max_corner=pts.max(0), search_radius=r)
    nhs = P.GridNeighborhoodSearch(2, search_radius=r, n_points=len(pts), cell_list=cl)
    assert nhs.mixed
    x = dcoords(pts)
    P.initialize(nhs, x, x)
    n = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(n), x, x, nhs)
    assert (int(n.min()), int(n.max())) == tuple(c["expected_extrema"])


@pytest.mark.parametrize("periodic", [False, True])
def test_mixed_pair_cache(P, O, periodic):
    """The pair cache over a mixed search's Float32 traversal: the density sweep records
    the pairs the exact Float32 test accepts, the force walks them; density bit-identical
    to the search without the cache, force within the FP32 bar of the FP64 oracle."""
    W = P.workloads
    x, v, _ = W.wcsph_cloud(20, seed=13, dtype=np.float64)
    n = len(x)
    r = np.float32(3.0)
    lo, hi = (np.zeros(3), np.full(3, 20.0)) if periodic else (np.full(3, -1.0), np.full(3, 21.0))
    if periodic:
        x = np.mod(x, 20.0)
    xd = dcoords(x)
    vd = torch.as_tensor(v.astype(np.float32), device="cuda").reshape(-1)
    out = []
    for cache in (False, True):
        box = P.PeriodicBox(min_corner=lo.astype(np.float32),
                            max_corner=hi.astype(np.float32)) if periodic else None
        cl = P.FullGridCellList(min_corner=lo, max_corner=hi, search_radius=r,
                                max_points_per_cell=0)
        nhs = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl,
                                       periodic_box=box, pair_cache=cache)
        assert nhs.mixed
        P.initialize(nhs, xd, xd)
        rho = torch.zeros(n, device="cuda")
        prs = torch.zeros(n, device="cuda")
        acc = torch.zeros(3 * n, device="cuda")
        for _ in range(2):  # the second step walks the cache
            P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd,
                                                 accel=acc, **W.WCSPH), xd, xd, nhs)
        out.append((rho.clone(), prs.clone(), acc.clone()))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    g = (O.grid_create_mixed(3, r, lo, hi, periodic_box=(lo, hi)) if periodic
         else O.grid_create_mixed(3, r, lo, hi))
    cl_o = O.build(g, x)
    c = W.WCSPH
    prm, keep = O.make_params(rho=out[1][0].cpu().numpy().astype(np.float64),
                              pressure=out[1][1].cpu().numpy().astype(np.float64),
                              vel=v.astype(np.float32).astype(np.float64),
                              r_min=float(np.sqrt(np.finfo(np.float32).eps)) * c["h"], **c)
    oacc, oabs = O.foreach(g, cl_o, x, x, O.F_WCSPH_FORCE, prm, want_abs=True)
    for k in (0, 1):
        got = out[k][2].cpu().numpy().astype(np.float64).reshape(n, 3)
        assert _rel_err(got, oacc, oabs) < TOL_F32
