"""PrecomputedNeighborhoodSearch (the pn_pre_* C ABI) against the reference's known answers,
the grid search and the FP64 oracle.

Bars: neighbour lists bit-exact (the reference's test/neighborhood_search.jl:163-180 known
answers, the grid search's lists, brute force); counts bit-exact; WCSPH density and force
within 1e-5 (FP32) of the FP64 oracle relative to sum |terms|, like the grid search."""
import numpy as np
import pytest
import torch

from test_gpu_parity import _periodic_setup, csr_rows, dcoords, make_nhs, _rel_err, TOL_F32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _pre(P, d, r, mn, mx, n, dtype=np.float64, box=None, max_neighbors=None, strategy=None):
    grid = make_nhs(P, d, r, mn, mx, n, dtype=dtype, box=box, strategy=strategy, max_ppc=0)
    return P.PrecomputedNeighborhoodSearch(d, n_points=n, update_neighborhood_search=grid,
                                           max_neighbors=max_neighbors)


def test_golden_periodic_neighbors_precomputed(P, golden):
    c = golden["periodic_neighbors"]
    for s in c["setups"]:
        y, bmin, bmax = _periodic_setup(s)
        d = y.shape[1]
        nhs = _pre(P, d, c["radius"], bmin, bmax, len(y), box=(bmin, bmax))
        x = dcoords(y)
        P.initialize(nhs, x, x)
        rows = csr_rows(*P.neighbor_lists(x, x, nhs))
        for i, exp in enumerate(c["expected"]):
            assert (rows[i] + 1).tolist() == exp, s["name"]
        cnt = torch.zeros(len(y), dtype=torch.int32, device="cuda")
        P.foreach_point_neighbor(P.CountNeighbors(cnt), x, x, nhs)
        assert cnt.cpu().tolist() == [len(e) for e in c["expected"]]


@pytest.mark.parametrize("shape", [(10, 11), (9, 10, 7), (39, 40, 41)])
def test_precomputed_lists_equal_grid_and_trivial(P, O, shape):
    W = P.workloads
    r = 2.5
    coords = W.reference_test_cloud(shape, r, seed=2)
    d = len(shape)
    mn, mx = coords.min(0) - r, coords.max(0) + r
    grid = make_nhs(P, d, r, mn, mx, len(coords))
    pre = _pre(P, d, r, mn, mx, len(coords))
    x = dcoords(coords)
    P.initialize(grid, x, x)
    P.initialize(pre, x, x)
    og, ng = P.neighbor_lists(x, x, grid)
    op, npre = P.neighbor_lists(x, x, pre)
    assert torch.equal(og, op) and torch.equal(ng, npre)
    g = O.grid_create(d, r, mn, mx)
    toff, tnb = O.trivial_lists(g, coords, coords)
    assert np.array_equal(op.cpu().numpy(), toff) and np.array_equal(npre.cpu().numpy(), tnb)
    # a subset of query points reads its rows through the slot map
    pts = np.arange(0, len(coords), 7)
    c1 = torch.zeros(len(coords), dtype=torch.int32, device="cuda")
    c2 = torch.zeros(len(coords), dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(c1), x, x, grid, points=pts)
    P.foreach_point_neighbor(P.CountNeighbors(c2), x, x, pre, points=pts)
    assert torch.equal(c1, c2)
    assert P.requires_update(pre) == (True, True) and P.requires_update(grid) == (False, True)


def test_precomputed_x_not_y_and_update(P, O):
    W = P.workloads
    y = W.perturbed_lattice((16, 16, 16), 0.25, seed=3)
    xq = W.perturbed_lattice((12, 12, 12), 0.4, seed=4) + 1.5
    r = 2.0
    mn, mx = np.full(3, -1.0), np.full(3, 18.0)
    pre = _pre(P, 3, r, mn, mx, len(y))
    grid = make_nhs(P, 3, r, mn, mx, len(y))
    xd, yd = dcoords(xq), dcoords(y)
    P.initialize(pre, xd, yd)
    P.initialize(grid, xd, yd)
    assert all(torch.equal(a, b) for a, b in zip(P.neighbor_lists(xd, yd, pre),
                                                 P.neighbor_lists(xd, yd, grid)))
    # update! after moving both sets: the lists follow
    rng = np.random.default_rng(5)
    y2 = y + rng.normal(0, 0.05, y.shape)
    x2 = xq + rng.normal(0, 0.05, xq.shape)
    xd2, yd2 = dcoords(x2), dcoords(y2)
    P.update(pre, xd2, yd2)
    P.initialize(grid, xd2, yd2)
    lp, lg = P.neighbor_lists(xd2, yd2, pre), P.neighbor_lists(xd2, yd2, grid)
    assert torch.equal(lp[0], lg[0]) and torch.equal(lp[1], lg[1])
    g = O.grid_create(3, r, mn, mx)
    toff, tnb = O.trivial_lists(g, x2, y2)
    assert np.array_equal(lp[0].cpu().numpy(), toff) and np.array_equal(lp[1].cpu().numpy(), tnb)


def test_precomputed_wcsph_vs_oracle(P, O):
    W = P.workloads
    x, v, dx = W.wcsph_cloud(24, seed=9, dtype=np.float32)
    n = len(x)
    r = np.float32(3.0)
    lo, hi = np.full(3, -1.0), np.full(3, 25.0)
    pre = _pre(P, 3, r, lo, hi, n, dtype=np.float32,
               strategy=P.ParallelIncrementalUpdate())
    xd = dcoords(x)
    P.initialize(pre, xd, xd)
    rho = torch.zeros(n, device="cuda")
    prs = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd, accel=acc,
                                         **W.WCSPH), xd, xd, pre)
    g = O.grid_create(3, r, lo.astype(np.float32), hi.astype(np.float32), dtype=np.float32)
    cl = O.build(g, x)
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl, x, x, O.F_WCSPH_DENSITY, prm, want_abs=True)
    assert _rel_err(rho.cpu().numpy().astype(np.float64), orho, oab) < TOL_F32
    # force: the oracle sums the same inputs (the GPU's density and pressure) in FP64
    c = W.WCSPH
    prm2, keep2 = O.make_params(rho=rho.cpu().numpy().astype(np.float64),
                                pressure=prs.cpu().numpy().astype(np.float64),
                                vel=v.astype(np.float64),
                                r_min=float(np.sqrt(np.finfo(np.float32).eps)) * c["h"], **c)
    oacc, oabs = O.foreach(g, cl, x, x, O.F_WCSPH_FORCE, prm2, want_abs=True)
    got = acc.cpu().numpy().astype(np.float64).reshape(n, 3)
    assert _rel_err(got, oacc, oabs) < TOL_F32
    # an update! along the displacement keeps the lists equal to a fresh build
    x1 = (x + dx).astype(np.float32)
    x1d = dcoords(x1)
    P.update(pre, x1d, x1d)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), x1d, x1d, pre)
    g1 = O.build(g, x1)
    assert np.array_equal(cnt.cpu().numpy(), O.foreach(g, g1, x1, x1, O.F_COUNT))


def test_precomputed_errors(P):
    y = np.random.default_rng(1).uniform(0, 4, size=(400, 3))
    pre = _pre(P, 3, 1.0, np.zeros(3), np.full(3, 4.0), len(y), max_neighbors=8)
    yd = dcoords(y)
    with pytest.raises(P.PointNeighborsError, match="cell list is full"):
        P.initialize(pre, yd, yd)
    pre2 = _pre(P, 3, 1.0, np.zeros(3), np.full(3, 4.0), len(y))
    with pytest.raises(P.PointNeighborsError, match="inactive points"):
        P.initialize(pre2, yd, yd, eachindex_y=range(0, 10))
