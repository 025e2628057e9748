"""Float64 WCSPH sweeps with double-float sums (3D, no periodic box): pos_diff from the
coordinates' three-part Float32 splits, d^2 and the pair arithmetic in double-float, the
neighbour test decided by the Float64 geometry inside a band of 1e-12 r^2 around r^2.

* neighbour sets: the pair cache recorded by the density sweep holds exactly the Float64
  neighbours; its counts (CountNeighbors walks the cache) equal the oracle's bit for bit,
  on a lattice of spacing r/2 where every axis-aligned pair at distance r has d^2 = r^2
  exactly (the band's case);
* sums: density and acceleration within 1e-12 of the FP64 oracle's sum of |terms|, for a
  cloud offset by 1e6 (pos_diff is then a small difference of large coordinates, exact
  only through the split), with and without the pair cache.
"""
import numpy as np
import pytest

from test_gpu_parity import TOL_F64, _rel_err, dcoords

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _search(P, n, lo, hi, r, cache):
    cl = P.FullGridCellList(min_corner=np.full(3, lo), max_corner=np.full(3, hi),
                            search_radius=r, max_points_per_cell=0)
    return P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl,
                                    pair_cache=cache)


def test_df64_cache_neighbours_at_the_radius(P, O):
    side, r, off = 18, 3.0, 1000.0
    x = P.workloads.lattice((side,) * 3, spacing=r / 2, origin=off, dtype=np.float64)
    n = len(x)
    lo, hi = off - 2.0, off + side * r / 2 + 2.0
    nhs = _search(P, n, lo, hi, r, True)
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    v = np.zeros((n, 3))
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    rho = torch.zeros(n, dtype=torch.float64, device="cuda")
    prs = torch.zeros(n, dtype=torch.float64, device="cuda")
    P.foreach_point_neighbor(P.WCSPHDensity(density=rho, pressure=prs, velocity=vd,
                                            **P.workloads.WCSPH), xd, xd, nhs)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, xd, nhs)  # walks the cache
    g = O.grid_create(3, r, np.full(3, lo), np.full(3, hi), dtype=np.float64)
    cl = O.build(g, x)
    ocnt = O.foreach(g, cl, x, x, O.F_COUNT)
    assert np.array_equal(cnt.cpu().numpy(), ocnt)
    # the pairs at exactly d = r are neighbours (d^2 <= r^2): 6 of them for an inner point
    inner = np.all((x > off + r) & (x < off + (side - 3) * r / 2), axis=1)
    assert inner.any() and np.all(ocnt[inner] == ocnt[inner][0])


@pytest.mark.parametrize("cache", [False, True])
def test_df64_wcsph_offset_cloud(P, O, cache):
    W = P.workloads
    x0, v, dx = W.wcsph_cloud(22, seed=9, dtype=np.float64)
    off = 1.0e6
    x = x0 + off
    n = len(x)
    lo, hi = off - 1.0, off + 23.0
    nhs = _search(P, n, lo, hi, 3.0, cache)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    rho = torch.zeros(n, dtype=torch.float64, device="cuda")
    prs = torch.zeros(n, dtype=torch.float64, device="cuda")
    acc = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    xd = dcoords(x)
    P.initialize(nhs, xd, xd)
    for _ in range(2):  # with the cache, the second step walks it
        P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd,
                                             accel=acc, **W.WCSPH), xd, xd, nhs)
    g = O.grid_create(3, 3.0, np.full(3, lo), np.full(3, hi), dtype=np.float64)
    cl = O.build(g, x)
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl, x, x, O.F_WCSPH_DENSITY, prm, want_abs=True)
    assert _rel_err(rho.cpu().numpy(), orho, oab) < TOL_F64
    prm, keep = O.make_params(rho=rho.cpu().numpy(), pressure=prs.cpu().numpy(), vel=v,
                              r_min=float(np.sqrt(np.finfo(np.float64).eps)) * W.WCSPH["h"],
                              **W.WCSPH)
    oacc, oab = O.foreach(g, cl, x, x, O.F_WCSPH_FORCE, prm, want_abs=True)
    assert _rel_err(acc.cpu().numpy().reshape(n, 3), oacc, oab) < TOL_F64
