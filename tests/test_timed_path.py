"""The benchmark's timed step at full size, checked against the FP64 oracle.

bench.py times, per step: update! of a ParallelIncrementalUpdate search (the points follow
a random walk, N(0, 0.05^2) per component per step), the WCSPH density sweep that also
records the pair cache, and the force sweep over the cache's hit masks.  This runs that
step sequence on the 200^3 = 8,000,000-point FP32 lattice and compares a sample of 20,000
query points with the oracle, which bins all 8M points: neighbour counts bit-exact (counted
over the same pair cache), density and acceleration within 1e-5 of the sum of |terms|.
With rebuild_fraction 0.01 every update! rebuilds (about 8 % of the points change cell per
step); with 1.0 it keeps overflow lists: the rows are clipped by the sort keys widened by
the largest in-place move, and the cache also holds each row's overflow run.
"""
import numpy as np
import pytest

from test_gpu_parity import TOL_F32, _rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


@pytest.mark.parametrize("fraction", [0.01, 1.0])
def test_timed_step_8m_vs_oracle(P, O, fraction):
    W = P.workloads
    x0, v, dx = W.wcsph_cloud(200, seed=1, dtype=np.float32)
    n = len(x0)
    T = np.float32
    cl = P.FullGridCellList(min_corner=np.full(3, -1.0, T), max_corner=np.full(3, 201.0, T),
                            search_radius=T(3.0), max_points_per_cell=0)
    nhs = P.GridNeighborhoodSearch(3, search_radius=T(3.0), n_points=n, cell_list=cl,
                                   update_strategy=P.ParallelIncrementalUpdate(fraction),
                                   pair_cache=1)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    rho = torch.zeros(n, device="cuda")
    prs = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    dens = P.WCSPHDensity(density=rho, pressure=prs, velocity=vd, **W.WCSPH)
    force = P.WCSPHForce(density=rho, pressure=prs, velocity=vd, accel=acc, reuse_state=True,
                         **W.WCSPH)
    x0d = torch.as_tensor(x0, device="cuda")
    P.initialize(nhs, x0d.T, x0d.T)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    xs = torch.as_tensor((x0.astype(np.float64) + dx).astype(np.float32), device="cuda")
    for step in range(6):
        if step:
            xs = xs + np.float32(0.05) * torch.randn(xs.shape, generator=gen, device="cuda")
        P.update(nhs, xs.T, xs.T)
        P.foreach_point_neighbor(dens, xs.T, xs.T, nhs)
        P.foreach_point_neighbor(force, xs.T, xs.T, nhs)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xs.T, xs.T, nhs)  # over the cache
    x = xs.cpu().numpy()
    g = O.grid_create(3, np.float32(3.0), np.full(3, -1.0, np.float32),
                      np.full(3, 201.0, np.float32), dtype=np.float32)
    cl = O.build(g, x)
    sample = np.random.default_rng(3).choice(n, 20000, replace=False).astype(np.int32)
    ocnt = O.foreach(g, cl, x, x, O.F_COUNT, points=sample)
    assert np.array_equal(cnt.cpu().numpy()[sample], ocnt[sample])
    prm, keep = O.make_params(**W.WCSPH)
    orho, oab = O.foreach(g, cl, x, x, O.F_WCSPH_DENSITY, prm, points=sample, want_abs=True)
    rho_h = rho.cpu().numpy().astype(np.float64)
    assert _rel_err(rho_h[sample], orho[sample], oab[sample]) < TOL_F32
    # the force of the sample from the GPU's density and pressure of every point
    prm, keep = O.make_params(rho=rho_h, pressure=prs.cpu().numpy().astype(np.float64),
                              vel=v.astype(np.float64),
                              r_min=float(np.sqrt(np.finfo(np.float32).eps)) * 1.5, **W.WCSPH)
    oacc, oab = O.foreach(g, cl, x, x, O.F_WCSPH_FORCE, prm, points=sample, want_abs=True)
    a = acc.cpu().numpy().reshape(n, 3).astype(np.float64)
    assert _rel_err(a[sample], oacc[sample], oab[sample]) < TOL_F32
