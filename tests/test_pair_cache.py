"""The pair cache of the grid search (pn_set_pair_cache): a density sweep records, per
query and stencil row, which candidates are neighbours, and the following sweeps visit
exactly those.  Against the same search without the
cache: counts and neighbour lists bit-exact, the density bit-exact (the same sweep), the
force and the adjoint gradient within the FP32 tolerance of the tests (1e-5 of sum |terms|
for the force against the FP64 oracle; 1e-4 of max |dL/dx| for the gradient); rows that
do not fit the capacity, and update!, are covered."""
import numpy as np
import pytest
import torch

from test_gpu_parity import dcoords, _rel_err, TOL_F32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _nhs(P, n, side, cache, strategy=None, periodic=False):
    r = np.float32(3.0)
    lo = np.full(3, 0.0 if periodic else -1.0, np.float32)
    hi = np.full(3, side + (0.0 if periodic else 1.0), np.float32)
    box = P.PeriodicBox(min_corner=lo, max_corner=hi) if periodic else None
    cl = P.FullGridCellList(min_corner=lo, max_corner=hi, search_radius=r, max_points_per_cell=0)
    return P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl,
                                    update_strategy=strategy, pair_cache=cache, periodic_box=box)


def _step(P, nhs, x, v):
    W = P.workloads
    n = x.shape[1]
    rho = torch.zeros(n, device="cuda")
    prs = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    P.foreach_point_neighbor(P.WCSPHDensity(density=rho, pressure=prs, velocity=v, **W.WCSPH),
                             x, x, nhs)
    P.foreach_point_neighbor(P.WCSPHForce(density=rho, pressure=prs, velocity=v, accel=acc,
                                          reuse_state=True, **W.WCSPH), x, x, nhs)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), x, x, nhs)
    lists = P.neighbor_lists(x, x, nhs)
    return rho, prs, acc, cnt, lists


# rebuild_fraction 1: update! keeps overflow lists (positions moved in place, rows clipped
# by the sort keys widened by the largest move; the cache also holds each row's overflow
# run); periodic: queries near the faces fall back to the stencil
@pytest.mark.parametrize("fraction,periodic", [(0.01, False), (1.0, False), (0.01, True)])
def test_pair_cache_equals_stencil(P, O, fraction, periodic):
    W = P.workloads
    side = 22
    x, v, dx = W.wcsph_cloud(side, seed=4, dtype=np.float32)
    if periodic:
        x = x - np.float32(0.5)  # the lattice 0.5..21.5 inside the box [0, 22)
    n = len(x)
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    ref = _nhs(P, n, side, False, P.ParallelIncrementalUpdate(fraction), periodic)
    pc = _nhs(P, n, side, True, P.ParallelIncrementalUpdate(fraction), periodic)
    for k, pos in enumerate([x, (x + dx).astype(np.float32), (x - dx).astype(np.float32)]):
        xd = dcoords(pos)
        if k == 0:
            P.initialize(ref, xd, xd)
            P.initialize(pc, xd, xd)
        else:
            P.update(ref, xd, xd)
            P.update(pc, xd, xd)
        a = _step(P, ref, xd, vd)
        b = _step(P, pc, xd, vd)
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])  # density, pressure
        assert torch.equal(a[3], b[3])                             # counts
        assert torch.equal(a[4][0], b[4][0]) and torch.equal(a[4][1], b[4][1])
        # force from the cached lists against the FP64 oracle on the same inputs
        lo = np.full(3, 0.0 if periodic else -1.0, np.float32)
        hi = np.full(3, side + (0.0 if periodic else 1.0), np.float32)
        g = O.grid_create(3, np.float32(3.0), lo, hi, dtype=np.float32,
                          periodic_box=(lo, hi) if periodic else None)
        cl = O.build(g, pos)
        c = W.WCSPH
        prm, keep = O.make_params(rho=b[0].cpu().numpy().astype(np.float64),
                                  pressure=b[1].cpu().numpy().astype(np.float64),
                                  vel=v.astype(np.float64),
                                  r_min=float(np.sqrt(np.finfo(np.float32).eps)) * c["h"], **c)
        oacc, oab = O.foreach(g, cl, pos, pos, O.F_WCSPH_FORCE, prm, want_abs=True)
        got = b[2].cpu().numpy().reshape(n, 3).astype(np.float64)
        assert _rel_err(got, oacc, oab) < TOL_F32
        want = a[2].cpu().numpy().reshape(n, 3).astype(np.float64)
        assert _rel_err(want, oacc, oab) < TOL_F32


def test_pair_cache_adjoint(P):
    W = P.workloads
    side = 16
    x = W.perturbed_lattice((side,) * 3, 0.25, seed=6, dtype=np.float32)
    n = len(x)
    consts = dict(mass=1.0, h=1.5, cutoff=3.0, lambda_pot=0.01)
    out = []
    for cache in (False, True):
        nhs = _nhs(P, n, side, cache)
        xd = dcoords(x)
        P.initialize(nhs, xd, xd)
        rho = torch.empty(n, device="cuda")
        terms = torch.empty(n, device="cuda")
        loss = torch.empty(1, dtype=torch.float64, device="cuda")
        P.foreach_point_neighbor(P.AdjointLossForward(density=rho, terms=terms, loss=loss,
                                                      **consts), xd, xd, nhs)
        grad = torch.empty(3 * n, device="cuda")
        P.foreach_point_neighbor(P.AdjointLossBackward(grad=grad, reuse_state=True, **consts),
                                 xd, xd, nhs)
        out.append((rho, loss, grad))
    assert torch.equal(out[0][0], out[1][0])  # density: the same sweep
    # the loss terms may round differently (FMA contraction in the fused sweep)
    assert abs(float(out[0][1]) - float(out[1][1])) <= 1e-6 * abs(float(out[0][1]))
    g0, g1 = out[0][2], out[1][2]
    assert float((g0 - g1).abs().max() / g0.abs().max()) < 1e-4


@pytest.mark.parametrize("d", [2, 3])
def test_keyed_clipping_with_overflow_lists(P, O, d):
    """Float32 searches that keep overflow lists (rebuild_fraction 1) over a random walk
    with large steps: the main slots move in place and the rows are clipped by the sort keys
    widened by their cells' largest move; the pair cache records each row's main and overflow
    runs.  After every update!: neighbour lists equal a fresh ParallelUpdate build, the
    counts over the pair cache equal the oracle's, and the density equals the same search's
    density without the cache bit for bit."""
    side = 26 if d == 2 else 16
    x0 = P.workloads.perturbed_lattice((side,) * d, 0.25, seed=7 + d, dtype=np.float32)
    n = len(x0)
    r = np.float32(3.0)
    lo, hi = np.full(d, -4.0, np.float32), np.full(d, side + 4.0, np.float32)

    def search(strategy, cache):
        cl = P.FullGridCellList(min_corner=lo, max_corner=hi, search_radius=r,
                                max_points_per_cell=0)
        return P.GridNeighborhoodSearch(d, search_radius=r, n_points=n, cell_list=cl,
                                        update_strategy=strategy, pair_cache=cache)

    inc = search(P.ParallelIncrementalUpdate(1.0), 1)
    inc_nc = search(P.ParallelIncrementalUpdate(1.0), 0)
    fresh = search(P.ParallelUpdate(), 0)
    xd = dcoords(x0)
    P.initialize(inc, xd, xd)
    P.initialize(inc_nc, xd, xd)
    rng = np.random.default_rng(20 + d)
    xs = x0.astype(np.float64)
    W = P.workloads
    consts = dict(W.WCSPH)
    for _ in range(4):
        xs = np.clip(xs + rng.normal(0.0, 0.4, xs.shape), 0.0, side)
        x = xs.astype(np.float32)
        xd = dcoords(x)
        P.update(inc, xd, xd)
        P.update(inc_nc, xd, xd)
        P.initialize(fresh, xd, xd)
        rho = [torch.zeros(n, device="cuda") for _ in range(2)]
        prs = [torch.zeros(n, device="cuda") for _ in range(2)]
        for k, nhs in enumerate((inc, inc_nc)):
            P.foreach_point_neighbor(P.WCSPHDensity(density=rho[k], pressure=prs[k], **consts),
                                     xd, xd, nhs)
        assert torch.equal(rho[0], rho[1])
        cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
        P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, xd, inc)  # walks the cache
        g = O.grid_create(d, r, lo, hi, dtype=np.float32)
        ocnt = O.foreach(g, O.build(g, x), x, x, O.F_COUNT)
        assert np.array_equal(cnt.cpu().numpy(), ocnt)
        oi, ni = P.neighbor_lists(xd, xd, inc)
        of, nf = P.neighbor_lists(xd, xd, fresh)
        assert torch.equal(oi, of) and torch.equal(ni, nf)
    assert inc.grid_info()["n_overflow"] > 0  # the overflow lists were in use
