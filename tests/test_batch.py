"""The batched form (BatchedNeighborhoodSearch over the pn_batch_* C ABI) against one
GridNeighborhoodSearch per cloud: bit-exact neighbour counts, and WCSPH density and
acceleration equal to the per-cloud results bit for bit (the same traversal per query, the
same candidate order); every tile schedule, the autotuner and the captured CUDA graph give
the same bits."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _clouds(P, n_clouds=24, seed=3):
    return P.workloads.batched_clouds(n_clouds=n_clouds, n_min=40, n_max=4000, seed=seed)


def _searches(P, clouds):
    out = []
    for c in clouds:
        r = np.float32(c["radius"])
        cl = P.FullGridCellList(min_corner=np.asarray(c["min_corner"], np.float32),
                                max_corner=np.asarray(c["max_corner"], np.float32),
                                search_radius=r, max_points_per_cell=0)
        out.append(P.GridNeighborhoodSearch(3, search_radius=r, n_points=len(c["x"]),
                                            cell_list=cl))
    return out


def _concat(clouds, key):
    return np.ascontiguousarray(np.concatenate([c[key] for c in clouds]))


def _wcsph(P, n, **kw):
    W = dict(P.workloads.WCSPH)
    W.update(kw)
    rho = torch.zeros(n, device="cuda")
    prs = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    return rho, prs, acc, W


def _per_cloud(P, clouds, searches, xs, vs):
    """Counts and the WCSPH step of every cloud through its own search."""
    n = sum(len(c["x"]) for c in clouds)
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    rho, prs, acc, W = _wcsph(P, n)
    off = 0
    for c, s in zip(clouds, searches):
        m = len(c["x"])
        x = xs[off:off + m].T
        v = vs[off:off + m].reshape(-1)
        P.initialize(s, x, x)
        P.foreach_point_neighbor(P.CountNeighbors(counts[off:off + m]), x, x, s)
        consts = dict(W, h=c["radius"] / 2)
        P.foreach_point_neighbor(P.WCSPHStep(density=rho[off:off + m], pressure=prs[off:off + m],
                                             velocity=v, accel=acc[3 * off:3 * (off + m)],
                                             **consts),
                                 x, x, s)
        off += m
    return counts, rho, acc


def _batched(P, clouds, batch, xs, vs):
    n = xs.shape[0]
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    batch.foreach_point_neighbor(P.CountNeighbors(counts), xs.T)
    rho, prs, acc, W = _wcsph(P, n)
    h = [c["radius"] / 2 for c in clouds]
    batch.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vs.reshape(-1),
                                             accel=acc, **dict(W, h=h)), xs.T)
    return counts, rho, acc


def test_batch_equals_per_cloud_searches(P):
    clouds = _clouds(P)
    searches = _searches(P, clouds)
    xs = torch.as_tensor(_concat(clouds, "x"), device="cuda")
    vs = torch.as_tensor(_concat(clouds, "v"), device="cuda")
    want = _per_cloud(P, clouds, searches, xs, vs)
    batch = P.BatchedNeighborhoodSearch(searches)
    batch.initialize(xs.T)
    got = _batched(P, clouds, batch, xs, vs)
    assert torch.equal(got[0], want[0])
    assert int(want[0].min()) >= 1
    assert torch.equal(got[1], want[1])
    assert torch.equal(got[2], want[2])
    # every tile schedule gives the same bits
    for block in (64, 128, 256):
        for order in (0, 1):
            for persistent in (0, 1):
                for ppt in (1, 2):
                    for fn in (P._lib.PN_F_COUNT, P._lib.PN_F_WCSPH_DENSITY,
                               P._lib.PN_F_WCSPH_FORCE):
                        batch.set_schedule(fn, block, order, persistent, ppt)
                    res = _batched(P, clouds, batch, xs, vs)
                    for a, b in zip(res, want):
                        assert torch.equal(a, b), (block, order, persistent, ppt)


def test_batch_update_autotune_and_graph(P, tmp_path):
    clouds = _clouds(P, n_clouds=40, seed=5)
    searches = _searches(P, clouds)
    x0 = torch.as_tensor(_concat(clouds, "x"), device="cuda")
    vs = torch.as_tensor(_concat(clouds, "v"), device="cuda")
    x1 = x0 + torch.as_tensor(_concat(clouds, "dx"), device="cuda")
    batch = P.BatchedNeighborhoodSearch(searches)
    batch.initialize(x0.T)
    batch.update(x1.T)
    want = _per_cloud(P, clouds, searches, x1, vs)
    n = x0.shape[0]
    rho, prs, acc, W = _wcsph(P, n)
    h = [c["radius"] / 2 for c in clouds]
    step = P.WCSPHStep(density=rho, pressure=prs, velocity=vs.reshape(-1), accel=acc,
                       **dict(W, h=h))
    cache = tmp_path / "schedules.txt"
    for f in (P.WCSPHDensity(density=rho, pressure=prs, velocity=vs.reshape(-1), **dict(W, h=h)),
              P.WCSPHForce(density=rho, pressure=prs, velocity=vs.reshape(-1), accel=acc,
                           reuse_state=True, **dict(W, h=h))):
        sched = batch.autotune(f, x1.T, reps=2, cache=cache)
        assert sched["block"] in (64, 128, 256) and sched["points_per_thread"] in (1, 2)
        # a second batch of the same kind takes the stored schedule untimed
        other = P.BatchedNeighborhoodSearch(searches)
        other.initialize(x1.T)
        other.set_schedule(f.functor, 64, 0, 0, 1)
        assert other.autotune(f, x1.T, reps=2, cache=cache) == sched
        assert batch.tune_key(f.functor) in cache.read_text()
    got = _batched(P, clouds, batch, x1, vs)
    assert torch.equal(got[1], want[1]) and torch.equal(got[2], want[2])
    # the captured graph: update!(xbuf) + density + force, replayed after xbuf moved
    xbuf = x0.clone()
    batch.capture_step(xbuf.T, step)
    rho.zero_()
    acc.zero_()
    xbuf.copy_(x1)
    batch.launch_step()
    batch.sync()
    assert torch.equal(rho, want[1]) and torch.equal(acc, want[2])


def test_batch_rejects_what_it_does_not_support(P):
    r = np.float32(2.0)
    cl = P.FullGridCellList(min_corner=np.zeros(3, np.float32), max_corner=np.full(3, 5.0, np.float32),
                            search_radius=r)
    ok = P.GridNeighborhoodSearch(3, search_radius=r, n_points=10, cell_list=cl)
    box = P.PeriodicBox(min_corner=np.zeros(3, np.float32), max_corner=np.full(3, 8.0, np.float32))
    cl8 = P.FullGridCellList(min_corner=np.zeros(3, np.float32), max_corner=np.full(3, 8.0, np.float32),
                             search_radius=r)
    per = P.GridNeighborhoodSearch(3, search_radius=r, n_points=10, cell_list=cl8, periodic_box=box)
    with pytest.raises(P.ArgumentError):
        P.BatchedNeighborhoodSearch([ok, per])
    cl64 = P.FullGridCellList(min_corner=np.zeros(3), max_corner=np.full(3, 5.0), search_radius=2.0)
    with pytest.raises(P.ArgumentError):
        P.BatchedNeighborhoodSearch([P.GridNeighborhoodSearch(3, search_radius=2.0, n_points=10,
                                                              cell_list=cl64)])
    # a point outside its cloud's domain: the reference's error
    batch = P.BatchedNeighborhoodSearch([ok, ok])
    x = torch.full((20, 3), 2.0, device="cuda")
    x[13, 0] = 50.0
    with pytest.raises(P.PointNeighborsError, match="outside the domain"):
        batch.initialize(x.T)


def test_batch_vs_oracle_64_clouds(P, O):
    """64 clouds of the batched workload's kind, each checked against the FP64 oracle of its
    own search (its corners, radius and h = radius / 2): counts bit-exact, density and
    acceleration within 1e-5 of the sum of |terms|."""
    from test_gpu_parity import TOL_F32, _rel_err
    clouds = P.workloads.batched_clouds(n_clouds=64, n_min=100, n_max=3000, seed=11)
    searches = _searches(P, clouds)
    xs = torch.as_tensor(_concat(clouds, "x"), device="cuda")
    vs = torch.as_tensor(_concat(clouds, "v"), device="cuda")
    batch = P.BatchedNeighborhoodSearch(searches)
    batch.initialize(xs.T)
    counts, rho, acc = _batched(P, clouds, batch, xs, vs)
    n = xs.shape[0]
    prs = torch.zeros(n, device="cuda")
    W = dict(P.workloads.WCSPH)
    h = [c["radius"] / 2 for c in clouds]
    batch.foreach_point_neighbor(P.WCSPHDensity(density=rho, pressure=prs,
                                                velocity=vs.reshape(-1), **dict(W, h=h)), xs.T)
    counts, rho_h, prs_h = counts.cpu().numpy(), rho.cpu().numpy(), prs.cpu().numpy()
    acc_h = acc.cpu().numpy().reshape(n, 3)
    off = 0
    for c in clouds:
        m = len(c["x"])
        x = np.asarray(c["x"], np.float32)
        v = np.asarray(c["v"], np.float64)
        r = np.float32(c["radius"])
        g = O.grid_create(3, r, np.asarray(c["min_corner"], np.float32),
                          np.asarray(c["max_corner"], np.float32), dtype=np.float32)
        cl = O.build(g, x)
        sl = slice(off, off + m)
        assert np.array_equal(counts[sl], O.foreach(g, cl, x, x, O.F_COUNT))
        consts = dict(W, h=c["radius"] / 2)
        prm, keep = O.make_params(**consts)
        orho, oab = O.foreach(g, cl, x, x, O.F_WCSPH_DENSITY, prm, want_abs=True)
        assert _rel_err(rho_h[sl].astype(np.float64), orho, oab) < TOL_F32
        prm, keep = O.make_params(rho=rho_h[sl].astype(np.float64),
                                  pressure=prs_h[sl].astype(np.float64), vel=v,
                                  r_min=float(np.sqrt(np.finfo(np.float32).eps)) * consts["h"],
                                  **consts)
        oacc, oab = O.foreach(g, cl, x, x, O.F_WCSPH_FORCE, prm, want_abs=True)
        assert _rel_err(acc_h[sl].astype(np.float64), oacc, oab) < TOL_F32
        off += m
