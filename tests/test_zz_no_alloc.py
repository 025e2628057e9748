"""pn_count_neighbors_noalloc (the entry point that allocates no device memory) against the
handle-based entry points, through the C ABI.

The no-allocation call must give, call after call, the counts that pn_initialize followed by
pn_foreach_point_neighbor(PN_F_COUNT) give for the same points and geometry: bit-exact, like
every integer result of this library.  Its scratch is shared by all calls and keeps the last
call's contents, so the calls below run back to back on different clouds and geometries.
This file is named to run last, and also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(pkg):
    pkg.build.build()


def _config(L, ndims, dtype, r, lo, hi, periodic=False, max_ppc=0):
    cfg = L.pn_config()
    cfg.ndims = ndims
    cfg.dtype = L.PN_FLOAT32 if dtype == np.float32 else L.PN_FLOAT64
    cfg.search_radius = float(dtype(r))
    for k in range(ndims):
        cfg.min_corner[k] = float(dtype(lo[k]))
        cfg.max_corner[k] = float(dtype(hi[k]))
        if periodic:
            cfg.periodic_min[k] = float(dtype(lo[k]))
            cfg.periodic_max[k] = float(dtype(hi[k]))
    cfg.periodic = 1 if periodic else 0
    cfg.update_strategy = L.PN_PARALLEL_UPDATE
    cfg.max_points_per_cell = max_ppc
    return cfg


def _counts_with_handle(L, cfg, xd, n, stream):
    """Counts through the handle-based entry points (pn_create allocates)."""
    import torch
    lib = L.load()
    h = C.c_void_p()
    assert lib.pn_create(C.byref(cfg), C.byref(h)) == 0
    try:
        assert lib.pn_initialize(h, C.c_void_p(xd.data_ptr()), n, None, 0, stream) == 0
        out = torch.zeros(n, dtype=torch.int32, device="cuda")
        prm = L.pn_count_params(C.c_void_p(out.data_ptr()))
        assert lib.pn_foreach_point_neighbor(h, L.PN_F_COUNT, C.c_void_p(xd.data_ptr()), n,
                                             C.c_void_p(xd.data_ptr()), n, None, 0,
                                             C.byref(prm), stream) == 0
        assert lib.pn_sync(h) == 0
    finally:
        lib.pn_destroy(h)
    return out.cpu().numpy()


def _counts_noalloc(L, cfg, xd, n, stream, fill=-7):
    import torch
    out = torch.full((max(n, 1),), fill, dtype=torch.int32, device="cuda")
    rc = L.load().pn_count_neighbors_noalloc(C.byref(cfg), C.c_void_p(xd.data_ptr()), n,
                                             C.c_void_p(out.data_ptr()), stream)
    return rc, out[:n].cpu().numpy()


def _cases(pkg):
    W = pkg.workloads
    x3 = W.perturbed_lattice((30, 30, 30), 0.25, seed=3, dtype=np.float32)      # 27,000
    x2 = W.periodic_nbody_cloud(256, seed=4, dtype=np.float64)[0]              # 65,536
    x3b = W.perturbed_lattice((20, 25, 18), 0.4, seed=5, dtype=np.float64)     # 9,000
    x1 = W.perturbed_lattice((40000,), 0.04, 0.1, 0.0, seed=6, dtype=np.float64)  # 40,000
    x3p = np.mod(W.perturbed_lattice((24, 24, 24), 0.3, seed=7, dtype=np.float64) - 0.5,
                 24.0).astype(np.float32)                                      # 13,824
    return [
        ("3D FP32 r=3", x3, 3, np.float32, 3.0, [-1.0] * 3, [32.0] * 3, False),
        ("2D FP64 periodic r=2.5", x2, 2, np.float64, 2.5, [0.0, 0.0], [256.0, 256.0], True),
        ("3D FP64 r=1.7", x3b, 3, np.float64, 1.7, [0.0] * 3, [27.0] * 3, False),
        ("1D FP64 r=1.3", x1, 1, np.float64, 1.3, [-1.0], [4001.0], False),
        ("3D FP32 periodic r=2", x3p, 3, np.float32, 2.0, [0.0] * 3, [24.0] * 3, True),
    ]


def test_noalloc_counts_equal_the_handle_entry_points(pkg, O):
    import torch
    L = pkg._lib
    L.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = _cases(pkg)
    # two calls in a row on different clouds, then the first again: each call must clear
    # what the previous one left in the shared scratch
    for name, x, d, dt, r, lo, hi, per in cases + cases[:1]:
        n = len(x)
        cfg = _config(L, d, dt, r, lo, hi, periodic=per)
        xd = torch.as_tensor(np.ascontiguousarray(x, dtype=dt), device="cuda")
        want = _counts_with_handle(L, cfg, xd, n, stream)
        rc, got = _counts_noalloc(L, cfg, xd, n, stream)
        assert rc == 0, (name, L.status_string(rc))
        assert np.array_equal(got, want), name
        assert want.min() >= 1, name  # the point itself is always counted
        # and both equal the oracle's restatement of the reference's grid search
        lo_t, hi_t = np.asarray(lo, dt), np.asarray(hi, dt)
        g = O.grid_create(d, dt(r), lo_t, hi_t, periodic_box=(lo_t, hi_t) if per else None,
                          dtype=dt)
        xa = np.ascontiguousarray(x, dtype=dt)
        assert np.array_equal(got, O.foreach(g, O.build(g, xa), xa, xa, O.F_COUNT)), name


def test_noalloc_repeated_calls_allocate_nothing(pkg):
    import torch
    L = pkg._lib
    L.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    name, x, d, dt, r, lo, hi, per = _cases(pkg)[0]
    n = len(x)
    cfg = _config(L, d, dt, r, lo, hi, periodic=per)
    xd = torch.as_tensor(x, device="cuda")
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    lib = L.load()
    assert lib.pn_count_neighbors_noalloc(C.byref(cfg), C.c_void_p(xd.data_ptr()), n,
                                          C.c_void_p(out.data_ptr()), stream) == 0
    first = out.cpu().numpy().copy()
    out.zero_()  # the loop's own torch calls, once before the measurement
    assert np.array_equal(first, first + out.cpu().numpy())
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        out.zero_()
        assert lib.pn_count_neighbors_noalloc(C.byref(cfg), C.c_void_p(xd.data_ptr()), n,
                                              C.c_void_p(out.data_ptr()), stream) == 0
        assert np.array_equal(out.cpu().numpy(), first)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_errors(pkg):
    import torch
    L = pkg._lib
    lib = L.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # beyond the scratch: 4 B per cell + 12 B per point + 20 B > 4 MiB -> rejected, untouched
    x = pkg.workloads.perturbed_lattice((70, 70, 70), 0.25, seed=1, dtype=np.float32)
    cfg = _config(L, 3, np.float32, 1.0, [-1.0] * 3, [72.0] * 3)
    xd = torch.as_tensor(x, device="cuda")
    rc, got = _counts_noalloc(L, cfg, xd, len(x), stream)
    assert rc == L.PN_ERR_SCRATCH_LIMIT
    assert "fixed scratch" in L.status_string(rc)
    assert (got == -7).all()
    # a point outside the domain: the reference's error, reported by the call itself
    x = pkg.workloads.perturbed_lattice((10, 10, 10), 0.25, seed=2, dtype=np.float64)
    x[17] = [100.0, 2.0, 2.0]
    cfg = _config(L, 3, np.float64, 2.0, [0.0] * 3, [12.0] * 3)
    rc, _ = _counts_noalloc(L, cfg, torch.as_tensor(x, device="cuda"), len(x), stream)
    assert rc == L.PN_ERR_OUT_OF_DOMAIN
    # a full cell, when max_points_per_cell is set
    x = np.full((50, 2), 5.5)
    cfg = _config(L, 2, np.float64, 1.0, [0.0, 0.0], [10.0, 10.0], max_ppc=10)
    rc, _ = _counts_noalloc(L, cfg, torch.as_tensor(x, device="cuda"), len(x), stream)
    assert rc == L.PN_ERR_CELL_FULL
    # and the next call, within limits, is correct again
    cfg = _config(L, 2, np.float64, 1.0, [0.0, 0.0], [10.0, 10.0])
    rc, got = _counts_noalloc(L, cfg, torch.as_tensor(x, device="cuda"), len(x), stream)
    assert rc == 0 and (got == 50).all()
    # empty input
    rc, _ = _counts_noalloc(L, cfg, torch.as_tensor(x, device="cuda"), 0, stream)
    assert rc == 0
