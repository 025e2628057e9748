"""Cases run by test_bounds_check.py in a child process, once with the normal library and
once with the bounds-checked one (PN_GB300_LIB names which): the parity suite's 2D and 3D
clouds through the build, the incremental update, every traversal form and the batched
form.  Writes every output and each search's status to the .npz named on the command line.

Usage: python tests/bounds_check_cases.py OUT.npz
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import torch  # noqa: E402

import __graft_entry__  # noqa: E402

P = __graft_entry__.package()
L = P._lib
W = P.workloads
out = {}
status = []


def dc(x):
    return torch.as_tensor(np.ascontiguousarray(x), device="cuda").T


def record(name, nhs):
    torch.cuda.synchronize()
    site, index = L.C.c_int32(0), L.C.c_int32(0)
    assert L.load().pn_bounds_failure(nhs.handle, L.C.byref(site), L.C.byref(index)) == 0
    status.append((name, L.load().pn_get_error(nhs.handle, 0), site.value, index.value))


def grid(d, r, mn, mx, n, T, box=None, strategy=None, cache=0, max_ppc=0):
    cl = P.FullGridCellList(min_corner=np.asarray(mn, T), max_corner=np.asarray(mx, T),
                            search_radius=T(r), max_points_per_cell=max_ppc)
    pb = None if box is None else P.PeriodicBox(min_corner=np.asarray(box[0], T),
                                                max_corner=np.asarray(box[1], T))
    return P.GridNeighborhoodSearch(d, search_radius=T(r), n_points=n, cell_list=cl,
                                    periodic_box=pb, update_strategy=strategy,
                                    pair_cache=cache)


def lists_and_counts(name, nhs, xd):
    off, nb = P.neighbor_lists(xd, xd, nhs)
    cnt = torch.zeros(xd.shape[1], dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, xd, nhs)
    out[name + "/off"], out[name + "/nb"] = off.cpu().numpy(), nb.cpu().numpy()
    out[name + "/count"] = cnt.cpu().numpy()


def wcsph(name, nhs, xd, v, T, steps=2):
    n = xd.shape[1]
    td = torch.float32 if T == np.float32 else torch.float64
    vd = torch.as_tensor(v.astype(T), device="cuda").reshape(-1)
    rho = torch.zeros(n, dtype=td, device="cuda")
    prs = torch.zeros(n, dtype=td, device="cuda")
    acc = torch.zeros(3 * n, dtype=td, device="cuda")
    for _ in range(steps):  # with a pair cache the second step walks it
        P.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vd, accel=acc,
                                             **W.WCSPH), xd, xd, nhs)
    out[name + "/rho"], out[name + "/acc"] = rho.cpu().numpy(), acc.cpu().numpy()


# 2D Float32 perturbed lattice, plain grid
x = W.perturbed_lattice((70, 70), 0.25, seed=2, dtype=np.float32)
nhs = grid(2, 1.7, [-1, -1], [72, 72], len(x), np.float32)
xd = dc(x)
P.initialize(nhs, xd, xd)
lists_and_counts("2d_f32", nhs, xd)
m = torch.ones(len(x), device="cuda")
a = torch.zeros(2 * len(x), device="cuda")
P.foreach_point_neighbor(P.NBodyAcceleration(m, 1.0, a), xd, xd, nhs)
out["2d_f32/nbody"] = a.cpu().numpy()
record("2d_f32", nhs)

# 2D Float64 periodic box
x = W.perturbed_lattice((48, 48), 0.3, origin=0.5, seed=3, dtype=np.float64)
nhs = grid(2, 2.0, [0, 0], [48, 48], len(x), np.float64, box=([0, 0], [48, 48]))
xd = dc(x)
P.initialize(nhs, xd, xd)
lists_and_counts("2d_f64_periodic", nhs, xd)
record("2d_f64_periodic", nhs)

# 3D WCSPH cloud: Float32 with the pair cache, Float64 (Float32 traversal, Float64 test)
x, v, dx = W.wcsph_cloud(22, seed=4, dtype=np.float32)
for T, tag in ((np.float32, "3d_f32_cache"), (np.float64, "3d_f64")):
    xt = x.astype(T)
    nhs = grid(3, 3.0, [-1] * 3, [23] * 3, len(x), T, cache=1 if T == np.float32 else 0)
    xd = dc(xt)
    P.initialize(nhs, xd, xd)
    xd = dc((xt.astype(np.float64) + dx).astype(T))
    P.update(nhs, xd, xd)
    lists_and_counts(tag, nhs, xd)
    wcsph(tag, nhs, xd, v, T)
    record(tag, nhs)

# 3D periodic box, Float32
xp = (x - np.float32(0.5)).astype(np.float32)
nhs = grid(3, 3.0, [0] * 3, [22] * 3, len(xp), np.float32, box=([0] * 3, [22] * 3))
xd = dc(xp)
P.initialize(nhs, xd, xd)
lists_and_counts("3d_f32_periodic", nhs, xd)
record("3d_f32_periodic", nhs)

# incremental update! that keeps overflow lists (fraction 1: never a rebuild)
nhs = grid(3, 3.0, [-1] * 3, [23] * 3, len(x), np.float32,
           strategy=P.ParallelIncrementalUpdate(1.0), cache=1)
xd = dc(x)
P.initialize(nhs, xd, xd)
rng = np.random.default_rng(5)
xs = x.astype(np.float64)
for k in range(3):
    xs = np.clip(xs + rng.normal(0.0, 0.3, xs.shape), -0.5, 22.5)
    xd = dc(xs.astype(np.float32))
    P.update(nhs, xd, xd)
out["incremental/n_overflow"] = np.array([nhs.grid_info()["n_overflow"]])
lists_and_counts("incremental", nhs, xd)
wcsph("incremental", nhs, xd, v, np.float32)
record("incremental", nhs)

# SpatialHashingCellList, hash-list layout (list_size below the occupied cells)
cl = P.SpatialHashingCellList(3, list_size=97, max_points_per_cell=0)
nhs = P.GridNeighborhoodSearch(3, search_radius=np.float32(3.0), n_points=len(x), cell_list=cl)
xd = dc(x)
P.initialize(nhs, xd, xd)
lists_and_counts("hash_lists", nhs, xd)
record("hash_lists", nhs)

# batched form: 12 clouds, counts and the WCSPH step
clouds = W.batched_clouds(n_clouds=12, n_min=40, n_max=3000, seed=3)
searches = []
for c in clouds:
    r = np.float32(c["radius"])
    cl = P.FullGridCellList(min_corner=np.asarray(c["min_corner"], np.float32),
                            max_corner=np.asarray(c["max_corner"], np.float32),
                            search_radius=r, max_points_per_cell=0)
    searches.append(P.GridNeighborhoodSearch(3, search_radius=r, n_points=len(c["x"]),
                                             cell_list=cl))
batch = P.BatchedNeighborhoodSearch(searches)
xs = torch.as_tensor(np.concatenate([c["x"] for c in clouds]), device="cuda")
vs = torch.as_tensor(np.concatenate([c["v"] for c in clouds]), device="cuda")
batch.initialize(xs.T)
n = xs.shape[0]
cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
batch.foreach_point_neighbor(P.CountNeighbors(cnt), xs.T)
rho = torch.zeros(n, device="cuda")
prs = torch.zeros(n, device="cuda")
acc = torch.zeros(3 * n, device="cuda")
batch.foreach_point_neighbor(P.WCSPHStep(density=rho, pressure=prs, velocity=vs.reshape(-1),
                                         accel=acc,
                                         **dict(W.WCSPH, h=[c["radius"] / 2 for c in clouds])),
                             xs.T)
torch.cuda.synchronize()
out["batch/count"], out["batch/rho"] = cnt.cpu().numpy(), rho.cpu().numpy()
out["batch/acc"] = acc.cpu().numpy()
berr = L.load().pn_batch_sync(batch._h)
status.append(("batch", berr, 0, 0))

out["build_flags"] = np.array([L.load().pn_build_flags()])
out["status"] = np.array([s[1:] for s in status], dtype=np.int64)
out["status_names"] = np.array([s[0] for s in status])
np.savez(sys.argv[1], **out)
