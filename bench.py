#!/usr/bin/env python
"""Benchmark: WCSPH pair-evaluations/s and update! ms on one GB300.

Workload (the default): a 200^3 = 8,000,000-point 3D lattice, spacing 1, uniform noise in
[-0.25, 0.25], Float32, search radius 3, FullGridCellList over [-1, 201]^3, velocities
N(0, 0.1^2).  A step is the hot path once over the whole cloud:
  update!(positions of a random walk, N(0, 0.05^2) per component per step)
                                                 (ParallelIncrementalUpdate)
  WCSPH density sweep (Wendland C2, h = 1.5) + Tait EOS
  WCSPH force sweep (pressure + Monaghan viscosity)
pair-evals/s = 2 sweeps x (ordered pairs with d^2 <= r^2, self included) per step / time.
`value` is device time with the inputs resident in HBM; `e2e` is the same step through the
C ABI with the coordinates and velocities copied from pinned host memory and the density
and acceleration copied back inside the timed region (double-buffered on two copy streams;
`e2e.h2d_ms`, `compute_ms` and `d2h_ms` are each phase's median duration per step, measured
with events on its own stream, and `*_max` the slowest step's).

`--impl reference` times the CPU restatement of the reference's algorithm (the oracle:
threaded cell-list build + per-point traversal, pair math in FP64) on the host cores, on a
bounded sample of query points of the same workload.

Multi-GPU (`--gpus N` under torchrun): independent replicas, one per GPU (the search does
not exchange data between GPUs); the time is the max over ranks and the value sums all
ranks' pairs.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
METRIC = "WCSPH pair-evals/s (8M pts, FP32, r=3, density+force+incremental update!)"
UNIT = "pair-evals/s"
# Algorithmic bytes per point of one force sweep (FP32): read x 12, v 12, rho 4, the
# point's index 4, write the acceleration 12.
FORCE_BYTES_PER_POINT = {"float32": 44, "float64": 84, "mixed": 56}
# DRAM bytes per point of one force sweep measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum, 4,096,000-point capture of the same workload): over the pair cache
# (the default) most of it is the cache's hit masks; without the cache (stencil) it is
# 49.1 B/point.  The ncu summaries are profiles/density_masks_force_masks_wcsph_4M.md and
# profiles/trav_force_density_wcsph_4M.md.
FORCE_TRAFFIC_BYTES_PER_POINT = {("float32", True): 227.8, ("float32", False): 49.1}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-side", type=int, default=200, help="lattice points per dimension")
    ap.add_argument("--dtype", default="float32", choices=["float32", "float64", "mixed"],
                    help="mixed: Float64 coordinates with a Float32 search radius (Float32 "
                         "pair arithmetic and arrays), the wcsph workload only")
    ap.add_argument("--cpu-sample", type=int, default=400_000,
                    help="query points in the CPU baseline sample")
    ap.add_argument("--pair-cache", type=int, default=1,
                    help="1: the grid search's pair cache (the density sweep records each "
                         "query's neighbours for the force sweep); 0: off")
    ap.add_argument("--cell-list", default="full_grid", choices=["full_grid", "spatial_hashing"],
                    help="wcsph workload: FullGridCellList [-1, n_side+1]^3 (incremental "
                         "update, pair cache) or SpatialHashingCellList(list_size = 2n) "
                         "(ParallelUpdate rebuild, no pair cache)")
    ap.add_argument("--list-size", type=int, default=0,
                    help="SpatialHashingCellList lists (default 2n); fewer lists than the "
                         "occupied cells' box has cells select the hash-list layout")
    ap.add_argument("--clouds", type=int, default=512,
                    help="batched workload: number of clouds")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="wcsph workload: leave out the batched, adjoint, Float64 and "
                         "update-path records that the default line carries")
    ap.add_argument("--rebuild-fraction", type=float, default=0.01,
                    help="ParallelIncrementalUpdate's rebuild fraction (1.0: update! keeps "
                         "overflow lists instead of rebuilding)")
    ap.add_argument("--workload", default="wcsph",
                    choices=["wcsph", "nbody2d", "count", "adjoint", "batched",
                             "precomputed"],
                    help="wcsph: the 3D WCSPH step (headline); nbody2d: 2D periodic "
                         "truncated potential on a 4096^2 lattice; count: neighbour counts "
                         "of the 50^3 Float64 lattice; adjoint: loss + dL/dx on the "
                         "100^3 lattice (backward/forward ratio); batched: 512 clouds, "
                         "one CUDA-graph step vs per-cloud launches; precomputed: the "
                         "WCSPH step with PrecomputedNeighborhoodSearch lists")
    return ap.parse_args()


# ------------------------------------------------------------------ distributed

def dist_setup(backend: str):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return rank, world, local


def aggregate(local_seconds: float, local_pairs: float, world: int, device=None):
    """Max of the timed region over ranks, sum of the evaluated pairs."""
    if world == 1:
        return local_seconds, local_pairs
    import torch
    import torch.distributed as dist
    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    p = torch.tensor([local_pairs], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t.item()), float(p.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------ clocks

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(prefix="pn_clocks_", suffix=".csv")
        self.proc = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={CLOCK_FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# Float32 operations of one WCSPH force pair evaluation (pos_diff and d2 8, r_min test 1,
# sqrt and q 3, the kernel's t, t^3 and gradient factor 6, v.x 9, mu 4, viscosity 5, the
# pair's factor 4, the accumulation 6); an FMA counts as two.
FORCE_FLOPS_PER_PAIR = 44


def fp32_peak(P):
    """The GPU's Float32 FMA issue peak in TFLOP/s: best of five timed launches of the
    library's FMA probe (8 independent FMA chains per thread, one wave of 152 x 8 blocks)."""
    import torch
    out = torch.empty(P._lib.PN_FMA_PROBE_THREADS, dtype=torch.float32, device="cuda")
    iters = 16384
    flops = 2.0 * 8 * iters * P._lib.PN_FMA_PROBE_THREADS
    st = P._stream()
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if P.lib().pn_fma_probe(out.data_ptr(), iters, st) != 0:
            raise RuntimeError("pn_fma_probe failed")
        e1.record()
        torch.cuda.synchronize()
        best = max(best, flops / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


# ------------------------------------------------------------------ GPU arm

def run_gpu(args, rank, world, local):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    P = __graft_entry__.package()
    W = P.workloads
    torch.cuda.set_device(local)
    # coordinates in dt, pair arithmetic and per-point arrays in vdt (Float32 for "mixed")
    dt = np.float32 if args.dtype == "float32" else np.float64
    vdt = np.float64 if args.dtype == "float64" else np.float32
    tcd = torch.float32 if dt == np.float32 else torch.float64
    tdt = torch.float32 if vdt == np.float32 else torch.float64
    n_side = args.n_side
    x0, v, dx = W.wcsph_cloud(n_side, seed=1, dtype=dt)
    v = v.astype(vdt)
    x1 = (x0.astype(np.float64) + dx).astype(dt)
    n = len(x0)
    r = vdt(3.0)
    hashing = args.cell_list == "spatial_hashing"
    if hashing:
        # the occupied cells fit 2n lists: the dense layout, which takes the pair cache
        cl = P.SpatialHashingCellList(3, list_size=args.list_size or 2 * n,
                                      max_points_per_cell=0)
        nhs = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl,
                                       update_strategy=P.ParallelUpdate(),
                                       pair_cache=args.pair_cache)
    else:
        cl = P.FullGridCellList(min_corner=np.full(3, -1.0, dt),
                                max_corner=np.full(3, n_side + 1.0, dt),
                                search_radius=r, max_points_per_cell=0)
        nhs = P.GridNeighborhoodSearch(
            3, search_radius=r, n_points=n, cell_list=cl,
            update_strategy=P.ParallelIncrementalUpdate(args.rebuild_fraction),
            pair_cache=args.pair_cache)
    x0d = torch.as_tensor(x0, device="cuda").T
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    rho = torch.zeros(n, dtype=tdt, device="cuda")
    prs = torch.zeros(n, dtype=tdt, device="cuda")
    acc = torch.zeros(3 * n, dtype=tdt, device="cuda")
    dens = P.WCSPHDensity(density=rho, pressure=prs, velocity=vd, **W.WCSPH)
    force = P.WCSPHForce(density=rho, pressure=prs, velocity=vd, accel=acc, reuse_state=True,
                         **W.WCSPH)
    # positions of every step: a random walk x_{s+1} = x_s + N(0, 0.05^2) per component
    # (x_0 = the displaced lattice), so every update! re-bins the points that really moved
    K, Wm = args.steps, args.warmup
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    walk = [torch.as_tensor(x1, device="cuda")]
    for _ in range(Wm + K - 1):
        walk.append(walk[-1] + dt(0.05) * torch.randn(walk[-1].shape, generator=gen,
                                                      device="cuda", dtype=tcd))
    # ordered pairs (self included) at every step's positions, with a separate search
    cl2 = P.FullGridCellList(min_corner=np.full(3, -1.0, dt), max_corner=np.full(3, n_side + 1.0, dt),
                             search_radius=r, max_points_per_cell=0)
    nhs_count = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl2)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    pairs = []
    for xs in walk:
        P.initialize(nhs_count, xs.T, xs.T)
        P.foreach_point_neighbor(P.CountNeighbors(cnt), xs.T, xs.T, nhs_count)
        pairs.append(int(cnt.to(torch.int64).sum()))
    del cnt, nhs_count
    pairs_timed = sum(pairs[Wm:])

    P.initialize(nhs, x0d, x0d)
    for s_ in range(Wm):
        xs = walk[s_].T
        P.update(nhs, xs, xs, check=False)
        P.foreach_point_neighbor(dens, xs, xs, nhs, check=False)
        P.foreach_point_neighbor(force, xs, xs, nhs, check=False)
    torch.cuda.synchronize()
    if P.lib().pn_sync(nhs.handle) != 0:
        raise RuntimeError("warm-up reported an error")

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(K)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    launches0 = P.lib().pn_launch_count()
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    t0.record()
    for k in range(K):
        e = ev[k]
        xs = walk[Wm + k].T
        e[0].record()
        P.update(nhs, xs, xs, check=False)
        e[1].record()
        P.foreach_point_neighbor(dens, xs, xs, nhs, check=False)
        e[2].record()
        P.foreach_point_neighbor(force, xs, xs, nhs, check=False)
        e[3].record()
    t1.record()
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - wall0
    launches = P.lib().pn_launch_count() - launches0
    clocks = sampler.stop() if sampler else None
    # which of update!'s two paths the timed steps took: the device rebuilds when the points
    # that left their cell of the last full build exceed rebuild_fraction of all points
    # (the points held in overflow lists after the last update!: 0 after a rebuild)
    movers = int(nhs.grid_info()["n_overflow"])
    if hashing:
        update_path = "rebuild (ParallelUpdate)"
    else:
        update_path = "overflow lists" if movers > 0 else "rebuild"
    st = P.lib().pn_sync(nhs.handle)
    if st != 0:
        raise RuntimeError(f"timed region reported status {st}")
    dev_s = t0.elapsed_time(t1) / 1e3
    upd = [ev[k][0].elapsed_time(ev[k][1]) for k in range(K)]
    den = [ev[k][1].elapsed_time(ev[k][2]) for k in range(K)]
    frc = [ev[k][2].elapsed_time(ev[k][3]) for k in range(K)]
    max_s, all_pairs = aggregate(dev_s, 2.0 * pairs_timed, world, device=torch.device("cuda"))
    value = all_pairs / max_s
    pairs_per_sweep = pairs_timed / K

    # ---- end to end through the C ABI with host buffers: the timed positions again (after a
    # warm-up at the first of them).  Every step copies
    # its positions and velocities from pinned host memory and its density and acceleration
    # back; the copies are double-buffered on two copy streams, so step k+1's inputs arrive
    # and step k-1's outputs leave while step k computes.
    e2e = None
    if not args.no_e2e:
        order = list(range(Wm, Wm + K))
        walk_h = [walk[i].cpu().pin_memory() for i in order]
        v_h = torch.as_tensor(v).reshape(-1).pin_memory()
        rho_h = [torch.empty(n, dtype=tdt).pin_memory() for _ in range(2)]
        acc_h = [torch.empty(3 * n, dtype=tdt).pin_memory() for _ in range(2)]
        xb = [torch.empty((n, 3), dtype=tcd, device="cuda") for _ in range(2)]
        xbT = [t.T for t in xb]
        vb = [torch.empty(3 * n, dtype=tdt, device="cuda") for _ in range(2)]
        rb = [torch.empty(n, dtype=tdt, device="cuda") for _ in range(2)]
        pb = [torch.empty(n, dtype=tdt, device="cuda") for _ in range(2)]
        ab = [torch.empty(3 * n, dtype=tdt, device="cuda") for _ in range(2)]
        dens_b = [P.WCSPHDensity(density=rb[i], pressure=pb[i], velocity=vb[i], **W.WCSPH)
                  for i in range(2)]
        force_b = [P.WCSPHForce(density=rb[i], pressure=pb[i], velocity=vb[i], accel=ab[i],
                                reuse_state=True, **W.WCSPH) for i in range(2)]
        comp = torch.cuda.current_stream()
        # positions and velocities are uploaded on two streams (two copy engines)
        s_in, s_in2, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        ev_in = [torch.cuda.Event() for _ in range(2)]
        ev_in2 = [torch.cuda.Event() for _ in range(2)]
        ev_done = [torch.cuda.Event() for _ in range(2)]
        ev_out = [torch.cuda.Event() for _ in range(2)]
        for e in ev_done + ev_out:
            e.record(comp)

        # per timed step: copy-in, compute and copy-out durations (events on their streams)
        tev = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(K)]
        timing = [False]

        def h2d(k, xh):
            bi = k % 2
            with torch.cuda.stream(s_in2):
                s_in2.wait_event(ev_done[bi])  # step k-2 no longer reads buffer bi
                vb[bi].copy_(v_h, non_blocking=True)
                ev_in2[bi].record(s_in2)
            with torch.cuda.stream(s_in):
                s_in.wait_event(ev_done[bi])
                if timing[0]:
                    tev[k][0].record(s_in)
                xb[bi].copy_(xh, non_blocking=True)
                s_in.wait_event(ev_in2[bi])  # the upload ends when both copies have
                if timing[0]:
                    tev[k][1].record(s_in)
                ev_in[bi].record(s_in)

        def compute(k):
            bi = k % 2
            comp.wait_event(ev_in[bi])
            comp.wait_event(ev_out[bi])  # step k-2's outputs have left
            if timing[0]:
                tev[k][2].record(comp)
            P.update(nhs, xbT[bi], xbT[bi], check=False)
            P.foreach_point_neighbor(dens_b[bi], xbT[bi], xbT[bi], nhs, check=False)
            P.foreach_point_neighbor(force_b[bi], xbT[bi], xbT[bi], nhs, check=False)
            if timing[0]:
                tev[k][3].record(comp)
            ev_done[bi].record(comp)

        def d2h(k):
            bi = k % 2
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_done[bi])
                if timing[0]:
                    tev[k][4].record(s_out)
                rho_h[bi].copy_(rb[bi], non_blocking=True)
                acc_h[bi].copy_(ab[bi], non_blocking=True)
                if timing[0]:
                    tev[k][5].record(s_out)
                ev_out[bi].record(s_out)

        def run(steps, src):
            h2d(0, src(0))
            for k in range(steps):
                if k + 1 < steps:
                    h2d(k + 1, src(k + 1))
                compute(k)
                d2h(k)
            comp.wait_event(ev_out[(steps - 1) % 2])

        run(3, lambda k: walk_h[0])
        torch.cuda.synchronize()
        barrier(world)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e2e_sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
        timing[0] = True
        a0.record(comp)
        s_in.wait_event(a0)
        s_in2.wait_event(a0)
        run(K, lambda k: walk_h[k])
        a1.record(comp)
        torch.cuda.synchronize()
        barrier(world)
        timing[0] = False
        e2e_clocks = e2e_sampler.stop() if e2e_sampler else None
        e2e_s, e2e_pairs = aggregate(a0.elapsed_time(a1) / 1e3, 2.0 * pairs_timed, world,
                                     device=torch.device("cuda"))
        if P.lib().pn_sync(nhs.handle) != 0:
            raise RuntimeError("e2e region reported an error")
        # the last step's outputs equal the device-timed run's (same positions, same search)
        same = bool(torch.equal(rho_h[(K - 1) % 2], rho.cpu()) and
                    torch.equal(acc_h[(K - 1) % 2], acc.cpu()))
        cb, vb_ = np.dtype(dt).itemsize, np.dtype(vdt).itemsize
        e2e = {"value": e2e_pairs / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": 3 * n * cb + 3 * n * vb_,
               "d2h_bytes_per_step": 4 * n * vb_, "ms_per_step": 1e3 * e2e_s / K,
               "outputs_equal_device_run": same,
               "h2d_ms": statistics.median(tev[k][0].elapsed_time(tev[k][1]) for k in range(K)),
               "compute_ms": statistics.median(tev[k][2].elapsed_time(tev[k][3])
                                               for k in range(K)),
               "d2h_ms": statistics.median(tev[k][4].elapsed_time(tev[k][5]) for k in range(K)),
               "h2d_ms_max": max(tev[k][0].elapsed_time(tev[k][1]) for k in range(K)),
               "compute_ms_max": max(tev[k][2].elapsed_time(tev[k][3]) for k in range(K)),
               "clocks": e2e_clocks,
               "path": "pinned host -> cudaMemcpyAsync (positions and velocities on two copy "
                       "streams, double-buffered) -> "
                       "pn_update + pn_foreach_point_neighbor (density, force) -> "
                       "cudaMemcpyAsync (second copy stream) -> pinned host density and "
                       "acceleration"}
        del walk_h
    del walk

    peak, peak_kind = hbm_peak()
    t_force = statistics.median(frc) / 1e3
    alg = FORCE_BYTES_PER_POINT[args.dtype] * n
    achieved = alg / t_force / 1e9
    tkey = (args.dtype, args.pair_cache > 0)
    roofline = {"bound": "hbm",
                "kernel": ("k_masks_sorted<FForce> (force sweep over the pair cache)"
                           if args.pair_cache > 0 else "k_trav_sorted<FForce> (force sweep)"),
                "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": (FORCE_TRAFFIC_BYTES_PER_POINT[tkey] * n
                            if tkey in FORCE_TRAFFIC_BYTES_PER_POINT and not hashing
                            else None),
                "layout": (("dense grid over the occupied cells" if nhs.grid_info()["grid_size"][0] > 1
                            else "hash lists") if hashing else "full grid"),
                "algorithmic_bytes_per_launch": alg,
                "note": ("force over the pair cache's hit masks and density + masks: "
                         "issue- and latency-bound (ncu at 4.1M points: issue slots 79 % / "
                         "88 %, L1 wavefronts 68 % / 71 %, DRAM < 5 % of peak; the force "
                         "walk waits on its neighbours' gathers)"
                         if args.pair_cache > 0 else
                         "issue-bound, not HBM-bound: ncu issue slots active 83 % (force), "
                         "93 % (density), DRAM < 2 % of peak")}

    # the roofline that binds: Float32 issue, for the force sweep's pair arithmetic (the
    # Float64 variant's pair arithmetic runs on the Float64 units: not reported)
    fp32_tf = fp32_peak(P)
    force_flops = FORCE_FLOPS_PER_PAIR * pairs_per_sweep
    fp32_roofline = None if args.dtype == "float64" else {
                     "bound": "fp32 issue", "kernel": roofline["kernel"],
                     "achieved": force_flops / t_force / 1e12, "peak": fp32_tf,
                     "peak_kind": "measured (pn_fma_probe)", "unit": "TFLOP/s",
                     "frac": force_flops / t_force / 1e12 / fp32_tf,
                     "flops_per_pair": FORCE_FLOPS_PER_PAIR,
                     "note": "pair arithmetic only (no candidate tests: the force sweep walks "
                             "the pair cache's neighbours); the rest of the issue slots go to "
                             "addressing, loads and the mask walk" if args.pair_cache > 0 else
                             "pair arithmetic only; the candidate tests and addressing take "
                             "the rest of the issue slots"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(x1, v, args, dt)

    metric = METRIC if args.dtype == "float32" else METRIC.replace(
        "FP32", "FP64" if args.dtype == "float64" else "FP64 coordinates, FP32 radius")
    out = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": 1e3 * max_s / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"float32": "f32", "float64": "f64",
                  "mixed": "f64 coordinates, f32 pair arithmetic"}[args.dtype],
        "data": "synthetic (seeded perturbed lattice, numpy PCG64)",
        "config": {"workload": f"WCSPH step, {n_side}^3 = {n:,} points 3D lattice, spacing 1, "
                               "U[-0.25,0.25] noise, r=3, " +
                               (f"SpatialHashingCellList(list_size={args.list_size or 2 * n}), "
                                "ParallelUpdate, "
                                if hashing else
                                f"FullGridCellList [-1,{n_side + 1}]^3, "
                                "ParallelIncrementalUpdate, ") +
                               "random walk N(0,0.05^2) per step",
                   "cell_list": args.cell_list,
                   "n_points": n, "search_radius": 3.0,
                   "pairs_per_sweep": pairs_per_sweep,
                   "pair_cache": args.pair_cache,
                   "parallelism": f"replicas x{world}",
                   "l2": "working set > L2 (coordinates, sorted copies and outputs ~1 GB), no flush"},
        "update_ms": statistics.median(upd), "density_ms": statistics.median(den),
        "force_ms": statistics.median(frc), "wall_ms_per_step": 1e3 * wall / K,
        "update_path": update_path, "points_in_overflow_lists": movers,
        "rebuild_fraction": None if hashing else args.rebuild_fraction,
        "gpu_launches": int(launches), "launches_per_step": launches / K,
        "roofline": roofline, "fp32_roofline": fp32_roofline, "e2e": e2e, "clocks": clocks,
        "cpu_baseline": cpu,
        "gpu": torch.cuda.get_device_name(),
    }
    return out


# ------------------------------------------------------------------ CPU (oracle)

def cpu_measure(x1, v, sample_n, dt, repeats=1):
    """Time the oracle on the host cores: threaded build of all points, then the density
    and force sweeps for `sample_n` query points.  Returns a dict of timings."""
    from oracle import pn_oracle as O
    from __graft_entry__ import package
    W = package().workloads
    n = len(x1)
    side = round(n ** (1 / 3))
    nthreads = O.n_threads_default()
    g = O.grid_create(3, dt(3.0), np.full(3, -1.0, dt), np.full(3, side + 1.0, dt),
                      max_ppc=64, dtype=dt)
    rng = np.random.default_rng(3)
    sample = np.sort(rng.choice(n, min(sample_n, n), replace=False)).astype(np.int32)
    t = time.perf_counter()
    cl = O.build(g, x1, parallel_threads=nthreads)
    t_build = time.perf_counter() - t
    prm, keep = O.make_params(**W.WCSPH)
    cnt = O.foreach(g, cl, x1, x1, O.F_COUNT, points=sample, n_threads=nthreads)
    pairs = int(cnt[sample].astype(np.int64).sum())
    best = None
    for _ in range(repeats):
        t = time.perf_counter()
        rho = O.foreach(g, cl, x1, x1, O.F_WCSPH_DENSITY, prm, points=sample, n_threads=nthreads)
        t_den = time.perf_counter() - t
        # pressure from the density (Tait), then the force sweep
        c = W.WCSPH
        p = c["c0"] ** 2 * c["rho0"] / c["gamma_exp"] * ((rho / c["rho0"]) ** c["gamma_exp"] - 1)
        rho_full = np.where(rho > 0, rho, 1.0)
        prm2, keep2 = O.make_params(rho=rho_full, pressure=p, vel=v.astype(np.float64),
                                    r_min=float(np.sqrt(np.finfo(dt).eps)) * c["h"], **c)
        t = time.perf_counter()
        O.foreach(g, cl, x1, x1, O.F_WCSPH_FORCE, prm2, points=sample, n_threads=nthreads)
        t_frc = time.perf_counter() - t
        cur = (t_den + t_frc, t_den, t_frc)
        best = cur if best is None or cur[0] < best[0] else best
    return {"pairs_sample": 2 * pairs, "t_sweeps": best[0], "t_density": best[1],
            "t_force": best[2], "t_build": t_build, "threads": nthreads,
            "sample": len(sample), "n": n}


def cpu_baseline(x1, v, args, dt):
    m = cpu_measure(x1, v, args.cpu_sample, dt)
    return {"value": m["pairs_sample"] / m["t_sweeps"], "unit": UNIT, "cores": m["threads"],
            "kind": "port",
            "sample": f"density+force sweeps for {m['sample']:,} of {m['n']:,} query points "
                      f"(cell list of all points, built in {m['t_build'] * 1e3:.0f} ms); "
                      "CPU restatement of the reference algorithm, pair math in FP64",
            "update_ms": m["t_build"] * 1e3}


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement on the host cores, rank 0 only."""
    if rank != 0:
        return
    from __graft_entry__ import package
    from oracle import build_oracle
    build_oracle.build()
    W = package().workloads
    dt = np.float32 if args.dtype == "float32" else np.float64
    x0, v, dx = W.wcsph_cloud(args.n_side, seed=1, dtype=dt)
    x1 = (x0.astype(np.float64) + dx).astype(dt)
    # each step is a bounded sample: the full cell-list build plus the two sweeps over a
    # sample of query points, sized so that warm-up + steps finish within minutes
    sample = max(10_000, args.cpu_sample // 8)
    for _ in range(args.warmup):
        cpu_measure(x1, v, sample // 4, dt)
    times, pairs, builds = [], 0, []
    for _ in range(args.steps):
        m = cpu_measure(x1, v, sample, dt)
        times.append(m["t_sweeps"])
        builds.append(m["t_build"])
        pairs += m["pairs_sample"]
    value = pairs / sum(times)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if dt == np.float32 else "f64", "data": "synthetic (seeded perturbed lattice)",
        "impl": "reference",
        "config": {"workload": f"WCSPH step, {args.n_side}^3 points, r=3 (CPU sample of "
                               f"{sample:,} query points per step)"},
        "update_ms": 1e3 * statistics.median(builds),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": m["threads"], "kind": "port",
                         "sample": f"{sample:,} query points per step, full cell-list build"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_gpu_sweep(args, rank, world, local):
    """Secondary workloads: one traversal per step (no update), device-timed."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    P = __graft_entry__.package()
    W = P.workloads
    torch.cuda.set_device(local)
    if args.workload == "nbody2d":
        side = 4096 if args.n_side == 200 else args.n_side
        x, m = W.periodic_nbody_cloud(side, seed=1, dtype=np.float32)
        n = len(x)
        box = P.PeriodicBox(min_corner=np.zeros(2, np.float32),
                            max_corner=np.full(2, float(side), np.float32))
        cl = P.FullGridCellList(min_corner=box.min_corner, max_corner=box.max_corner,
                                search_radius=np.float32(2.5), max_points_per_cell=0)
        nhs = P.GridNeighborhoodSearch(2, search_radius=np.float32(2.5), n_points=n,
                                       periodic_box=box, cell_list=cl)
        xd = torch.as_tensor(x, device="cuda").T
        md = torch.as_tensor(m, device="cuda")
        e = torch.zeros(n, device="cuda")
        f = P.TruncatedPotential(md, 2.5, e)
        desc = (f"2D periodic truncated potential, {side}^2 = {n:,} points, box [0,{side})^2, "
                "U[-0.3,0.3] noise, r=2.5, FP32")
        metric = "n-body pair-evals/s (2D periodic, FP32, r=2.5)"
        dt = "f32"
    else:
        x = W.perturbed_lattice((50, 50, 50), 0.25, seed=1, dtype=np.float64)
        n = len(x)
        cl = P.FullGridCellList(min_corner=np.full(3, -1.0), max_corner=np.full(3, 51.0),
                                search_radius=3.0, max_points_per_cell=0)
        nhs = P.GridNeighborhoodSearch(3, search_radius=3.0, n_points=n, cell_list=cl)
        xd = torch.as_tensor(x, device="cuda").T
        cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
        f = P.CountNeighbors(cnt)
        desc = "neighbour count, 50^3 = 125,000 points, U[-0.25,0.25] noise, r=3, FP64"
        metric = "count pair-evals/s (50^3, FP64, r=3)"
        dt = "f64"
    t = time.perf_counter()
    P.initialize(nhs, xd, xd)
    torch.cuda.synchronize()
    cnt2 = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt2), xd, xd, nhs)
    pairs = int(cnt2.to(torch.int64).sum())
    for _ in range(args.warmup):
        P.foreach_point_neighbor(f, xd, xd, nhs, check=False)
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record()
    P.initialize(nhs, xd, xd, check=False)
    b1.record()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = P.lib().pn_launch_count()
    t0.record()
    for _ in range(args.steps):
        P.foreach_point_neighbor(f, xd, xd, nhs, check=False)
    t1.record()
    torch.cuda.synchronize()
    if P.lib().pn_sync(nhs.handle) != 0:
        raise RuntimeError("timed region reported an error")
    sec = t0.elapsed_time(t1) / 1e3
    out = {"metric": metric, "value": pairs * args.steps / sec, "unit": "pair-evals/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": dt, "data": "synthetic (seeded perturbed lattice)",
           "config": {"workload": desc, "n_points": n, "pairs_per_sweep": pairs},
           "build_ms": b0.elapsed_time(b1),
           "gpu_launches": int(P.lib().pn_launch_count() - launches0),
           "gpu": torch.cuda.get_device_name()}
    return out


def run_gpu_adjoint(args, rank, world, local):
    """The adjoint workload: 100^3 = 1,000,000 points (lattice + U[-0.25, 0.25]), r = 3,
    L = sum (rho - 1)^2 + 0.01 E; a step is the forward sweep (density, loss terms, FP64
    loss) and the backward sweep (dL/dx, neighbour set fixed), both device-timed."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    P = __graft_entry__.package()
    torch.cuda.set_device(local)
    side = 100 if args.n_side == 200 else args.n_side
    dt = np.float32 if args.dtype == "float32" else np.float64
    tdt = torch.float32 if dt == np.float32 else torch.float64
    x = P.workloads.perturbed_lattice((side,) * 3, 0.25, seed=1, dtype=dt)
    n = len(x)
    r = dt(3.0)
    cl = P.FullGridCellList(min_corner=np.full(3, -1.0, dt), max_corner=np.full(3, side + 1.0, dt),
                            search_radius=r, max_points_per_cell=0)
    nhs = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl)
    xd = torch.as_tensor(x, device="cuda").T
    P.initialize(nhs, xd, xd)
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    P.foreach_point_neighbor(P.CountNeighbors(cnt), xd, xd, nhs)
    pairs = int(cnt.to(torch.int64).sum())
    consts = dict(mass=1.0, h=1.5, cutoff=3.0, lambda_pot=0.01)
    rho = torch.empty(n, dtype=tdt, device="cuda")
    terms = torch.empty(n, dtype=tdt, device="cuda")
    loss = torch.empty(1, dtype=torch.float64, device="cuda")
    grad = torch.empty(3 * n, dtype=tdt, device="cuda")
    fwd = P.AdjointLossForward(density=rho, terms=terms, loss=loss, **consts)
    bwd = P.AdjointLossBackward(grad=grad, reuse_state=True, **consts)
    for _ in range(args.warmup):
        P.foreach_point_neighbor(fwd, xd, xd, nhs, check=False)
        P.foreach_point_neighbor(bwd, xd, xd, nhs, check=False)
    torch.cuda.synchronize()
    K = args.steps
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(K)]
    launches0 = P.lib().pn_launch_count()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    torch.cuda.synchronize()
    for k in range(K):
        ev[k][0].record()
        P.foreach_point_neighbor(fwd, xd, xd, nhs, check=False)
        ev[k][1].record()
        P.foreach_point_neighbor(bwd, xd, xd, nhs, check=False)
        ev[k][2].record()
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    if P.lib().pn_sync(nhs.handle) != 0:
        raise RuntimeError("timed region reported an error")
    f_ms = statistics.median(ev[k][0].elapsed_time(ev[k][1]) for k in range(K))
    b_ms = statistics.median(ev[k][1].elapsed_time(ev[k][2]) for k in range(K))
    tot_s = sum(ev[k][0].elapsed_time(ev[k][2]) for k in range(K)) / 1e3
    grad_err = grad_err_all = None
    grad_set_diff = None
    if dt == np.float32:
        # the Float32 gradient against the library's Float64 one on the same points (the
        # Float64 forward/backward agree with the FP64 oracle to 1e-10 in tests/test_adjoint.py)
        x64 = torch.as_tensor(x.astype(np.float64), device="cuda").T
        cl64 = P.FullGridCellList(min_corner=np.full(3, -1.0), max_corner=np.full(3, side + 1.0),
                                  search_radius=3.0, max_points_per_cell=0)
        nhs64 = P.GridNeighborhoodSearch(3, search_radius=3.0, n_points=n, cell_list=cl64)
        P.initialize(nhs64, x64, x64)
        g64 = torch.empty(3 * n, dtype=torch.float64, device="cuda")
        P.foreach_point_neighbor(P.AdjointLossForward(
            density=torch.empty(n, dtype=torch.float64, device="cuda"),
            terms=torch.empty(n, dtype=torch.float64, device="cuda"),
            loss=torch.empty(1, dtype=torch.float64, device="cuda"), **consts), x64, x64, nhs64)
        P.foreach_point_neighbor(P.AdjointLossBackward(grad=g64, reuse_state=True, **consts),
                                 x64, x64, nhs64)
        # The two searches decide pairs at d ~ r in their own precision, and the truncated
        # potential's derivative does not vanish at the cutoff, so a pair that one precision
        # puts at d < r and the other at d >= r moves both its points' gradients by about
        # lambda / r^2.  Compare the other points: those whose neighbour counts agree and
        # have no pair whose Float32 d^2 lies in the last rounding step below r^2 (found by
        # a count at the next smaller Float32 radius); the rest are reported.
        c32 = torch.zeros(n, dtype=torch.int32, device="cuda")
        c64 = torch.zeros(n, dtype=torch.int32, device="cuda")
        cin = torch.zeros(n, dtype=torch.int32, device="cuda")
        P.foreach_point_neighbor(P.CountNeighbors(c32), xd, xd, nhs)
        P.foreach_point_neighbor(P.CountNeighbors(c64), x64, x64, nhs64)
        r_in = np.nextafter(np.float32(3.0), np.float32(0.0))
        cl_in = P.FullGridCellList(min_corner=np.full(3, -1.0, np.float32),
                                   max_corner=np.full(3, side + 1.0, np.float32),
                                   search_radius=r_in, max_points_per_cell=0)
        nhs_in = P.GridNeighborhoodSearch(3, search_radius=r_in, n_points=n, cell_list=cl_in)
        P.initialize(nhs_in, xd, xd)
        P.foreach_point_neighbor(P.CountNeighbors(cin), xd, xd, nhs_in)
        ok = (c32 == c64) & (c32 == cin)
        diff = (grad.double() - g64).abs()
        grad_err = float(diff[ok.repeat_interleave(3)].max() / g64.abs().max())
        grad_err_all = float(diff.max() / g64.abs().max())
        grad_set_diff = int((~ok).sum())
    out = {"metric": f"adjoint pair-evals/s (1M pts, {'FP32' if dt == np.float32 else 'FP64'}, "
                     "r=3, forward loss + backward dL/dx)",
           "value": 2.0 * pairs * K / tot_s, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / K, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if dt == np.float32 else "f64", "data": "synthetic (seeded perturbed lattice)",
           "config": {"workload": f"adjoint loss sum (rho-1)^2 + 0.01 E, {side}^3 = {n:,} points, "
                                  "U[-0.25,0.25] noise, r=3, Wendland h=1.5, 1/r potential cutoff 3",
                      "pairs_per_sweep": pairs},
           "forward_ms": f_ms, "backward_ms": b_ms, "backward_over_forward": b_ms / f_ms,
           "grad_rel_err_vs_f64": grad_err,
           "grad_rel_err_definition": "max |dL/dx (FP32) - dL/dx (FP64, this library)| / "
                                      "max |dL/dx (FP64)|, over the points with no pair at "
                                      "the cutoff within Float32 rounding (same neighbour "
                                      "count in FP32 and FP64, and at the next smaller FP32 "
                                      "radius)",
           "grad_rel_err_all_points": grad_err_all,
           "points_with_a_pair_at_the_cutoff": grad_set_diff,
           "loss": float(loss.item()),
           "gpu_launches": int(P.lib().pn_launch_count() - launches0), "clocks": clocks,
           "gpu": torch.cuda.get_device_name()}
    return out


def run_gpu_batched(args, rank, world, local):
    """512 independent 3D FP32 clouds (N log-uniform in [1e3, 2e5], perturbed cubic
    lattices, radius U[2, 3.5], h = r/2): a step is update! (every point displaced by
    N(0, 0.05^2)) + WCSPH density + force of every cloud.  Timed three ways on the same GPU: one search per
    cloud with its own launches (C ABI calls in a loop), the batch's direct calls, and the
    batch's captured CUDA graph (including the copy of the step's positions into the graph's
    input buffer)."""
    import ctypes as C
    import torch
    import __graft_entry__
    __graft_entry__.build()
    P = __graft_entry__.package()
    L = P._lib
    lib = P.lib()
    torch.cuda.set_device(local)
    clouds = P.workloads.batched_clouds(n_clouds=args.clouds, seed=1)
    ncl = len(clouds)
    sizes = [len(c["x"]) for c in clouds]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    N = int(off[-1])
    searches = []
    for c in clouds:
        r = np.float32(c["radius"])
        cl = P.FullGridCellList(min_corner=np.asarray(c["min_corner"], np.float32),
                                max_corner=np.asarray(c["max_corner"], np.float32),
                                search_radius=r, max_points_per_cell=0)
        searches.append(P.GridNeighborhoodSearch(3, search_radius=r, n_points=len(c["x"]),
                                                 cell_list=cl))
    K, Wm = args.steps, args.warmup
    # positions: the lattices x0 and x1 = x0 + N(0, 0.05^2), alternating (every update!
    # re-bins all points; each step moves every point by one displacement)
    x0 = torch.as_tensor(np.concatenate([c["x"] for c in clouds]), device="cuda")
    x1 = x0 + torch.as_tensor(np.concatenate([c["dx"] for c in clouds]), device="cuda")
    walk = [x1 if s_ % 2 == 0 else x0 for s_ in range(Wm + K)]
    v = torch.as_tensor(np.concatenate([c["v"] for c in clouds]), device="cuda").reshape(-1)
    Wc = dict(P.workloads.WCSPH)
    h = [c["radius"] / 2 for c in clouds]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def outputs():
        return (torch.zeros(N, device="cuda"), torch.zeros(N, device="cuda"),
                torch.zeros(3 * N, device="cuda"))

    # ---- per-cloud searches, their own launches
    rho1, prs1, acc1 = outputs()
    eps = float(np.sqrt(np.finfo(np.float32).eps))
    dens_p, forc_p = [], []
    for k in range(ncl):
        common = dict(mass=Wc["mass"], h=h[k], c0=Wc["c0"], rho0=Wc["rho0"],
                      gamma_exp=Wc["gamma_exp"], alpha=Wc["alpha"], eps_visc=Wc["eps_visc"],
                      r_min=eps * h[k], density=rho1.data_ptr() + 4 * int(off[k]),
                      pressure=prs1.data_ptr() + 4 * int(off[k]),
                      velocity=v.data_ptr() + 12 * int(off[k]))
        dens_p.append(L.pn_wcsph_params(**common))
        forc_p.append(L.pn_wcsph_params(accel=acc1.data_ptr() + 12 * int(off[k]), reuse_state=1,
                                        **common))
    handles = [s.handle for s in searches]
    for k in range(ncl):
        xk = C.c_void_p(x0.data_ptr() + 12 * int(off[k]))
        if lib.pn_initialize(handles[k], xk, sizes[k], None, 0, stream) != 0:
            raise RuntimeError("per-cloud initialize failed")

    def per_cloud_step(xs):
        base = xs.data_ptr()
        for k in range(ncl):
            xk = C.c_void_p(base + 12 * int(off[k]))
            lib.pn_update(handles[k], xk, sizes[k], None, 0, 1, stream)
            lib.pn_foreach_point_neighbor(handles[k], L.PN_F_WCSPH_DENSITY, xk, sizes[k], xk,
                                          sizes[k], None, 0, C.byref(dens_p[k]), stream)
            lib.pn_foreach_point_neighbor(handles[k], L.PN_F_WCSPH_FORCE, xk, sizes[k], xk,
                                          sizes[k], None, 0, C.byref(forc_p[k]), stream)

    def timed(fn):
        for s_ in range(Wm):
            fn(walk[s_])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for s_ in range(K):
            fn(walk[Wm + s_])
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K

    launches0 = lib.pn_launch_count()
    per_cloud_ms = timed(per_cloud_step)
    per_cloud_launches = (lib.pn_launch_count() - launches0) / (Wm + K)
    for k, hd in enumerate(handles):
        st = lib.pn_sync(hd)
        if st != 0:
            raise RuntimeError(f"per-cloud path reported status {st} on cloud {k}")

    # ---- the batch: direct calls, then the captured graph
    batch = P.BatchedNeighborhoodSearch(searches)
    rho2, prs2, acc2 = outputs()
    step = P.WCSPHStep(density=rho2, pressure=prs2, velocity=v, accel=acc2, **dict(Wc, h=h))
    batch.initialize(x0.T)
    dens = P.WCSPHDensity(density=rho2, pressure=prs2, velocity=v, **dict(Wc, h=h))
    forc = P.WCSPHForce(density=rho2, pressure=prs2, velocity=v, accel=acc2, reuse_state=True,
                        **dict(Wc, h=h))
    t_tune = time.perf_counter()
    sched = {"density": batch.autotune(dens, x0.T, reps=3),
             "force": batch.autotune(forc, x0.T, reps=3)}
    t_tune = time.perf_counter() - t_tune

    def batch_step(xs):
        batch.update(xs.T, check=False)
        batch.foreach_point_neighbor(step, xs.T, check=False)

    launches0 = lib.pn_launch_count()
    batch_ms = timed(batch_step)
    batch_launches = (lib.pn_launch_count() - launches0) / (Wm + K)
    batch.sync()
    same_direct = bool(torch.equal(rho1, rho2) and torch.equal(acc1, acc2))

    xbuf = x0.clone()
    batch.capture_step(xbuf.T, step)

    def graph_step(xs):
        xbuf.copy_(xs)
        batch.launch_step()

    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    launches0 = lib.pn_launch_count()
    graph_ms = timed(graph_step)
    clocks = sampler.stop() if sampler else None
    batch.sync()
    same_graph = bool(torch.equal(rho1, rho2) and torch.equal(acc1, acc2))

    # ordered pairs (self included) at the timed positions, for pair-evals/s
    cnt = torch.zeros(N, dtype=torch.int32, device="cuda")
    pairs = 0
    for xs in (x0, x1):
        batch.update(xs.T)
        batch.foreach_point_neighbor(P.CountNeighbors(cnt), xs.T)
        pairs += int(cnt.to(torch.int64).sum()) * sum(1 for s_ in range(Wm, Wm + K)
                                                      if walk[s_] is xs)
    out = {"metric": "batched WCSPH step speed-up: per-cloud launches / CUDA-graph batch "
                     f"({args.clouds} clouds, same GPU)",
           "value": per_cloud_ms / graph_ms, "unit": "x", "n_gpus": world, "steps": K,
           "warmup": Wm, "ms_per_step": graph_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded perturbed lattices)",
           "config": {"workload": f"{args.clouds} clouds, N log-uniform [1e3, 2e5] (side round(N^(1/3)), "
                                  f"total {N:,} points), radius U[2, 3.5], h = r/2, box "
                                  "[-1, side+1]^3, positions alternating x0 / x0 + N(0,0.05^2), "
                                  "update! + WCSPH density + force",
                      "n_points": N, "pairs_per_step": pairs // K},
           "per_cloud_ms": per_cloud_ms, "batch_direct_ms": batch_ms, "batch_graph_ms": graph_ms,
           "pair_evals_per_s_graph": 2.0 * pairs / K / (graph_ms / 1e3),
           "launches_per_step": {"per_cloud": per_cloud_launches, "batch": batch_launches},
           "schedules": sched, "autotune_s": t_tune,
           "identical_results": {"direct": same_direct, "graph": same_graph},
           "gpu_launches": int(batch_launches * K), "clocks": clocks,
           "gpu": torch.cuda.get_device_name()}
    return out


def run_gpu_precomputed(args, rank, world, local):
    """The 8M-point FP32 WCSPH step with a PrecomputedNeighborhoodSearch: update! rebuilds
    the neighbour lists (through the grid search), then the density and force sweeps walk
    them.  Same positions (random walk N(0, 0.05^2)), constants and metric as the default
    workload; `loops_ms` times the two sweeps alone (lists reused), the case the
    precomputed search is for."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    P = __graft_entry__.package()
    W = P.workloads
    torch.cuda.set_device(local)
    n_side = args.n_side
    x0, v, dx = W.wcsph_cloud(n_side, seed=1, dtype=np.float32)
    x1 = (x0.astype(np.float64) + dx).astype(np.float32)
    n = len(x0)
    r = np.float32(3.0)
    cl = P.FullGridCellList(min_corner=np.full(3, -1.0, np.float32),
                            max_corner=np.full(3, n_side + 1.0, np.float32), search_radius=r,
                            max_points_per_cell=0)
    grid = P.GridNeighborhoodSearch(3, search_radius=r, n_points=n, cell_list=cl,
                                    update_strategy=P.ParallelIncrementalUpdate())
    # the reference's default capacity (320 neighbours per point in 3D): lists of fixed
    # capacity, built in one pass without a host synchronisation
    pre = P.PrecomputedNeighborhoodSearch(3, n_points=n, update_neighborhood_search=grid)
    K, Wm = args.steps, args.warmup
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    walk = [torch.as_tensor(x1, device="cuda")]
    for _ in range(Wm + K - 1):
        walk.append(walk[-1] + 0.05 * torch.randn(walk[-1].shape, generator=gen, device="cuda"))
    vd = torch.as_tensor(v, device="cuda").reshape(-1)
    rho = torch.zeros(n, device="cuda")
    prs = torch.zeros(n, device="cuda")
    acc = torch.zeros(3 * n, device="cuda")
    dens = P.WCSPHDensity(density=rho, pressure=prs, velocity=vd, **W.WCSPH)
    force = P.WCSPHForce(density=rho, pressure=prs, velocity=vd, accel=acc, reuse_state=True,
                         **W.WCSPH)
    x0d = torch.as_tensor(x0, device="cuda").T
    P.initialize(pre, x0d, x0d)
    for s_ in range(Wm):
        xs = walk[s_].T
        P.update(pre, xs, xs)
        P.foreach_point_neighbor(dens, xs, xs, pre, check=False)
        P.foreach_point_neighbor(force, xs, xs, pre, check=False)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(K)]
    pairs = 0
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    wall0 = time.perf_counter()
    upd_wall = 0.0
    for k in range(K):
        xs = walk[Wm + k].T
        e = ev[k]
        e[0].record()
        t = time.perf_counter()
        P.update(pre, xs, xs, check=False)
        upd_wall += time.perf_counter() - t
        e[1].record()
        P.foreach_point_neighbor(dens, xs, xs, pre, check=False)
        e[2].record()
        P.foreach_point_neighbor(force, xs, xs, pre, check=False)
        e[3].record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if pre._sync() != 0:
        raise RuntimeError("timed region reported an error")
    for k in range(K):
        xs = walk[Wm + k].T
        P.update(pre, xs, xs)
        P.foreach_point_neighbor(P.CountNeighbors(cnt), xs, xs, pre)
        pairs += int(cnt.to(torch.int64).sum())
    upd = [ev[k][0].elapsed_time(ev[k][1]) for k in range(K)]
    den = [ev[k][1].elapsed_time(ev[k][2]) for k in range(K)]
    frc = [ev[k][2].elapsed_time(ev[k][3]) for k in range(K)]
    step_ms = sum(ev[k][0].elapsed_time(ev[k][3]) for k in range(K)) / K
    # the two sweeps alone, lists reused (the precomputed search's purpose)
    xs = walk[-1].T
    P.update(pre, xs, xs)
    l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0.record()
    for _ in range(K):
        P.foreach_point_neighbor(dens, xs, xs, pre, check=False)
        P.foreach_point_neighbor(force, xs, xs, pre, check=False)
    l1.record()
    torch.cuda.synchronize()
    loops_ms = l0.elapsed_time(l1) / K
    out = {"metric": "WCSPH pair-evals/s (8M pts, FP32, r=3, PrecomputedNeighborhoodSearch: "
                     "update! with list rebuild + density + force)",
           "value": 2.0 * pairs / (step_ms * K / 1e3), "unit": UNIT, "n_gpus": world,
           "steps": K, "warmup": Wm, "ms_per_step": step_ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded perturbed lattice, numpy PCG64)",
           "config": {"workload": f"WCSPH step, {n_side}^3 = {n:,} points, as the default "
                                  "workload, PrecomputedNeighborhoodSearch over the grid search",
                      "pairs_per_sweep": pairs / K},
           "update_ms": statistics.median(upd), "density_ms": statistics.median(den),
           "force_ms": statistics.median(frc), "loops_ms": loops_ms,
           "loops_pair_evals_per_s": 2.0 * pairs / K / (loops_ms / 1e3),
           "wall_ms_per_step": 1e3 * wall / K, "update_host_ms": 1e3 * upd_wall / K,
           "gpu": torch.cuda.get_device_name()}
    return out


def extra_records(args, rank, world, local):
    """The rest of the headline metric ("batched & adjoint vs plain, same GPU"), measured in
    the same run on the same GPU after the plain step: the batched 512-cloud step against
    per-cloud launches, the adjoint step's backward/forward ratio, the 8M step in Float64,
    and the plain step with update! forced onto its overflow-list path.  Each record carries
    its own CUDA-event times and clock samples."""
    import copy
    K, Wm = args.steps, args.warmup

    def sub(**kw):
        a = copy.copy(args)
        a.no_e2e, a.no_cpu, a.no_extras = True, True, True
        for k, v in kw.items():
            setattr(a, k, v)
        return a

    rec = {}
    t = time.perf_counter()
    rec["update_paths"] = {
        "overflow": _path_record(run_gpu(sub(rebuild_fraction=1.0), rank, world, local)),
        "note": "rebuild_fraction 1.0: update! keeps the movers in overflow lists (never "
                "rebuilds) and moves the other points in place; the rows are clipped by the "
                "sort keys widened by the largest in-place move, and the pair cache also "
                "holds each row's overflow run"}
    rec["batched"] = run_gpu_batched(sub(steps=min(K, 10), warmup=min(Wm, 3)), rank, world, local)
    rec["adjoint"] = run_gpu_adjoint(sub(dtype="float32"), rank, world, local)
    rec["fp64"] = _path_record(run_gpu(sub(dtype="float64", steps=min(K, 5),
                                           warmup=min(Wm, 3)), rank, world, local))
    rec["extras_wall_s"] = time.perf_counter() - t
    return rec


def _path_record(o):
    keep = ("metric", "value", "unit", "ms_per_step", "update_ms", "density_ms", "force_ms",
            "update_path", "points_in_overflow_lists", "dtype", "steps", "warmup", "clocks",
            "gpu_launches")
    return {k: o[k] for k in keep if k in o}


def main():
    args = parse()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, rank, world)
        return
    rank, world, local = dist_setup("nccl")
    try:
        if args.workload == "wcsph":
            out = run_gpu(args, rank, world, local)
            if not args.no_extras and args.dtype == "float32" and args.cell_list == "full_grid":
                out.update(extra_records(args, rank, world, local))
        elif args.workload == "adjoint":
            out = run_gpu_adjoint(args, rank, world, local)
        elif args.workload == "batched":
            out = run_gpu_batched(args, rank, world, local)
        elif args.workload == "precomputed":
            out = run_gpu_precomputed(args, rank, world, local)
        else:
            out = run_gpu_sweep(args, rank, world, local)
        if rank == 0:
            print(json.dumps(out))
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
