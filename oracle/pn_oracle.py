"""ctypes wrapper around the CPU oracle (oracle/pn_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by the
CPU-baseline leg of bench.py, always as the answer the CUDA path is compared with or the
timed CPU restatement, never as part of the product path.

Arrays of points use the reference's memory layout: a Julia `T[d, N]` column-major
matrix is a C-contiguous numpy array of shape (N, d) here.  Point indices are 0-based.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

PNO_OK, PNO_ERR_OUT_OF_DOMAIN, PNO_ERR_INVALID_ARG, PNO_ERR_CELL_FULL = 0, 1, 2, 6
F_COUNT, F_NBODY_ACCEL, F_POTENTIAL, F_WCSPH_DENSITY, F_WCSPH_FORCE, F_INDEX_SUM = 0, 2, 3, 4, 5, 7


class OracleError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: oracle status {status}")
        self.status = status


class Grid(C.Structure):
    _fields_ = [
        ("ndims", C.c_int32), ("periodic", C.c_int32), ("dtype", C.c_int32),
        ("max_ppc", C.c_int32), ("n", C.c_int64 * 3), ("n_cells", C.c_int64 * 3),
        ("n_total", C.c_int64), ("min_pad", C.c_double * 3), ("max_pad", C.c_double * 3),
        ("cell_size", C.c_double * 3), ("box_min", C.c_double * 3),
        ("box_max", C.c_double * 3), ("box_size", C.c_double * 3), ("radius", C.c_double),
        ("is_template", C.c_int32), ("mixed", C.c_int32), ("list_size", C.c_int64),
    ]


class Params(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("masses", C.c_void_p), ("G", C.c_double),
        ("cutoff", C.c_double), ("h", C.c_double), ("c0", C.c_double),
        ("rho0", C.c_double), ("gamma_exp", C.c_double), ("alpha", C.c_double),
        ("eps_visc", C.c_double), ("r_min", C.c_double), ("rho", C.c_void_p),
        ("pressure", C.c_void_p), ("vel", C.c_void_p), ("lambda_pot", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle.build())
    return _lib


def _sfx(dtype) -> str:
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f(dtype, name):
    fn = getattr(lib(), f"pno_{name}_{_sfx(dtype)}")
    return fn


def n_threads_default() -> int:
    return len(os.sched_getaffinity(0))


# ---------------------------------------------------------------- geometry


def floor_to_int(x, dtype=np.float64) -> int:
    fn = _f(dtype, "floor_to_int")
    fn.restype = C.c_int64
    fn.argtypes = [C.c_float if np.dtype(dtype) == np.float32 else C.c_double]
    return int(fn(float(x)))


def grid_create(ndims, radius, min_corner, max_corner, periodic_box=None, max_ppc=100,
                dtype=np.float64) -> Grid:
    """FullGridCellList + GridNeighborhoodSearch geometry (full_grid.jl:48-82,
    nhs_grid.jl:77-129).  `periodic_box` is a (min_corner, max_corner) pair or None."""
    dt = np.dtype(dtype)
    g = Grid()
    mn = np.ascontiguousarray(min_corner, dtype=dt)
    mx = np.ascontiguousarray(max_corner, dtype=dt)
    pmn = pmx = None
    if periodic_box is not None:
        pmn = np.ascontiguousarray(periodic_box[0], dtype=dt)
        pmx = np.ascontiguousarray(periodic_box[1], dtype=dt)
    fn = _f(dt, "grid_create")
    ctyp = C.c_float if dt == np.float32 else C.c_double
    fn.argtypes = [C.c_int32, ctyp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_int32, C.POINTER(Grid)]
    st = fn(ndims, float(dt.type(radius)), _ptr(mn), _ptr(mx), _ptr(pmn), _ptr(pmx),
            int(max_ppc), C.byref(g))
    if st != PNO_OK:
        raise OracleError(st, "grid_create")
    return g


def grid_create_mixed(ndims, radius, min_corner, max_corner, periodic_box=None, max_ppc=100):
    """Float64 coordinates with a Float32 search radius (pno_grid_create_mixed); the grid is
    then used with the Float64 functions."""
    mn = np.ascontiguousarray(min_corner, dtype=np.float64)
    mx = np.ascontiguousarray(max_corner, dtype=np.float64)
    pmn = pmx = None
    if periodic_box is not None:
        pmn = np.ascontiguousarray(periodic_box[0], dtype=np.float32)
        pmx = np.ascontiguousarray(periodic_box[1], dtype=np.float32)
    fn = lib().pno_grid_create_mixed
    fn.argtypes = [C.c_int32, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_int32, C.POINTER(Grid)]
    st = fn(ndims, float(np.float32(radius)), _ptr(mn), _ptr(mx), _ptr(pmn), _ptr(pmx),
            int(max_ppc), C.byref(g := Grid()))
    if st != PNO_OK:
        raise OracleError(st, "grid_create_mixed")
    return g


def cell_coords(g: Grid, x, dtype=None) -> tuple:
    dt = np.dtype(dtype or (np.float32 if g.dtype == 0 else np.float64))
    xa = np.ascontiguousarray(x, dtype=dt)
    out = np.zeros(3, dtype=np.int64)
    fn = _f(dt, "cell_coords")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p]
    fn(C.byref(g), _ptr(xa), _ptr(out))
    return tuple(int(v) for v in out[: g.ndims])


def cell_coords_dict(g: Grid, x) -> tuple:
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt)
    out = np.zeros(3, dtype=np.int64)
    fn = _f(dt, "cell_coords_dict")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p]
    fn(C.byref(g), _ptr(xa), _ptr(out))
    return tuple(int(v) for v in out[: g.ndims])


def periodic_coords(g: Grid, x):
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt)
    out = np.zeros(g.ndims, dtype=dt)
    fn = _f(dt, "periodic_coords")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p]
    fn(C.byref(g), _ptr(xa), _ptr(out))
    return out


# ---------------------------------------------------------------- cell list


class CellList:
    """DynamicVectorOfVectors backend (max_ppc x n_cells) plus lengths, like the reference."""

    def __init__(self, g: Grid):
        self.g = g
        self.cells = np.zeros(max(g.n_total, 1) * g.max_ppc, dtype=np.int32)
        self.lengths = np.zeros(max(g.n_total, 1), dtype=np.int32)

    def column(self, lin: int) -> np.ndarray:
        return self.cells[lin * self.g.max_ppc: lin * self.g.max_ppc + self.lengths[lin]]

    def as_csr(self):
        """(counts[n_cells], points) with each cell's points in column order."""
        pts = [self.column(c) for c in range(self.g.n_total)]
        return self.lengths.copy(), (np.concatenate(pts) if pts else np.zeros(0, np.int32))


def build(g: Grid, y, idx=None, parallel_threads: int = 0) -> CellList:
    dt = np.float32 if g.dtype == 0 else np.float64
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, g.ndims)
    cl = CellList(g)
    if parallel_threads > 0:
        fn = _f(dt, "build_parallel")
        fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32]
        st = fn(C.byref(g), _ptr(ya), ya.shape[0], _ptr(cl.cells), _ptr(cl.lengths),
                int(parallel_threads))
    else:
        ia = None if idx is None else np.ascontiguousarray(idx, dtype=np.int32)
        fn = _f(dt, "build")
        fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                       C.c_void_p, C.c_void_p]
        st = fn(C.byref(g), _ptr(ya), ya.shape[0], _ptr(ia), 0 if ia is None else ia.size,
                _ptr(cl.cells), _ptr(cl.lengths))
    if st != PNO_OK:
        raise OracleError(st, "build")
    return cl


# ---------------------------------------------------------------- traversal


def make_params(**kw) -> tuple[Params, list]:
    """Params struct plus the list of arrays it points into (kept alive by the caller)."""
    p = Params()
    keep = []
    for name, _ in Params._fields_:
        if name in kw:
            v = kw[name]
            if name in ("masses", "rho", "pressure", "vel"):
                a = np.ascontiguousarray(v, dtype=np.float64)
                keep.append(a)
                setattr(p, name, a.ctypes.data)
            else:
                setattr(p, name, float(v))
    return p, keep


def foreach(g: Grid, cl: CellList, x, y, functor: int, params: Params | None = None,
            points=None, n_threads: int = 0, want_abs: bool = False):
    dt = np.float32 if g.dtype == 0 else np.float64
    d = g.ndims
    xa = np.ascontiguousarray(x, dtype=dt).reshape(-1, d)
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, d)
    nx = xa.shape[0]
    if functor == F_COUNT:
        out = np.zeros(nx, dtype=np.int32)
    elif functor == F_INDEX_SUM:
        out = np.zeros(nx, dtype=np.int64)
    elif functor in (F_NBODY_ACCEL, F_WCSPH_FORCE):
        out = np.zeros((nx, d), dtype=np.float64)
    else:
        out = np.zeros(nx, dtype=np.float64)
    ab = np.zeros_like(out, dtype=np.float64) if want_abs else None
    pa = None if points is None else np.ascontiguousarray(points, dtype=np.int32)
    if params is None:
        params = Params()
    fn = _f(dt, "foreach")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32,
                   C.POINTER(Params), C.c_void_p, C.c_void_p, C.c_int32]
    st = fn(C.byref(g), _ptr(cl.cells), _ptr(cl.lengths), _ptr(xa), nx, _ptr(ya),
            ya.shape[0], _ptr(pa), 0 if pa is None else pa.size, functor, C.byref(params),
            _ptr(out), _ptr(ab), int(n_threads or n_threads_default()))
    if st != PNO_OK:
        raise OracleError(st, "foreach")
    return (out, ab) if want_abs else out


def _lists(fn_name, args_head, g, nx, n_threads):
    dt = np.float32 if g.dtype == 0 else np.float64
    fn = _f(dt, fn_name)
    counts = np.zeros(nx, dtype=np.int32)
    st = fn(*args_head, None, _ptr(counts), None, int(n_threads or n_threads_default()))
    if st != PNO_OK:
        raise OracleError(st, fn_name)
    offsets = np.zeros(nx + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    nbrs = np.zeros(int(offsets[-1]), dtype=np.int32)
    st = fn(*args_head, _ptr(offsets), _ptr(counts), _ptr(nbrs),
            int(n_threads or n_threads_default()))
    if st != PNO_OK:
        raise OracleError(st, fn_name)
    return offsets, nbrs


def neighbor_lists(g: Grid, cl: CellList, x, y, n_threads: int = 0):
    """CSR (offsets[n_x+1], nbrs) in the reference's traversal order."""
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt).reshape(-1, g.ndims)
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, g.ndims)
    fn = _f(dt, "neighbor_lists")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    head = (C.byref(g), _ptr(cl.cells), _ptr(cl.lengths), _ptr(xa), xa.shape[0], _ptr(ya),
            ya.shape[0])
    return _lists("neighbor_lists", head, g, xa.shape[0], n_threads)


def trivial_lists(g: Grid, x, y, n_threads: int = 0):
    """Brute force (TrivialNeighborhoodSearch), CSR in ascending j."""
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt).reshape(-1, g.ndims)
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, g.ndims)
    fn = _f(dt, "trivial_lists")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    head = (C.byref(g), _ptr(xa), xa.shape[0], _ptr(ya), ya.shape[0])
    return _lists("trivial_lists", head, g, xa.shape[0], n_threads)


def eachneighbor(g: Grid, cl: CellList, q) -> np.ndarray:
    dt = np.float32 if g.dtype == 0 else np.float64
    qa = np.ascontiguousarray(q, dtype=dt)
    fn = _f(dt, "eachneighbor")
    fn.restype = C.c_int64
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
    cap = 1 << 16
    out = np.zeros(cap, dtype=np.int32)
    n = fn(C.byref(g), _ptr(cl.cells), _ptr(cl.lengths), _ptr(qa), _ptr(out), cap)
    if n < 0:
        raise OracleError(PNO_ERR_OUT_OF_DOMAIN, "eachneighbor")
    return out[:n].copy()


def eachneighbor_dict(g: Grid, y, q) -> np.ndarray:
    dt = np.float32 if g.dtype == 0 else np.float64
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, g.ndims)
    qa = np.ascontiguousarray(q, dtype=dt)
    fn = _f(dt, "eachneighbor_dict")
    fn.restype = C.c_int64
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64]
    cap = 1 << 16
    out = np.zeros(cap, dtype=np.int32)
    n = fn(C.byref(g), _ptr(ya), ya.shape[0], _ptr(qa), _ptr(out), cap)
    return out[:n].copy()


def loss_grad(g: Grid, cl: CellList, x, params: Params, n_threads: int = 0, grad=True):
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt).reshape(-1, g.ndims)
    n = xa.shape[0]
    rho = np.zeros(n, dtype=np.float64)
    loss = C.c_double(0.0)
    gr = np.zeros((n, g.ndims), dtype=np.float64) if grad else None
    fn = _f(dt, "loss_grad")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                   C.POINTER(Params), C.c_void_p, C.POINTER(C.c_double), C.c_void_p, C.c_int32]
    st = fn(C.byref(g), _ptr(cl.cells), _ptr(cl.lengths), _ptr(xa), n, C.byref(params),
            _ptr(rho), C.byref(loss), _ptr(gr), int(n_threads or n_threads_default()))
    if st != PNO_OK:
        raise OracleError(st, "loss_grad")
    return loss.value, rho, gr


def loss_fd(g: Grid, cl: CellList, x, params: Params, rho, which, step=1e-6):
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt).reshape(-1, g.ndims)
    wa = np.ascontiguousarray(which, dtype=np.int64)
    ra = np.ascontiguousarray(rho, dtype=np.float64)
    fd = np.zeros(wa.size, dtype=np.float64)
    fn = _f(dt, "loss_fd")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                   C.POINTER(Params), C.c_void_p, C.c_void_p, C.c_int64, C.c_double,
                   C.c_void_p]
    fn(C.byref(g), _ptr(cl.cells), _ptr(cl.lengths), _ptr(xa), xa.shape[0],
       C.byref(params), _ptr(ra), _ptr(wa), wa.size, float(step), _ptr(fd))
    return fd


# ---------------------------------------------------------------- SpatialHashingCellList


def spatial_hash(cell, list_size: int) -> int:
    """spatial_hash(cell, list_size) - 1 (0-based)."""
    c = (C.c_int64 * 3)(*[int(v) for v in cell], *([0] * (3 - len(cell))))
    fn = lib().pno_spatial_hash
    fn.restype = C.c_int64
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_int64]
    return int(fn(c, len(cell), int(list_size)))


def coordinates_flattened(cell) -> int:
    """coordinates_flattened(cell) as a Python int (raises OracleError where the reference
    throws InexactError)."""
    c = (C.c_int64 * 3)(*[max(min(int(v), 2**63 - 1), -2**63) for v in cell],
                        *([0] * (3 - len(cell))))
    out = (C.c_uint32 * 4)()
    fn = lib().pno_coordinates_flattened
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
    st = fn(c, len(cell), out)
    if st != PNO_OK:
        raise OracleError(st, "coordinates_flattened")
    return sum(int(out[k]) << (32 * k) for k in range(4))


def grid_create_hash(ndims, radius, list_size, periodic_box=None, max_ppc=100,
                     dtype=np.float64) -> Grid:
    """GridNeighborhoodSearch over SpatialHashingCellList{ndims}(; list_size,
    max_points_per_cell)."""
    dt = np.dtype(dtype)
    g = Grid()
    pmn = pmx = None
    if periodic_box is not None:
        pmn = np.ascontiguousarray(periodic_box[0], dtype=dt)
        pmx = np.ascontiguousarray(periodic_box[1], dtype=dt)
    fn = _f(dt, "grid_create_hash")
    ctyp = C.c_float if dt == np.float32 else C.c_double
    fn.argtypes = [C.c_int32, ctyp, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32,
                   C.POINTER(Grid)]
    st = fn(ndims, float(dt.type(radius)), _ptr(pmn), _ptr(pmx), int(list_size), int(max_ppc),
            C.byref(g))
    if st != PNO_OK:
        raise OracleError(st, "grid_create_hash")
    return g


class HashCellList:
    """The reference's SpatialHashingCellList: list_size lists (DynamicVectorOfVectors),
    the flattened coordinates stored per list and the collision flags."""

    def __init__(self, g: Grid):
        self.g = g
        self.cells = np.zeros(g.list_size * g.max_ppc, dtype=np.int32)
        self.lengths = np.zeros(g.list_size, dtype=np.int32)
        self.coords = np.zeros(4 * g.list_size, dtype=np.uint32)
        self.collisions = np.zeros(g.list_size, dtype=np.uint8)

    def __getitem__(self, cell):
        """cell_list[cell]: the points of the cell's hash list (0-based)."""
        h = spatial_hash(cell, self.g.list_size)
        return self.cells[h * self.g.max_ppc: h * self.g.max_ppc + self.lengths[h]]


def hash_build(g: Grid, y, atomic: bool = True) -> HashCellList:
    """initialize! with push_cell_atomic! (ParallelUpdate, atomic=True) or push_cell!
    (SerialUpdate), in point order."""
    dt = np.float32 if g.dtype == 0 else np.float64
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, g.ndims)
    hl = HashCellList(g)
    fn = _f(dt, "hash_build")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_int32]
    st = fn(C.byref(g), _ptr(ya), ya.shape[0], _ptr(hl.cells), _ptr(hl.lengths),
            _ptr(hl.coords), _ptr(hl.collisions), 1 if atomic else 0)
    if st != PNO_OK:
        raise OracleError(st, "hash_build")
    return hl


def hash_neighbor_lists(g: Grid, hl: HashCellList, x, y, n_threads: int = 0):
    """CSR (offsets[n_x+1], nbrs) in the reference's traversal order."""
    dt = np.float32 if g.dtype == 0 else np.float64
    xa = np.ascontiguousarray(x, dtype=dt).reshape(-1, g.ndims)
    ya = np.ascontiguousarray(y, dtype=dt).reshape(-1, g.ndims)
    fn = _f(dt, "hash_neighbor_lists")
    fn.argtypes = [C.POINTER(Grid), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_int32]
    head = (C.byref(g), _ptr(hl.cells), _ptr(hl.lengths), _ptr(hl.coords),
            _ptr(hl.collisions), _ptr(xa), xa.shape[0], _ptr(ya), ya.shape[0])
    return _lists("hash_neighbor_lists", head, g, xa.shape[0], n_threads)

