"""The drop-in boundary with a search the reference built: pn_create_from_grid takes a
FullGridCellList's stored state (padded corners, size(linear_indices), the backend's
capacity; full_grid.jl:30-35) as it is, and copy_neighborhood_search pads the template's
stored corners by the new radius like copy_cell_list (full_grid.jl:179-185)."""
import numpy as np
import pytest

from test_gpu_parity import dcoords

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


@pytest.mark.parametrize("d,dtype,periodic", [(3, np.float64, False), (3, np.float32, False),
                                               (2, np.float32, True)])
def test_search_from_stored_cell_list_state(P, O, d, dtype, periodic):
    W = P.workloads
    side = 16
    x = W.perturbed_lattice((side,) * d, 0.25, seed=8, dtype=dtype)
    r = dtype(2.5)
    lo, hi = np.zeros(d, dtype), np.full(d, side + 1.0, dtype)
    if periodic:
        x = (x % dtype(side + 1.0)).astype(dtype)
    box = P.PeriodicBox(min_corner=lo, max_corner=hi) if periodic else None
    ref = P.FullGridCellList(min_corner=lo, max_corner=hi, search_radius=r,
                             max_points_per_cell=64)
    a = P.GridNeighborhoodSearch(d, search_radius=r, n_points=len(x), cell_list=ref,
                                 periodic_box=box)
    # what a Julia binding reads from the reference's structs
    state = P.FullGridCellList.from_state(min_corner=ref.min_corner, max_corner=ref.max_corner,
                                          grid_size=a.grid_info()["grid_size"],
                                          max_points_per_cell=64, search_radius=r)
    b = P.GridNeighborhoodSearch(d, search_radius=r, n_points=len(x), cell_list=state,
                                 periodic_box=box)
    assert a.grid_info() == b.grid_info()
    xd = dcoords(x)
    counts = []
    for s in (a, b):
        P.initialize(s, xd, xd)
        c = torch.zeros(len(x), dtype=torch.int32, device="cuda")
        P.foreach_point_neighbor(P.CountNeighbors(c), xd, xd, s)
        counts.append(c.cpu().numpy())
    ca, pa = P.export_cells(a)
    cb, pb = P.export_cells(b)
    assert np.array_equal(ca, cb) and np.array_equal(pa, pb)
    assert np.array_equal(counts[0], counts[1])
    g = O.grid_create(d, r, lo, hi, dtype=dtype, max_ppc=64,
                      periodic_box=(lo, hi) if periodic else None)
    assert np.array_equal(counts[1], O.foreach(g, O.build(g, x), x, x, O.F_COUNT))


def test_copy_pads_the_stored_corners(P):
    T = np.float64
    lo, hi = np.zeros(3), np.full(3, 10.0)
    tmpl = P.GridNeighborhoodSearch(3, search_radius=0.0, cell_list=P.FullGridCellList(
        min_corner=lo, max_corner=hi, search_radius=0.0))
    full = P.GridNeighborhoodSearch(3, search_radius=1.0, cell_list=P.FullGridCellList(
        min_corner=lo, max_corner=hi, search_radius=1.0))
    pad2 = T(T(1001) / T(1000)) * T(2.0)
    c1 = P.copy_neighborhood_search(tmpl, 2.0, 100)
    assert c1.grid_info()["min_corner"] == tuple(lo - pad2)
    # a search with a radius stores padded corners, which the copy pads again
    c2 = P.copy_neighborhood_search(full, 2.0, 100)
    stored = np.array(full.grid_info()["min_corner"])
    assert c2.grid_info()["min_corner"] == tuple(stored - pad2)
    assert c2.grid_info()["max_corner"] == tuple(np.array(full.grid_info()["max_corner"]) + pad2)
