"""The adjoint form (AdjointLossForward / AdjointLossBackward and the torch.autograd
Function `adjoint_loss`) against the FP64 oracle's loss and gradient and its central finite
differences, through the C ABI.

Loss: L = sum_i (rho_i - 1)^2 + lambda E, Wendland C2 density (h = 1.5, m = 1), truncated
1/r potential E = 1/2 sum_i sum_{j != i, 0 < d < 3} (1/d - 1/3), lambda = 0.01, over the
neighbour pairs of the search (r = 3), held fixed.

Tolerances: FP64 loss and density within 1e-12 relative, FP64 gradient within 1e-10 of
max |dL/dx|, FP32 gradient within 1e-4 of max |dL/dx| (against the FP64 oracle on the same
FP32 coordinates), finite differences (step 1e-6, FP64) within 1e-6 of max |dL/dx|."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

CONSTS = dict(mass=1.0, h=1.5, cutoff=3.0, lambda_pot=0.01)


@pytest.fixture(scope="module")
def P(pkg):
    import __graft_entry__
    __graft_entry__.build()
    return pkg


def _cloud(P, side, dt, seed=4):
    x = P.workloads.perturbed_lattice((side,) * 3, 0.25, seed=seed, dtype=dt)
    return x, [-1.0] * 3, [side + 1.0] * 3


def _nhs(P, dt, lo, hi, n):
    T = dt
    cl = P.FullGridCellList(min_corner=np.asarray(lo, T), max_corner=np.asarray(hi, T),
                            search_radius=T(3.0), max_points_per_cell=0)
    return P.GridNeighborhoodSearch(3, search_radius=T(3.0), n_points=n, cell_list=cl)


def _gpu_loss_grad(P, x, nhs, dt):
    tdt = torch.float32 if dt == np.float32 else torch.float64
    n = len(x)
    xd = torch.as_tensor(x, device="cuda").T
    P.initialize(nhs, xd, xd)
    rho = torch.empty(n, dtype=tdt, device="cuda")
    terms = torch.empty(n, dtype=tdt, device="cuda")
    loss = torch.empty(1, dtype=torch.float64, device="cuda")
    P.foreach_point_neighbor(P.AdjointLossForward(density=rho, terms=terms, loss=loss, **CONSTS),
                             xd, xd, nhs)
    grad = torch.empty(3 * n, dtype=tdt, device="cuda")
    P.foreach_point_neighbor(P.AdjointLossBackward(grad=grad, reuse_state=True, **CONSTS),
                             xd, xd, nhs)
    grad2 = torch.empty(3 * n, dtype=tdt, device="cuda")
    P.foreach_point_neighbor(P.AdjointLossBackward(density=rho, grad=grad2, **CONSTS),
                             xd, xd, nhs)
    assert torch.equal(grad, grad2)  # state kept by the forward == state rebuilt from rho
    return (float(loss.item()), rho.cpu().numpy().astype(np.float64),
            grad.cpu().numpy().astype(np.float64).reshape(n, 3))


def _oracle(O, x, lo, hi, dt):
    g = O.grid_create(3, dt(3.0), np.asarray(lo, dt), np.asarray(hi, dt), dtype=dt)
    cl = O.build(g, x)
    prm, keep = O.make_params(**CONSTS)
    loss, rho, gr = O.loss_grad(g, cl, x, prm)
    return g, cl, prm, keep, loss, rho, gr


def test_adjoint_fp64_vs_oracle_and_finite_differences(P, O):
    x, lo, hi = _cloud(P, 20, np.float64)
    nhs = _nhs(P, np.float64, lo, hi, len(x))
    loss, rho, grad = _gpu_loss_grad(P, x, nhs, np.float64)
    g, cl, prm, keep, oloss, orho, ogr = _oracle(O, x, lo, hi, np.float64)
    assert abs(loss - oloss) <= 1e-12 * abs(oloss)
    assert np.max(np.abs(rho - orho) / np.abs(orho)) < 1e-12
    scale = np.abs(ogr).max()
    assert np.abs(grad - ogr).max() <= 1e-10 * scale
    # central finite differences of the loss (neighbour set fixed) on 200 coordinates
    rng = np.random.default_rng(9)
    which = rng.choice(x.size, 200, replace=False)
    fd = O.loss_fd(g, cl, x, prm, orho, which, step=1e-6)
    assert np.abs(fd - grad.reshape(-1)[which]).max() <= 1e-6 * scale


def test_adjoint_fp32_vs_fp64_oracle(P, O):
    x, lo, hi = _cloud(P, 24, np.float32, seed=5)
    nhs = _nhs(P, np.float32, lo, hi, len(x))
    loss, rho, grad = _gpu_loss_grad(P, x, nhs, np.float32)
    _, _, _, _, oloss, orho, ogr = _oracle(O, x, lo, hi, np.float32)
    assert abs(loss - oloss) <= 1e-4 * abs(oloss)
    assert np.max(np.abs(rho - orho) / np.abs(orho)) < 1e-5
    assert np.abs(grad - ogr).max() <= 1e-4 * np.abs(ogr).max()


def test_adjoint_loss_autograd(P, O):
    x, lo, hi = _cloud(P, 12, np.float64, seed=6)
    nhs = _nhs(P, np.float64, lo, hi, len(x))
    xt = torch.as_tensor(x, device="cuda").T
    P.initialize(nhs, xt, xt)
    xg = xt.detach().clone().requires_grad_(True)
    L = P.adjoint_loss(xg, nhs, **CONSTS)
    (3.0 * L).backward()
    _, _, _, _, oloss, _, ogr = _oracle(O, x, lo, hi, np.float64)
    assert abs(float(L.detach()) - oloss) <= 1e-12 * abs(oloss)
    got = xg.grad.T.cpu().numpy()
    assert np.abs(got - 3.0 * ogr).max() <= 1e-10 * np.abs(3.0 * ogr).max()
    # a search re-binned elsewhere between forward and backward is re-binned at the
    # forward's positions by the backward pass
    first = got.copy()
    xg.grad = None
    L2 = P.adjoint_loss(xg, nhs, **CONSTS)
    P.update(nhs, xt + 0.1, xt + 0.1)
    (3.0 * L2).backward()
    assert np.array_equal(xg.grad.T.cpu().numpy(), first)


def test_adjoint_gradcheck_small(P):
    x, lo, hi = _cloud(P, 4, np.float64, seed=8)
    nhs = _nhs(P, np.float64, lo, hi, len(x))
    xt = torch.as_tensor(x, device="cuda").T
    P.initialize(nhs, xt, xt)
    xg = xt.detach().clone().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda a: P.adjoint_loss(a, nhs, **CONSTS), (xg,),
                                    eps=1e-6, atol=1e-6, rtol=1e-5)
