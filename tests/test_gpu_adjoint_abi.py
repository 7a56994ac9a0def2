"""The forward / backward entry points of the C ABI (gb_grid_forward,
gb_grid_backward, gb_degrid_forward, gb_degrid_backward and their _f64
forms), called through ctypes, against the FP64 oracle: grid forward
accumulates G vis into the grid it is given, grid backward writes
G^H grid_grad (the oracle's conj-GCF degridding), degrid forward writes
D grid, degrid backward accumulates G pred_grad.  The dot-product identity
<G x, y> = <x, G^H y> through the forward / backward pair, and a torch
gradcheck of the autograd binding that calls them.  Bars: FP64 1e-12, FP32
1e-5 (relative L2)."""
import numpy as np
import pytest

from tests.conftest import rel_l2
from tests.test_gpu_engine import make_plan, oracle_degrid, oracle_grid, random_case

pytestmark = pytest.mark.gpu

TOL = {"c64": 1e-5, "c128": 1e-12}


def _t(a, dtype):
    import torch

    return torch.tensor(a, dtype=dtype, device="cuda")


@pytest.fixture(scope="module")
def case():
    c = random_case(71, n=4000, G=192, supports=(8, 14, 33))
    c["P"] = make_plan(c)
    return c


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_forward_backward_entries_against_the_oracle(case, prec):
    import torch

    c, P = case, case["P"]
    dt = torch.complex64 if prec == "c64" else torch.complex128
    tol = TOL[prec]
    rng = np.random.default_rng(5)
    G = c["G"]
    g0 = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    y = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    gcf = _t(c["gcf"], dt)
    vis = _t(c["vis"], dt)

    # grid forward: grid += G vis, on a grid that already holds g0
    grid = _t(g0, dt)
    P.grid_forward(gcf, vis, grid)
    exp = oracle_grid(c)
    assert np.abs(exp).max() > 0
    assert rel_l2(grid.cpu().numpy() - g0, exp) < tol

    # grid backward: vis_grad = G^H y (overwrites what the output held)
    out = _t(np.full(c["uvw"].shape[0], 7 + 7j), dt)
    P.grid_backward(gcf, _t(y, dt), out=out)
    exp_v = oracle_degrid(c, y, mode=0)
    assert rel_l2(out.cpu().numpy(), exp_v) < tol
    skipped = c["plane"] < 0
    assert (out.cpu().numpy()[skipped] == 0).all()

    # degrid forward: the same operator under its other name
    pred = P.degrid_forward(gcf, _t(y, dt))
    assert rel_l2(pred.cpu().numpy(), exp_v) < tol

    # degrid backward: grid_grad += G pred_grad
    gg = _t(g0, dt)
    P.degrid_backward(gcf, vis, gg)
    assert rel_l2(gg.cpu().numpy() - g0, exp) < tol

    # dot-product identity through the pair: <G x, y> = <x, G^H y>
    gx = torch.zeros((G, G), dtype=dt, device="cuda")
    P.grid_forward(gcf, vis, gx)
    lhs = complex(torch.vdot(_t(y, dt).flatten(), gx.flatten()))
    rhs = complex(torch.vdot(P.grid_backward(gcf, _t(y, dt)), vis))
    assert abs(lhs - rhs) <= (1e-5 if prec == "c64" else 1e-11) * abs(lhs)


def test_forward_backward_entries_reject_bad_arguments(case):
    from rc_gb300 import lib

    L, P = lib.load(), case["P"]
    for name in ("gb_grid_forward", "gb_grid_backward", "gb_degrid_forward",
                 "gb_degrid_backward"):
        for suffix in ("", "_f64"):
            assert getattr(L, name + suffix)(None, 1, 1, 1, None) == lib.ERR_ARG, name + suffix
    # a NULL output with visibilities to write
    assert L.gb_grid_backward(P.h, 1, 1, None, None) == lib.ERR_ARG
    assert L.gb_degrid_forward_f64(P.h, 1, 1, None, None) == lib.ERR_ARG


def test_autograd_grid_gradcheck():
    """torch.autograd.gradcheck of rc_gb300.autograd.Grid and Degrid (FP64):
    backward through gb_grid_backward / gb_degrid_backward equals the
    finite-difference Jacobian of the forward through gb_grid_forward /
    gb_degrid_forward.  nondet_tol: FP64 atomics add in varying order."""
    import torch

    from rc_gb300.autograd import Degrid, Grid

    c = random_case(72, n=60, G=48, supports=(8, 6))
    P = make_plan(c)
    gcf = _t(c["gcf"], torch.complex128)
    vis = _t(c["vis"], torch.complex128).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda v: Grid.apply(v, P, gcf), (vis,), eps=1e-6,
                                    atol=1e-9, rtol=1e-7, fast_mode=True,
                                    nondet_tol=1e-10)
    grid = _t(np.random.default_rng(3).standard_normal((48, 48)), torch.complex128)
    grid.requires_grad_(True)
    assert torch.autograd.gradcheck(lambda g: Degrid.apply(g, P, gcf), (grid,), eps=1e-6,
                                    atol=1e-9, rtol=1e-7, fast_mode=True,
                                    nondet_tol=1e-10)
