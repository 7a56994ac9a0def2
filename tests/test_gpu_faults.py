"""Host-side fault injection: the library's device allocations are made to
fail on purpose (gb_debug_fail_allocs), one at a time at every allocation of
plan creation, batch creation, GCF generation and a reference-ABI call.  Each
entry point returns GB_ERR_NOMEM with a message, leaves no object behind, and
the library works normally afterwards.  No GPU fault is involved."""
import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat, lib
from tests.conftest import rel_l2
from tests.test_gpu_engine import TOL32, make_plan, oracle_grid, random_case

pytestmark = pytest.mark.gpu


def _each_allocation(fn, limit=64):
    """Fail allocation k (k = 0, 1, ...) of fn() until fn succeeds; returns
    how many allocations failed cleanly and fn's result."""
    L = lib.load()
    fails = 0
    try:
        for k in range(limit):
            assert L.gb_debug_fail_allocs(k, 1) == 0
            try:
                out = fn()
            except lib.GbError as e:
                assert e.code == lib.ERR_NOMEM, e
                assert "injected" in lib.last_error()
                fails += 1
                continue
            return fails, out
        raise AssertionError("fn kept failing")
    finally:
        L.gb_debug_fail_allocs(0, 0)


def test_plan_creation_at_every_allocation():
    import torch

    c = random_case(21, supports=(8, 20, 44))
    fails, P = _each_allocation(lambda: make_plan(c))
    assert fails >= 5
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    grid = torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(c["vis"], dtype=torch.complex64, device="cuda"), d_gcf, grid)
    assert rel_l2(grid.cpu().numpy(), oracle_grid(c)) < TOL32


def test_batch_and_gcf_generation_at_every_allocation():
    import torch

    from rc_gb300 import gcf as G
    from rc_gb300.engine import Batch

    c = random_case(22, supports=(8, 24))
    uvw = torch.tensor(c["uvw"], device="cuda")
    plane = torch.tensor(c["plane"], device="cuda")
    spec = [dict(uvw=uvw, plane=plane, scale=1.0, grid_size=c["G"], grid_shape=(c["G"], c["G"]),
                 supports=c["sup"], gcf_offsets=c["offs"], margin=int(c["sup"].max()))] * 2
    fails, B = _each_allocation(lambda: Batch(spec))
    assert fails >= 5
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    grids = [torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda") for _ in range(2)]
    vis = torch.tensor(c["vis"], dtype=torch.complex64, device="cuda")
    B.grid([vis, vis], d_gcf, grids)
    for g in grids:
        assert rel_l2(g.cpu().numpy(), oracle_grid(c)) < TOL32
    B.close()

    ws, sup = np.array([0.0, 250.0]), np.array([16, 12], np.int32)
    fails, out = _each_allocation(lambda: G.generate(ws, sup, 16, 0.08))
    assert fails >= 1
    g64 = out[0].cpu().numpy()
    offs = out[2]
    for p, (w, S) in enumerate(zip(ws, sup)):
        exp = O.gcf_layers(w, int(S), 16, 0.08).reshape(-1)
        assert rel_l2(g64[offs[p]:offs[p] + 64 * S * S], exp) < 1e-12


def test_reference_abi_call_at_a_failed_staging_allocation():
    L = lib.load()
    rng = np.random.default_rng(23)
    n, G, S = 500, 4096, 16  # a grid larger than any staging buffer so far
    vis5 = np.zeros((n, 5))
    vis5[:, :2] = rng.uniform(-0.4 * G, 0.4 * G, (n, 2))
    vis5[:, 3:] = rng.standard_normal((n, 2))
    gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    grid = np.zeros((G, G), np.complex128)
    assert L.gb_debug_fail_allocs(0, 1) == 0
    try:
        rc = compat.call_scatter("kern_scatter_gpu1", 1.0, G, S, vis5, gcf, grid)
    finally:
        L.gb_debug_fail_allocs(0, 0)
    assert rc == lib.ERR_NOMEM and np.all(grid == 0)
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, G, S, vis5, gcf, grid) == 0
    exp = np.zeros_like(grid)
    O.scatter(1.0, G, S, vis5, gcf, exp)
    assert rel_l2(grid, exp) < 1e-12
