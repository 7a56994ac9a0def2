"""De-tiling and facet rotation (reference ABI and device entries) against
the oracle's restatements of detile.cpp and rotate.cpp."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat, lib
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tile_min", [(96, 200), (-8, -8), (500, 500), (1000, 3)])
def test_kern_detile_adds_the_overlap(tile_min):
    rng = np.random.default_rng(abs(tile_min[0]) + 1)
    tile = rng.standard_normal((80, 72)) + 1j * rng.standard_normal((80, 72))
    grid = rng.standard_normal((512, 512)) + 1j * rng.standard_normal((512, 512))
    exp = O.detile(tile, tile_min, grid, (0, 0))
    got = grid.copy()
    L = lib.load()
    rc = L.kern_detile(C.byref(compat.grid_buf(tile, *tile_min)), C.byref(compat.grid_buf(got)))
    assert rc == 0
    assert np.array_equal(got, exp)


def test_gb_detile_f32_on_device():
    import torch

    rng = np.random.default_rng(3)
    tile = (rng.standard_normal((48, 40)) + 1j * rng.standard_normal((48, 40))).astype(np.complex64)
    grid = (rng.standard_normal((256, 256)) + 1j * rng.standard_normal((256, 256))).astype(np.complex64)
    exp = O.detile(tile, (230, -5), grid, (0, 0))
    d_t = torch.tensor(tile, device="cuda")
    d_g = torch.tensor(grid, device="cuda")
    L = lib.load()
    lib.check(L.gb_detile_f32(d_t.data_ptr(), 40, 230, -5, 40, 48, d_g.data_ptr(), 256, 0, 0, 256,
                              256, torch.cuda.current_stream().cuda_stream), "gb_detile_f32")
    assert np.array_equal(d_g.cpu().numpy(), exp)


@pytest.mark.parametrize("uvproj", [0, 1])
def test_kern_rotate_matches_restatement(uvproj):
    rng = np.random.default_rng(7 + uvproj)
    n = 5000
    vis5 = np.column_stack([rng.uniform(-3e3, 3e3, n), rng.uniform(-3e3, 3e3, n),
                            rng.uniform(-200, 200, n), rng.standard_normal(n),
                            rng.standard_normal(n)])
    in_lon, in_lat = 1.2, -0.52
    lon0, lat0, dlon, dlat = 1.19, -0.53, 1e-4, 2e-4
    lmin, mmin = 37, 55
    out = np.zeros_like(vis5)
    ob = compat.buf(out, [(5, 1), (n, 5), (1, 0), (1, 0)], (0, 0, lmin, mmin))
    L = lib.load()
    rc = L.kern_rotate(in_lon, in_lat, lon0, lat0, dlon, dlat, uvproj,
                       C.byref(compat.vis_buf(vis5)), C.byref(ob))
    assert rc == 0
    exp = O.rotate(in_lon, in_lat, lon0 + lmin * dlon, lat0 + mmin * dlat, uvproj, vis5)
    assert rel_l2(out[:, :3], exp[:, :3]) < 1e-13
    assert rel_l2(out[:, 3:], exp[:, 3:]) < 1e-11
    if not uvproj:
        assert np.array_equal(out[:, :3], vis5[:, :3])
