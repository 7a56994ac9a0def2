"""Reference-ABI entry points (host buffer_t, synchronous) on the GPU against
the oracle, called the way the reference's Flow.Halide marshaller calls them."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat, lib
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def case(seed, n=4000, G=256, S=16, spread=0.47):
    rng = np.random.default_rng(seed)
    lim = spread * G
    vis5 = np.zeros((n, 5))
    vis5[:, 0] = rng.uniform(-lim, lim, n)
    vis5[:, 1] = rng.uniform(-lim, lim, n)
    vis5[:, 2] = rng.uniform(-5, 5, n)
    vis5[:, 3:] = rng.standard_normal((n, 2))
    vis5[:50, 0] = 1e9  # out of bounds
    vis5[50:100, :2] = np.round(vis5[50:100, :2] * 2) / 2  # ties
    gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    return vis5, gcf


@pytest.mark.parametrize("name", ["kern_scatter_gpu1", "kern_scatter", "nvGridder"])
@pytest.mark.parametrize("S", [8, 16, 32, 64])
def test_scatter_symbols_match_oracle(name, S):
    vis5, gcf = case(10 + S, S=S)
    G = 256
    scale, margin = 1.0, 64
    grid0 = np.random.default_rng(1).standard_normal((G, G)) * (1 + 0.5j)
    got = grid0.copy()
    assert compat.call_scatter(name, scale, G, margin, vis5, gcf, got) == 0
    exp = grid0.copy()
    O.scatter(scale, G, margin, vis5, gcf, exp)
    assert rel_l2(got - grid0, exp - grid0) < TOL64  # accumulates in place


def test_scatter_on_a_margin_tile():
    """A (W+2m) x (H+2m) tile with non-zero mins, as UVGMarginRepr passes it."""
    vis5, gcf = case(3, n=3000, G=512, S=16, spread=0.2)
    G, m = 512, 8
    W = H = 128
    tile = np.zeros((H + 2 * m, W + 2 * m), np.complex128)
    mx, my = 256 - 64 - m, 256 - 32 - m
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, G, 2 * m, vis5, gcf, tile, mx, my) == 0
    exp = np.zeros_like(tile)
    O.scatter(1.0, G, 2 * m, vis5, gcf, exp, mx, my)
    assert np.abs(exp).sum() > 0
    assert rel_l2(tile, exp) < TOL64


@pytest.mark.parametrize("name", ["kern_degrid_gpu1", "kern_degrid"])
@pytest.mark.parametrize("S", [8, 32])
def test_degrid_symbols_match_oracle(name, S):
    vis5, gcf = case(20 + S, S=S)
    G = 256
    grid = np.random.default_rng(2).standard_normal((G, G)) + 1j * np.random.default_rng(
        3).standard_normal((G, G))
    out = np.zeros_like(vis5)
    assert compat.call_degrid(name, 1.0, G, S, gcf, grid, vis5, out) == 0
    exp = O.degrid(1.0, G, S, gcf, grid, vis5)
    assert np.array_equal(out[:, :3], exp[:, :3])
    assert rel_l2(out[:, 3:], exp[:, 3:]) < TOL64
    assert np.array_equal(out[:50], vis5[:50])  # out-of-bound records pass through


def test_legacy_size_codes():
    vis5, gcf = case(4, n=10, S=12)
    grid = np.zeros((64, 64), np.complex128)
    out = np.zeros_like(vis5)
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, 64, 12, vis5, gcf, grid) == -222
    assert compat.call_scatter("kern_scatter", 1.0, 64, 12, vis5, gcf, grid) == -444
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, 64, 12, gcf, grid, vis5, out) == -333
    assert compat.call_degrid("kern_degrid", 1.0, 64, 12, gcf, grid, vis5, out) == -555


def test_malformed_buffers_are_rejected():
    L = lib.load()
    vis5, gcf = case(5, n=10, S=8)
    grid = np.zeros((64, 64), np.complex128)
    vb, gb, ub = compat.vis_buf(vis5), compat.gcf_buf(gcf), compat.grid_buf(grid)
    gb.stride[2] = 3  # not dense
    assert L.kern_scatter_gpu1(1.0, 64, 8, C.byref(vb), C.byref(gb), C.byref(ub)) == lib.ERR_ARG
    assert b"gcf" in L.gb_last_error()
    gb = compat.gcf_buf(gcf)
    vb.extent[0] = 4
    assert L.kern_scatter_gpu1(1.0, 64, 8, C.byref(vb), C.byref(gb), C.byref(ub)) == lib.ERR_ARG
    assert L.kern_scatter_gpu1(1.0, 64, 8, None, C.byref(gb), C.byref(ub)) == lib.ERR_ARG


def test_empty_visibility_buffer():
    vis5 = np.zeros((0, 5))
    gcf = np.ones((64, 8, 8), np.complex128)
    grid = np.full((32, 32), 1 + 1j)
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, 32, 8, vis5, gcf, grid) == 0
    assert np.all(grid == 1 + 1j)


def test_init_and_psf_vis():
    L = lib.load()
    grid = np.full((16, 24), 3 + 4j)
    ub = compat.grid_buf(grid)
    assert L.kern_init(C.byref(ub)) == 0
    assert np.all(grid == 0)
    vis5 = np.arange(50, dtype=np.float64).reshape(10, 5)
    out = np.zeros_like(vis5)
    assert L.kern_psf_vis(C.byref(compat.vis_buf(vis5)), C.byref(compat.vis_buf(out))) == 0
    assert np.array_equal(out[:, :3], vis5[:, :3])
    assert np.all(out[:, 3] == 1.0) and np.all(out[:, 4] == 0.0)


def test_config1_slice_through_the_abi():
    """A slice of the config-1 observation (PSWF 7x7 in S=8) through
    kern_scatter_gpu1 / kern_degrid_gpu1."""
    from rc_gb300 import gcf as G
    from rc_gb300 import synth

    ob = synth.config("c1", n_t=16)
    vis5 = ob.vis5()
    gcf = G.pswf_uv_gcf(8, 7)
    grid = np.zeros((ob.grid_size, ob.grid_size), np.complex128)
    assert compat.call_scatter("kern_scatter_gpu1", ob.scale, ob.grid_size, 8, vis5, gcf, grid) == 0
    exp = np.zeros_like(grid)
    O.scatter(ob.scale, ob.grid_size, 8, vis5, gcf, exp)
    assert rel_l2(grid, exp) < TOL64
    out = np.zeros_like(vis5)
    assert compat.call_degrid("kern_degrid_gpu1", ob.scale, ob.grid_size, 8, gcf, exp, vis5,
                              out) == 0
    ref = O.degrid(ob.scale, ob.grid_size, 8, gcf, exp, vis5)
    assert rel_l2(out[:, 3:], ref[:, 3:]) < TOL64


@pytest.mark.parametrize("S", [8, 64])
def test_degrid_single_and_out_of_bound_records(S):
    """A call with one record (its taps then split over all the block's warps)
    and a call whose records all fall outside the grid (copied through)."""
    _, gcf = case(30 + S, n=10, S=S)
    G = 256
    grid = np.random.default_rng(4).standard_normal((G, G)) * (1 - 2j)
    one = np.array([[3.3, -7.8, 1.0, 0.5, -0.25]])
    out = np.zeros_like(one)
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, G, S, gcf, grid, one, out) == 0
    exp = O.degrid(1.0, G, S, gcf, grid, one)
    assert np.array_equal(out[:, :3], one[:, :3])
    assert rel_l2(out[:, 3:], exp[:, 3:]) < TOL64
    far = np.array([[1e9, 0.0, 0.0, 1.0, 2.0], [0.0, -1e9, 0.0, 3.0, 4.0], [5e8, 5e8, 1.0, 5.0, 6.0]])
    out = np.zeros_like(far)
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, G, S, gcf, grid, far, out) == 0
    assert np.array_equal(out, far)
