"""The MS5 binding variant (librc_gb300_ms5.so) on the GPU against the oracle.

MS5's kern_scatter (MS5/kernel/cpu/gridding/scatter.cpp:10-121) is MS6's
gridder with the GCF size fixed at 16 and the corner bounds min .. min +
extent - 16 - 1, which is the oracle's scatter with margin = support = 16.
MS5's kern_fft (MS5/kernel/cpu/gridding/fft.cpp:540-605) is MS6's kern_ifft
pipeline without the 1/2 of the hermitisation and without the division by n
(the c2r helper is the same definition in both files), so it equals
2 n times the oracle's kern_ifft.  Both within relative L2 1e-12 (FP64)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat, lib
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def scatter5(scale, G, vis5, gcf, grid, mx=0, my=0):
    L5 = lib.load_ms5()
    vb, gb, ub = compat.vis_buf(vis5), compat.gcf_buf(gcf), compat.grid_buf(grid, mx, my)
    return L5.kern_scatter(scale, G, C.byref(vb), C.byref(gb), C.byref(ub))


def vis_case(seed, n, G, spread):
    rng = np.random.default_rng(seed)
    lim = spread * G
    vis5 = np.zeros((n, 5))
    vis5[:, :2] = rng.uniform(-lim, lim, (n, 2))
    vis5[:, 2] = rng.uniform(-5, 5, n)
    vis5[:, 3:] = rng.standard_normal((n, 2))
    vis5[:40, 0] = 1e9  # out of bounds
    vis5[40:80, :2] = np.round(vis5[40:80, :2] * 2) / 2  # ties
    gcf = rng.standard_normal((64, 16, 16)) + 1j * rng.standard_normal((64, 16, 16))
    return vis5, gcf


@pytest.mark.parametrize("G,spread", [(256, 0.49), (512, 0.52)])
def test_ms5_kern_scatter_matches_the_oracle_with_margin_16(G, spread):
    vis5, gcf = vis_case(G, 6000, G, spread)
    grid0 = np.random.default_rng(5).standard_normal((G, G)) * (1 - 0.25j)
    got = grid0.copy()
    assert scatter5(1.0, G, vis5, gcf, got) == 0
    exp = grid0.copy()
    O.scatter(1.0, G, 16, vis5, gcf, exp)
    assert rel_l2(got - grid0, exp - grid0) < TOL64  # accumulates in place
    # the spread puts corners on both sides of the bounds
    inb = O.index(vis5, 1.0, G, 16, 16, 0, 0, G, G)[:, 4]
    assert 0 < inb.sum() < len(vis5) - 40


def test_ms5_kern_scatter_on_a_tile_with_mins():
    vis5, gcf = vis_case(9, 4000, 512, 0.2)
    tile = np.zeros((160, 144), np.complex128)
    mx, my = 200, 180
    assert scatter5(1.0, 512, vis5, gcf, tile, mx, my) == 0
    exp = np.zeros_like(tile)
    O.scatter(1.0, 512, 16, vis5, gcf, exp, mx, my)
    assert np.abs(exp).sum() > 0
    assert rel_l2(tile, exp) < TOL64


def test_ms5_kern_fft_is_2n_times_kern_ifft():
    n = 2048
    rng = np.random.default_rng(11)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    L5 = lib.load_ms5()
    out = np.zeros((n, n))
    assert L5.kern_fft(C.byref(compat.grid_buf(g)), C.byref(compat.image_buf(out))) == 0
    assert rel_l2(out, 2 * n * O.kern_ifft(g)) < TOL64
    # the MS6 symbols the variant shares are unchanged
    out6 = np.zeros((n, n))
    assert L5.kern_ifft(C.byref(compat.grid_buf(g)), C.byref(compat.image_buf(out6))) == 0
    assert rel_l2(out6 * 2 * n, out) < TOL64
