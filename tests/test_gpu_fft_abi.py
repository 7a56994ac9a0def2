"""kern_fft / kern_ifft on the GPU against the oracle's restatement of the
reference's Halide FFT kernels: within relative L2 1e-12 (FP64), including a
radix-3 size, padded row pitches and the closed-form cases."""
import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


@pytest.mark.parametrize("n", [1024, 3072])
def test_kern_fft_and_kern_ifft_match_the_oracle(n):
    rng = np.random.default_rng(n)
    img = rng.standard_normal((n, n))
    grid = np.zeros((n, n), np.complex128)
    assert compat.call_fft(img, grid) == 0
    assert rel_l2(grid, O.kern_fft(img)) < TOL64
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    out = np.zeros((n, n))
    assert compat.call_ifft(g, out) == 0
    assert rel_l2(out, O.kern_ifft(g)) < TOL64


def test_closed_forms_on_the_gpu():
    n, h = 2048, 1024
    img = np.zeros((n, n))
    img[h, h] = 1.0
    grid = np.zeros((n, n), np.complex128)
    assert compat.call_fft(img, grid) == 0
    exp = np.full((n, n), 1.0 / n, np.complex128)
    exp[0, :] = exp[n - 1, :] = 2.0 / n
    assert np.abs(grid - exp).max() < 1e-15
    out = np.zeros((n, n))
    assert compat.call_ifft(np.ones((n, n), np.complex128), out) == 0
    exp2 = np.zeros((n, n))
    exp2[h, h] = n
    assert np.abs(out - exp2).max() < 1e-9


def test_padded_row_pitches():
    """Buffers whose rows are longer than n (the Halide layouts allow any
    outer stride): only the n x n region is read and written."""
    import ctypes as C

    from rc_gb300 import lib

    n, pad = 1024, 40
    rng = np.random.default_rng(7)
    img_big = rng.standard_normal((n, n + pad))
    grid_big = np.full((n, n + pad), 5.0 + 5.0j)
    ib = compat.buf(img_big, [(n, 1), (n, n + pad)])
    gb = compat.buf(grid_big.view(np.float64), [(2, 1), (n, 2), (n, 2 * (n + pad))])
    L = lib.load()
    assert L.kern_fft(C.byref(ib), C.byref(gb)) == 0
    assert rel_l2(grid_big[:, :n], O.kern_fft(img_big[:, :n])) < TOL64
    assert np.all(grid_big[:, n:] == 5.0 + 5.0j)
    out_big = np.full((n, n + pad), 9.0)
    ob = compat.buf(out_big, [(n, 1), (n, n + pad)])
    assert L.kern_ifft(C.byref(gb), C.byref(ob)) == 0
    assert rel_l2(out_big[:, :n], O.kern_ifft(grid_big[:, :n])) < TOL64
    assert np.all(out_big[:, n:] == 9.0)
