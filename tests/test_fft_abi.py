"""kern_fft / kern_ifft without a GPU: the oracle's restatement of the
reference's Halide FFT kernels (MS6/kernel/cpu/gridding/fft.cpp:546-662) on
closed-form cases derived from those definitions, and the library's size and
buffer checks, which return before any GPU work (fft1.cpp:3-11, 29-57)."""
import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat, lib


@pytest.mark.parametrize("n", [64, 1024])
def test_oracle_kern_fft_of_a_centred_delta(n):
    # delta at (h, h) -> rotated to (0, 0) -> flat spectrum; rows v <= h kept;
    # the two shifted halves overlap on rows 0 and n-1
    h = n // 2
    img = np.zeros((n, n))
    img[h, h] = 1.0
    exp = np.full((n, n), 1.0 / n, np.complex128)
    exp[0, :] = exp[n - 1, :] = 2.0 / n
    assert np.abs(O.kern_fft(img) - exp).max() < 1e-15


@pytest.mark.parametrize("n", [64, 1024])
def test_oracle_kern_ifft_of_a_constant_grid(n):
    # a real constant is its own hermitised form; the inverse DFTs collapse it
    # to n^2 at the origin, rotated to (h, h) and divided by n
    h = n // 2
    exp = np.zeros((n, n))
    exp[h, h] = n
    assert np.abs(O.kern_ifft(np.ones((n, n), np.complex128)) - exp).max() < 1e-9


def test_oracle_transforms_are_linear_and_real():
    rng = np.random.default_rng(3)
    n = 128
    a, b = rng.standard_normal((2, n, n))
    assert np.allclose(O.kern_fft(2 * a - b), 2 * O.kern_fft(a) - O.kern_fft(b), atol=1e-12)
    g, k = rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))
    out = O.kern_ifft(g + 3 * k)
    assert out.dtype == np.float64
    assert np.allclose(out, O.kern_ifft(g) + 3 * O.kern_ifft(k), atol=1e-9)


def test_library_rejects_sizes_and_buffers_before_gpu_work():
    lib.load()
    for n in (512, 1000):
        img = np.zeros((n, n))
        grid = np.zeros((n, n), np.complex128)
        assert compat.call_fft(img, grid) == lib.ERR_FFT_SIZE
        assert compat.call_ifft(grid, img) == lib.ERR_FFT_SIZE
    # image and grid of different sizes
    assert compat.call_fft(np.zeros((1024, 1024)), np.zeros((2048, 2048), np.complex128)) == \
        lib.ERR_FFT_SIZE
    # a malformed grid buffer (elements not interleaved)
    img = np.zeros((1024, 1024))
    d = np.zeros(2 * 1024 * 1024)
    bad = compat.buf(d, [(2, 1024 * 1024), (1024, 1), (1024, 1024)])
    import ctypes as C

    L = lib.load()
    assert L.kern_fft(C.byref(compat.image_buf(img)), C.byref(bad)) == lib.ERR_ARG
    assert L.kern_ifft(C.byref(bad), C.byref(compat.image_buf(img))) == lib.ERR_ARG
    assert L.kern_fft(None, None) == lib.ERR_ARG
