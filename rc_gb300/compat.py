"""Calling the reference-ABI symbols the way the reference's Haskell marshaller
does (MS6/dna/flow/Flow/Halide/Marshal.hs:233-313): host arrays wrapped in
72-byte buffer_t descriptors, dev = 0, host_dirty = 1.

These helpers build buffer_t's for numpy arrays; the calls themselves go
straight to librc_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _lib


def buf(arr: np.ndarray, dims, mins=(0, 0, 0, 0)) -> _lib.BufferT:
    """buffer_t over a float64 numpy array; dims = [(extent, stride), ...]
    innermost first, strides in elements."""
    assert arr.dtype == np.float64
    b = _lib.BufferT()
    b.dev = 0
    b.host = arr.ctypes.data
    for k in range(4):
        e, s = dims[k] if k < len(dims) else (0, 0)
        b.extent[k] = e
        b.stride[k] = s
        b.min[k] = mins[k] if k < len(mins) else 0
    b.elem_size = 8
    b.host_dirty = True
    b.dev_dirty = False
    return b


def vis_buf(vis5: np.ndarray, vmin=0):
    """(N, 5) doubles: dims (5, N), strides (1, 5) (Kernel/Data.hs:115-123)."""
    assert vis5.flags.c_contiguous and vis5.shape[1] == 5
    return buf(vis5, [(5, 1), (vis5.shape[0], 5), (1, 0), (1, 0)], (0, vmin, 0, 0))


def gcf_buf(gcf: np.ndarray):
    """complex128 [64][S][S] viewed as doubles: dims (2, S, S, 64) (Kernel/Data.hs:125-133)."""
    assert gcf.dtype == np.complex128 and gcf.flags.c_contiguous
    S = gcf.shape[-1]
    d = gcf.view(np.float64)
    return buf(d, [(2, 1), (S, 2), (S, 2 * S), (64, 2 * S * S)])


def grid_buf(grid: np.ndarray, min_x=0, min_y=0):
    """complex128 [H][W] viewed as doubles: dims (2, W, H), strides (1, 2, 2W)."""
    assert grid.dtype == np.complex128 and grid.flags.c_contiguous
    H, W = grid.shape
    d = grid.view(np.float64)
    return buf(d, [(2, 1), (W, 2), (H, 2 * W)], (0, min_x, min_y, 0))


def image_buf(img: np.ndarray):
    """(n, n) doubles, [y][x]: dims (n, n), strides (1, n) (the reference's
    real image buffers, MS6/kernel/cpu/gridding/fft.cpp:609-611)."""
    assert img.flags.c_contiguous and img.ndim == 2
    return buf(img, [(img.shape[1], 1), (img.shape[0], img.shape[1])])


def call_fft(image, grid):
    """kern_fft: real image (n, n) -> complex grid (n, n) in place."""
    L = _lib.load()
    ib, gb = image_buf(image), grid_buf(grid)
    return L.kern_fft(C.byref(ib), C.byref(gb))


def call_ifft(grid, image):
    """kern_ifft: complex grid (n, n) -> real image (n, n) in place."""
    L = _lib.load()
    gb, ib = grid_buf(grid), image_buf(image)
    return L.kern_ifft(C.byref(gb), C.byref(ib))


def call_scatter(name, scale, grid_size, margin, vis5, gcf, grid, min_x=0, min_y=0):
    L = _lib.load()
    vb, gb, ub = vis_buf(vis5), gcf_buf(gcf), grid_buf(grid, min_x, min_y)
    return getattr(L, name)(scale, grid_size, margin, C.byref(vb), C.byref(gb), C.byref(ub))


def call_degrid(name, scale, grid_size, margin, gcf, grid, vis5, out5):
    L = _lib.load()
    gb, ub, vb, ob = gcf_buf(gcf), grid_buf(grid), vis_buf(vis5), vis_buf(out5)
    return getattr(L, name)(scale, grid_size, margin, C.byref(gb), C.byref(ub), C.byref(vb),
                            C.byref(ob))
