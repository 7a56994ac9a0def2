"""The MS5 binding variant (librc_gb300_ms5.so, -DGB_MS5_ABI) without a GPU:
it builds, exports the same symbols as the MS6 library, and its two MS5-only
bindings check their arguments the way MS5's generated kernels fix them
(MS5/kernel/cpu/gridding/scatter.cpp:9-31: GCF size 16; fft.cpp:540-605:
2048 x 2048) before any GPU work."""
import ctypes as C
import subprocess

import numpy as np

from rc_gb300 import compat, lib


def exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_ms5_library_exports_the_same_symbols():
    L5 = lib.load_ms5()
    L6 = lib.load()
    assert exports(L5._name) == exports(L6._name)
    for name in lib.MS5_SIGNATURES:
        assert hasattr(L5, name)


def test_ms5_kern_scatter_takes_no_margin_and_only_gcf_size_16():
    L5 = lib.load_ms5()
    vis5 = np.zeros((4, 5))
    grid = np.zeros((64, 64), np.complex128)
    for S in (8, 32):
        gcf = np.zeros((64, S, S), np.complex128)
        rc = L5.kern_scatter(1.0, 64, C.byref(compat.vis_buf(vis5)), C.byref(compat.gcf_buf(gcf)),
                             C.byref(compat.grid_buf(grid)))
        assert rc == lib.ERR_ARG
    assert L5.kern_scatter(1.0, 64, None, None, None) == lib.ERR_ARG


def test_ms5_kern_fft_is_grid_to_image_at_2048_only():
    L5 = lib.load_ms5()
    n = 1024
    grid = np.zeros((n, n), np.complex128)
    img = np.zeros((n, n))
    assert L5.kern_fft(C.byref(compat.grid_buf(grid)), C.byref(compat.image_buf(img))) == lib.ERR_ARG
    # the MS6 argument order (image first) is a malformed grid here
    img2 = np.zeros((2048, 2048))
    grid2 = np.zeros((2048, 2048), np.complex128)
    assert L5.kern_fft(C.byref(compat.image_buf(img2)), C.byref(compat.grid_buf(grid2))) == lib.ERR_ARG
    assert L5.kern_fft(None, None) == lib.ERR_ARG
