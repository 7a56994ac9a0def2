"""Without a GPU the product fails loudly: the reference-ABI entry points
return GB_ERR_CUDA and leave the caller's buffers as they were, and the
engine cannot make a plan.  Nothing is computed on the host instead.  (Run
where no GPU is visible; on a GPU machine the same calls compute, and the
-m gpu tests cover them.)"""
import ctypes as C

import numpy as np
import pytest

from rc_gb300 import compat, lib

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.skipif(torch.cuda.is_available(), reason="a GPU is visible")


def test_abi_calls_return_a_cuda_error():
    L = lib.load()
    vis5 = np.array([[1.0, 2.0, 0.0, 1.0, 0.5]])
    gcf = np.ones((64, 8, 8), np.complex128)
    grid = np.zeros((64, 64), np.complex128)
    for name in ("kern_scatter_gpu1", "kern_scatter", "nvGridder"):
        assert compat.call_scatter(name, 1.0, 64, 8, vis5, gcf, grid) == lib.ERR_CUDA
        assert "CUDA" in lib.last_error() or "cuda" in lib.last_error()
    assert not grid.any()
    out = np.full_like(vis5, 7.0)
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, 64, 8, gcf, grid, vis5, out) == lib.ERR_CUDA
    assert (out == 7.0).all()
    img = np.zeros((1024, 1024))
    assert compat.call_ifft(np.ones((1024, 1024), np.complex128), img) == lib.ERR_CUDA
    assert not img.any()


def test_engine_cannot_plan_without_a_device():
    L = lib.load()
    geo = lib.Geometry()
    geo.scale, geo.grid_size, geo.margin = 1.0, 64, 8
    geo.ext_x = geo.ext_y = geo.pitch = 64
    geo.n_planes = 1
    sup = (C.c_int32 * 1)(8)
    offs = (C.c_int64 * 1)(0)
    geo.supports = C.cast(sup, C.POINTER(C.c_int32))
    geo.gcf_offsets = C.cast(offs, C.POINTER(C.c_int64))
    geo.w_low, geo.w_high = -1.0, 1.0
    h = C.c_void_p()
    # no visibilities and no arrays: valid on a GPU, so nothing here can fault one
    rc = L.gb_plan_create(C.byref(geo), 0, None, 3, None, None, C.byref(h))
    assert rc == lib.ERR_CUDA and not h.value
