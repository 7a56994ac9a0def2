"""Python face of the engine API (gb_* in include/rc_gb300.h) on torch CUDA tensors.

    plan = Plan(uvw, scale=..., grid_size=..., grid_shape=(H, W), supports=..., w_range=(lo, hi))
    plan.grid(vis_c64, gcf_c64, grid_c64)          # grid += G vis        (FP32 tiled)
    pred = plan.degrid(gcf_c64, grid_c64)          # pred  = D grid = G^H grid
    plan.grid64(vis_c128, gcf_c128, grid_c128)     # plain FP64 path
    pred64 = plan.degrid64(gcf_c128, grid_c128)

torch is used for device memory and streams only; every operation is one
call into librc_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _lib
from .gcf import layout


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def _ptr(t):
    return None if t is None else t.data_ptr()


class Plan:
    def __init__(self, uvw, *, scale, grid_size, grid_shape, supports, gcf_offsets=None,
                 margin=None, w_range=None, plane=None, tile=0, threads=0, period_cap=0,
                 bundles_per_cta=0, stream=None):
        import torch

        assert uvw.is_cuda and uvw.dtype == torch.float64 and uvw.dim() == 2
        assert uvw.stride(1) == 1 and uvw.shape[1] >= 3
        self.L = _lib.load()
        self.uvw = uvw  # the plan keeps the address: hold the tensor
        self.n = uvw.shape[0]
        self.supports = np.ascontiguousarray(supports, np.int32)
        if gcf_offsets is None:
            gcf_offsets, self.gcf_len = layout(self.supports)
        else:
            self.gcf_len = int(max(o + 64 * s * s for o, s in zip(gcf_offsets, self.supports)))
        self.gcf_offsets = np.ascontiguousarray(gcf_offsets, np.int64)
        H, W = grid_shape
        self.grid_shape = (H, W)
        g = _lib.Geometry()
        g.scale = float(scale)
        g.grid_size = int(grid_size)
        g.margin = int(self.supports.max() if margin is None else margin)
        g.ext_x, g.ext_y, g.pitch = W, H, W
        g.n_planes = len(self.supports)
        g.tile, g.threads, g.period_cap = tile, threads, period_cap
        g.bundles_per_cta = bundles_per_cta
        g.supports = self.supports.ctypes.data_as(C.POINTER(C.c_int32))
        g.gcf_offsets = self.gcf_offsets.ctypes.data_as(C.POINTER(C.c_int64))
        lo, hi = w_range if w_range is not None else (-np.inf, np.inf)
        g.w_low, g.w_high = float(lo), float(hi)
        self.geo = g
        self.plane_in = plane
        h = C.c_void_p()
        _lib.check(self.L.gb_plan_create(C.byref(g), self.n, uvw.data_ptr(), uvw.stride(0),
                                         _ptr(plane), _stream(stream), C.byref(h)),
                   "gb_plan_create")
        self.h = h

    # -------------------------------------------------------------- info
    def stats(self):
        st = (C.c_int64 * 7)()
        _lib.check(self.L.gb_plan_stats(self.h, st), "gb_plan_stats")
        keys = ["kept", "taps", "items", "tiles", "tile", "max_support", "threads"]
        return dict(zip(keys, list(st)))

    def export_index(self, stream=None):
        import torch

        out = torch.empty((self.n, 5), dtype=torch.int32, device=self.uvw.device)
        _lib.check(self.L.gb_plan_export_index(self.h, out.data_ptr(), _stream(stream)),
                   "gb_plan_export_index")
        return out

    # -------------------------------------------------------------- FP32 pair
    def grid(self, vis, gcf, grid, stream=None):
        import torch

        assert vis.dtype == torch.complex64 and gcf.dtype == torch.complex64
        assert grid.dtype == torch.complex64 and grid.is_contiguous()
        assert grid.shape == self.grid_shape and vis.numel() == self.n
        assert gcf.numel() >= self.gcf_len, "GCF array shorter than the plan's layout"
        _lib.check(self.L.gb_grid_f32(self.h, vis.data_ptr(), gcf.data_ptr(), grid.data_ptr(),
                                      _stream(stream)), "gb_grid_f32")
        return grid

    def degrid(self, gcf, grid, out=None, mode=0, stream=None):
        import torch

        assert gcf.dtype == torch.complex64 and grid.dtype == torch.complex64
        assert grid.shape == self.grid_shape and grid.is_contiguous()
        assert gcf.numel() >= self.gcf_len, "GCF array shorter than the plan's layout"
        if out is None:
            out = torch.empty(self.n, dtype=torch.complex64, device=grid.device)
        _lib.check(self.L.gb_degrid_f32(self.h, gcf.data_ptr(), grid.data_ptr(), out.data_ptr(),
                                        int(mode), _stream(stream)), "gb_degrid_f32")
        return out

    # -------------------------------------------------------------- plain FP64
    def grid64(self, vis, gcf, grid, stream=None):
        import torch

        assert vis.dtype == torch.complex128 and gcf.dtype == torch.complex128
        assert grid.dtype == torch.complex128 and grid.is_contiguous()
        assert grid.shape == self.grid_shape and vis.numel() == self.n
        assert gcf.numel() >= self.gcf_len, "GCF array shorter than the plan's layout"
        _lib.check(self.L.gb_grid_f64(self.h, vis.data_ptr(), gcf.data_ptr(), grid.data_ptr(),
                                      _stream(stream)), "gb_grid_f64")
        return grid

    def degrid64(self, gcf, grid, out=None, mode=0, stream=None):
        import torch

        assert gcf.dtype == torch.complex128 and grid.dtype == torch.complex128
        assert grid.shape == self.grid_shape and grid.is_contiguous()
        assert gcf.numel() >= self.gcf_len, "GCF array shorter than the plan's layout"
        if out is None:
            out = torch.empty(self.n, dtype=torch.complex128, device=grid.device)
        _lib.check(self.L.gb_degrid_f64(self.h, gcf.data_ptr(), grid.data_ptr(), out.data_ptr(),
                                        int(mode), _stream(stream)), "gb_degrid_f64")
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.gb_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
