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

    def set_stage(self, stage):
        """Force how FP32 degridding stages grid regions (lib.STAGE_SPLIT,
        STAGE_TMA, STAGE_ROWS) or restore the automatic choice (STAGE_AUTO)."""
        _lib.check(self.L.gb_plan_set_stage(self.h, int(stage)), "gb_plan_set_stage")

    def device_status(self, stream=None):
        """(error, stage) of the last degridding launches: error = 1 when a
        TMA stage did not complete in time (cleared by this call); stage = the
        lib.STAGE_* form the last launch used."""
        out = (C.c_int32 * 2)()
        rc = self.L.gb_plan_device_status(self.h, out, _stream(stream))
        if rc not in (_lib.GB_OK, _lib.ERR_TIMEOUT):
            _lib.check(rc, "gb_plan_device_status")
        return int(out[0]), int(out[1])

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

    # -------------------------------------------------------------- forward / backward
    # gb_grid_forward / _backward and gb_degrid_forward / _backward (and their
    # _f64 forms): complex64 tensors take the FP32 tiled pair, complex128 the
    # plain FP64 pair.
    def _pair(self, name, *ts):
        import torch

        dt = ts[0].dtype
        assert dt in (torch.complex64, torch.complex128)
        assert all(t.dtype == dt and t.is_contiguous() for t in ts)
        assert ts[0].numel() >= self.gcf_len, "GCF array shorter than the plan's layout"
        fn = name if dt == torch.complex64 else name + "_f64"
        return fn, getattr(self.L, fn)

    def grid_forward(self, gcf, vis, grid, stream=None):
        """grid += G vis."""
        assert vis.numel() == self.n and grid.shape == self.grid_shape
        name, fn = self._pair("gb_grid_forward", gcf, vis, grid)
        _lib.check(fn(self.h, gcf.data_ptr(), vis.data_ptr(), grid.data_ptr(), _stream(stream)),
                   name)
        return grid

    def grid_backward(self, gcf, grid_grad, out=None, stream=None):
        """vis_grad = G^H grid_grad (overwrites out)."""
        import torch

        assert grid_grad.shape == self.grid_shape
        if out is None:
            out = torch.empty(self.n, dtype=grid_grad.dtype, device=grid_grad.device)
        name, fn = self._pair("gb_grid_backward", gcf, grid_grad, out)
        _lib.check(fn(self.h, gcf.data_ptr(), grid_grad.data_ptr(), out.data_ptr(),
                      _stream(stream)), name)
        return out

    def degrid_forward(self, gcf, grid, out=None, stream=None):
        """pred = D grid = G^H grid."""
        import torch

        assert grid.shape == self.grid_shape
        if out is None:
            out = torch.empty(self.n, dtype=grid.dtype, device=grid.device)
        name, fn = self._pair("gb_degrid_forward", gcf, grid, out)
        _lib.check(fn(self.h, gcf.data_ptr(), grid.data_ptr(), out.data_ptr(), _stream(stream)),
                   name)
        return out

    def degrid_backward(self, gcf, pred_grad, grid_grad, stream=None):
        """grid_grad += D^H pred_grad = G pred_grad."""
        assert pred_grad.numel() == self.n and grid_grad.shape == self.grid_shape
        name, fn = self._pair("gb_degrid_backward", gcf, pred_grad, grid_grad)
        _lib.check(fn(self.h, gcf.data_ptr(), pred_grad.data_ptr(), grid_grad.data_ptr(),
                      _stream(stream)), name)
        return grid_grad

    def close(self):
        if getattr(self, "h", None):
            self.L.gb_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several grids in one persistent launch (gb_batch_*).

    members: list of dicts with the Plan keyword arguments (uvw, scale,
    grid_size, grid_shape, supports, gcf_offsets, margin, w_range, plane);
    tile/threads/period_cap/bundles_per_cta apply to all.  The GCF array is
    shared: every member's gcf_offsets index into the one passed to grid()."""

    def __init__(self, members, *, tile=0, threads=0, period_cap=0, bundles_per_cta=0,
                 stream=None):
        import torch

        self.L = _lib.load()
        n = len(members)
        assert 1 <= n <= _lib.MAX_BATCH
        arr = (_lib.BatchMember * n)()
        self._keep = []
        self.shapes, self.ns, self.gcf_len = [], [], 0
        for i, m in enumerate(members):
            uvw = m["uvw"]
            assert uvw.is_cuda and uvw.dtype == torch.float64 and uvw.stride(1) == 1
            sup = np.ascontiguousarray(m["supports"], np.int32)
            offs = m.get("gcf_offsets")
            if offs is None:
                offs, total = layout(sup)
            else:
                total = int(max(o + 64 * s * s for o, s in zip(offs, sup)))
            offs = np.ascontiguousarray(offs, np.int64)
            self.gcf_len = max(self.gcf_len, total)
            H, W = m["grid_shape"]
            g = arr[i].geo
            g.scale = float(m["scale"])
            g.grid_size = int(m["grid_size"])
            g.margin = int(sup.max() if m.get("margin") is None else m["margin"])
            g.ext_x, g.ext_y, g.pitch = W, H, W
            g.n_planes = len(sup)
            g.tile, g.threads, g.period_cap = tile, threads, period_cap
            g.bundles_per_cta = bundles_per_cta
            g.supports = sup.ctypes.data_as(C.POINTER(C.c_int32))
            g.gcf_offsets = offs.ctypes.data_as(C.POINTER(C.c_int64))
            lo, hi = m.get("w_range") or (-np.inf, np.inf)
            g.w_low, g.w_high = float(lo), float(hi)
            arr[i].n_vis = uvw.shape[0]
            arr[i].d_uvw = uvw.data_ptr()
            arr[i].uvw_stride = uvw.stride(0)
            arr[i].d_plane = _ptr(m.get("plane"))
            self._keep += [uvw, sup, offs, m.get("plane")]
            self.shapes.append((H, W))
            self.ns.append(uvw.shape[0])
        h = C.c_void_p()
        _lib.check(self.L.gb_batch_create(n, arr, _stream(stream), C.byref(h)), "gb_batch_create")
        self.h = h
        self.n = n

    def stats(self):
        st = (C.c_int64 * 7)()
        _lib.check(self.L.gb_batch_stats(self.h, st), "gb_batch_stats")
        return dict(zip(["kept", "taps", "items", "bundles", "tile", "members", "threads"],
                        list(st)))

    def _ptrs(self, ts):
        return (C.c_void_p * self.n)(*[t.data_ptr() for t in ts])

    def grid(self, vis_list, gcf, grids, stream=None):
        assert len(vis_list) == self.n and len(grids) == self.n
        assert gcf.numel() >= self.gcf_len
        for v, g, shp, nv in zip(vis_list, grids, self.shapes, self.ns):
            assert v.numel() == nv and tuple(g.shape) == shp and g.is_contiguous()
        _lib.check(self.L.gb_batch_grid_f32(self.h, self._ptrs(vis_list), gcf.data_ptr(),
                                            self._ptrs(grids), _stream(stream)),
                   "gb_batch_grid_f32")
        return grids

    def degrid(self, gcf, grids, preds=None, mode=0, stream=None):
        import torch

        assert len(grids) == self.n and gcf.numel() >= self.gcf_len
        if preds is None:
            preds = [torch.empty(nv, dtype=torch.complex64, device=gcf.device) for nv in self.ns]
        _lib.check(self.L.gb_batch_degrid_f32(self.h, gcf.data_ptr(), self._ptrs(grids),
                                              self._ptrs(preds), int(mode), _stream(stream)),
                   "gb_batch_degrid_f32")
        return preds

    def grid64(self, vis_list, gcf, grids, stream=None):
        _lib.check(self.L.gb_batch_grid_f64(self.h, self._ptrs(vis_list), gcf.data_ptr(),
                                            self._ptrs(grids), _stream(stream)),
                   "gb_batch_grid_f64")
        return grids

    def degrid64(self, gcf, grids, preds, mode=0, stream=None):
        _lib.check(self.L.gb_batch_degrid_f64(self.h, gcf.data_ptr(), self._ptrs(grids),
                                              self._ptrs(preds), int(mode), _stream(stream)),
                   "gb_batch_degrid_f64")
        return preds

    def close(self):
        if getattr(self, "h", None):
            self.L.gb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
