"""torch.autograd test binding of the least-squares imaging model, over the C ABI.

    grid = ImageToGrid.apply(image, taper)        # grid correction + centred FFT
    vis  = Degrid.apply(grid, plan, gcf)          # D = G^H (tiled FP32 or plain FP64)
    grid = Grid.apply(vis, plan, gcf)             # G (the adjoint direction)

Backward passes are the hand-written adjoints, through the C ABI's
forward / backward entry points: Degrid's is the gridding kernel (G,
gb_degrid_backward), Grid's the degridding kernel (D, gb_grid_backward),
ImageToGrid's is gb_grid_to_image (Re[C^-1 S F^H S]).  complex64
tensors run the FP32 tiled pair, complex128 the plain FP64 pair.  torch is
used for device memory, streams and autograd bookkeeping only.
"""
from __future__ import annotations

import torch

from . import lib as _lib


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else t.data_ptr()


class ImageToGrid(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, taper):
        L = _lib.load()
        image = image.contiguous()
        n = image.shape[-1]
        assert image.shape == (n, n) and image.is_cuda
        if image.dtype == torch.float32:
            grid = torch.empty((n, n), dtype=torch.complex64, device=image.device)
            fn = L.gb_image_to_grid_f32
        elif image.dtype == torch.float64:
            grid = torch.empty((n, n), dtype=torch.complex128, device=image.device)
            fn = L.gb_image_to_grid_f64
        else:
            raise TypeError("image must be float32 or float64")
        if taper is not None:
            taper = taper.to(image.dtype).contiguous()
        _lib.check(fn(image.data_ptr(), _ptr(taper), n, grid.data_ptr(), _stream()),
                   "gb_image_to_grid")
        ctx.save_for_backward(taper if taper is not None else torch.empty(0))
        ctx.has_taper = taper is not None
        ctx.n = n
        return grid

    @staticmethod
    def backward(ctx, g):
        return grid_to_image(g, ctx.saved_tensors[0] if ctx.has_taper else None), None


def grid_to_image(grid, taper=None):
    """The adjoint transform (dirty image of a grid, divided by the taper)."""
    L = _lib.load()
    g = grid.contiguous()
    n = g.shape[-1]
    if g.dtype == torch.complex64:
        real, fn = torch.float32, L.gb_grid_to_image_f32
    else:
        real, fn = torch.float64, L.gb_grid_to_image_f64
    out = torch.empty((n, n), dtype=real, device=g.device)
    work = torch.empty_like(g)
    t = taper.to(real).contiguous() if taper is not None else None
    _lib.check(fn(g.data_ptr(), _ptr(t), n, work.data_ptr(), out.data_ptr(), _stream()),
               "gb_grid_to_image")
    return out


class Degrid(torch.autograd.Function):
    """pred = D grid through gb_degrid_forward; backward through
    gb_degrid_backward (the gridding kernel, G = D^H)."""

    @staticmethod
    def forward(ctx, grid, plan, gcf):
        grid = grid.contiguous()
        pred = plan.degrid_forward(gcf, grid)
        ctx.plan, ctx.gcf, ctx.shape, ctx.dtype = plan, gcf, grid.shape, grid.dtype
        return pred

    @staticmethod
    def backward(ctx, gp):
        gp = gp.to(ctx.dtype).contiguous()
        out = torch.zeros(ctx.shape, dtype=ctx.dtype, device=gp.device)
        ctx.plan.degrid_backward(ctx.gcf, gp, out)
        return out, None, None


class Grid(torch.autograd.Function):
    """grid = G vis through gb_grid_forward (into a zeroed grid); backward
    through gb_grid_backward (the degridding kernel, D = G^H)."""

    @staticmethod
    def forward(ctx, vis, plan, gcf):
        vis = vis.contiguous()
        grid = torch.zeros(plan.grid_shape, dtype=vis.dtype, device=vis.device)
        plan.grid_forward(gcf, vis, grid)
        ctx.plan, ctx.gcf, ctx.dtype = plan, gcf, vis.dtype
        return grid

    @staticmethod
    def backward(ctx, gg):
        gg = gg.to(ctx.dtype).contiguous()
        return ctx.plan.grid_backward(ctx.gcf, gg), None, None


def forward_model(image, taper, plan, gcf):
    """Predicted visibilities of a real sky image."""
    return Degrid.apply(ImageToGrid.apply(image, taper), plan, gcf)
