"""Imaging major cycle on one GPU (the reference's continuum pipeline,
MS6/programs/continuum.hs:213-298: grid the residual visibilities, FFT,
Hogbom minor loop, degrid the model, subtract), built from the C-ABI pieces:

    psf      = A^H A delta / peak                   (response to a unit source at the centre)
    repeat n_major:
      dirty  = A^H r / peak                         (gb_grid_f32 + gb_grid_to_image_f32)
      model += CLEAN(dirty, psf)                    (gb_hogbom_f32, n_minor iterations)
      r      = v - A model                          (gb_image_to_grid_f32 + gb_degrid_f32)

with A x = D F(x / t) the forward model (grid correction by the taper t, centred
FFT, degridding D = G^H).  torch holds device memory and runs the vector
subtraction; every transform is one call into librc_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import lib as _lib
from .autograd import ImageToGrid, grid_to_image


class MajorCycle:
    def __init__(self, plan, gcf32, taper_img, psf_half=None, window=0.5):
        """plan: engine.Plan of the observation; gcf32: its complex64 GCFs;
        taper_img: float32 (n,) image-domain taper; psf_half: half-size of the
        PSF patch CLEAN subtracts (default n/4); window: CLEAN searches and
        places components only in the central window*n square, where the grid
        correction 1/t is well conditioned (towards the field edge it grows
        to ~1/t(1)^2 and would make edge artefacts the brightest pixels)."""
        self.L = _lib.load()
        self.plan = plan
        self.gcf = gcf32
        self.n = plan.grid_shape[0]
        assert plan.grid_shape == (self.n, self.n)
        self.t = taper_img.float().contiguous()
        self.h = psf_half or self.n // 4
        self.q = int(round(self.n * (1.0 - window) / 2))
        self.nw = self.n - 2 * self.q
        dev = gcf32.device
        self.grid = torch.zeros((self.n, self.n), dtype=torch.complex64, device=dev)
        wb = C.c_int64()
        _lib.check(self.L.gb_hogbom_work_bytes(self.nw, self.nw, C.byref(wb)),
                   "gb_hogbom_work_bytes")
        self.work = torch.empty(wb.value, dtype=torch.uint8, device=dev)
        self.work_bytes = wb.value
        self._psf()

    def _adjoint(self, vis):
        self.grid.zero_()
        self.plan.grid(vis, self.gcf, self.grid)
        return grid_to_image(self.grid, self.t)

    def _psf(self):
        # the response A^H A delta to a unit source at the centre (this carries
        # the degridding kernel's own gain, which A^H 1 would miss)
        c = self.n // 2
        delta = torch.zeros((self.n, self.n), dtype=torch.float32, device=self.gcf.device)
        delta[c, c] = 1.0
        img = self._adjoint(self.forward(delta))
        self.peak = float(img[c, c])
        h = self.h
        self.psf = (img[c - h:c + h, c - h:c + h] / self.peak).contiguous()

    def forward(self, model):
        """Model visibilities A x."""
        with torch.no_grad():
            return self.plan.degrid(self.gcf, ImageToGrid.apply(model, self.t))

    def run(self, vis, n_major=5, n_minor=1000, gain=0.1, threshold=0.0, log=None):
        """Returns (model image, residual visibilities, per-cycle stats)."""
        dev = vis.device
        q, nw = self.q, self.nw
        model = torch.zeros((self.n, self.n), dtype=torch.float32, device=dev)
        mwin = torch.zeros((nw, nw), dtype=torch.float32, device=dev)
        resid = vis.clone()
        stats = []
        s = torch.cuda.current_stream().cuda_stream
        for cyc in range(n_major):
            dirty = (self._adjoint(resid)[q:q + nw, q:q + nw] / self.peak).contiguous()
            _lib.check(self.L.gb_hogbom_f32(dirty.data_ptr(), nw, nw,
                                            self.psf.data_ptr(), 2 * self.h, 2 * self.h, self.h,
                                            self.h, float(gain), float(threshold), int(n_minor),
                                            mwin.data_ptr(), self.work.data_ptr(),
                                            self.work_bytes, s), "gb_hogbom_f32")
            model[q:q + nw, q:q + nw] = mwin
            resid = vis - self.forward(model)
            it = C.c_int32()
            _lib.check(self.L.gb_hogbom_iterations(self.work.data_ptr(), C.byref(it), s),
                       "gb_hogbom_iterations")
            rms = float(torch.sqrt(torch.mean(resid.real ** 2 + resid.imag ** 2)))
            stats.append({"cycle": cyc, "minor_iterations": it.value, "residual_rms": rms})
            if log:
                log(stats[-1])
        return model, resid, stats
