"""OSKAR 2.6 visibility files onto the GPU.

Python face of include/rc_oskar.h, mirroring the reference's Haskell reader
(MS6/kernel/oskar/OskarReader.hs:45-130: TaskData, readOskarData,
readOskarDataHeader, tdVisibilityPtr / tdUVWPtr) and the pipeline kernel that
turns it into 5-double visibility records (MS6/programs/Kernel/IO.hs:22-74).
Every step runs in librc_gb300.so; there is no Python or CPU path.

    td = read_oskar_data("obs.vis")            # device arrays, CRC-checked
    rec = oskar_reader(td, freq=0, pol=0)      # (n, 5) float64 records on the GPU
    uvw, vis = extract(td, freq=0, pol=0)      # gridding-engine inputs (c64)
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import lib as _lib


@dataclass
class TaskData:
    """OskarReader.hs:45-54.  visibilities: (points, 4) complex128 in
    [baseline][time][channel] order; uvws: (points, 3) float64 wavelengths."""
    baselines: int
    times: int
    channels: int
    points: int
    metrix: dict | None
    bl_minmax: np.ndarray | None       # (baselines, 2): max w, min w
    visibilities: torch.Tensor | None
    uvws: torch.Tensor | None
    header: _lib.VisData

    def visibility_index(self, bl, t, ch):
        """Row of (baseline, time, channel) (tdVisibilityPtr, OskarReader.hs:64-71)."""
        return ch + self.channels * (t + self.times * bl)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _open(path) -> _lib.VisData:
    L = _lib.load()
    vd = _lib.VisData()
    _lib.check(L.mkFromFile(C.byref(vd), os.fsencode(os.fspath(path))), f"mkFromFile({path})")
    return vd


def read_oskar_data_header(path) -> TaskData:
    """Counts only (readOskarDataHeader, OskarReader.hs:98-99)."""
    L = _lib.load()
    vd = _open(path)
    L.freeBinHandler(C.byref(vd))
    return TaskData(vd.num_baselines, vd.num_times, vd.num_channels, vd.num_points, None, None,
                    None, None, vd)


def read_oskar_data(path, device=None) -> TaskData:
    """readOskarData (OskarReader.hs:95-130) with the arrays left on the GPU."""
    L = _lib.load()
    dev = torch.device(device or "cuda")
    vd = _open(path)
    try:
        P, B = vd.num_points, vd.num_baselines
        vis = torch.empty((P, 4), dtype=torch.complex128, device=dev)
        uvw = torch.empty((P, 3), dtype=torch.float64, device=dev)
        mx = _lib.Metrix()
        blw = (_lib.WMaxMin * max(B, 1))()
        with torch.cuda.device(dev):
            _lib.check(L.gb_oskar_read_device(C.byref(vd), vis.data_ptr(), uvw.data_ptr(),
                                              C.byref(mx), blw, _stream()),
                       f"gb_oskar_read_device({path})")
    finally:
        L.freeBinHandler(C.byref(vd))
    metrix = {n: getattr(mx, n) for n, _ in _lib.Metrix._fields_}
    bl = np.frombuffer(blw, np.float64).reshape(-1, 2)[:B].copy()
    return TaskData(B, vd.num_times, vd.num_channels, P, metrix, bl, vis, uvw, vd)


def read_and_reshuffle(path):
    """The reference ABI (mkFromFile + readAndReshuffle) into host arrays:
    (VisData, amps (P, 4) complex128, uvws (P, 3), Metrix, (B, 2) w extrema)."""
    L = _lib.load()
    vd = _open(path)
    try:
        P, B = vd.num_points, vd.num_baselines
        amps = np.empty((P, 4), np.complex128)
        uvw = np.empty((P, 3), np.float64)
        mx = _lib.Metrix()
        blw = (_lib.WMaxMin * max(B, 1))()
        _lib.check(L.readAndReshuffle(C.byref(vd), amps.ctypes.data, uvw.ctypes.data,
                                      C.byref(mx), blw), f"readAndReshuffle({path})")
    finally:
        L.freeBinHandler(C.byref(vd))
    return vd, amps, uvw, mx, np.frombuffer(blw, np.float64).reshape(-1, 2)[:B].copy()


def oskar_reader(td: TaskData, freq=0, pol=0, dom_low=0, dom_high=None,
                 reference_uvw_index=False) -> torch.Tensor:
    """(n, 5) float64 records u, v, w, re, im of points [dom_low, dom_high)
    (baseline-major) for one channel and polarisation (IO.hs:22-74)."""
    L = _lib.load()
    hi = td.baselines * td.times if dom_high is None else dom_high
    out = torch.empty((max(hi - dom_low, 0), 5), dtype=torch.float64,
                      device=td.visibilities.device)
    with torch.cuda.device(out.device):
        _lib.check(L.gb_oskar_records(C.byref(td.header), td.visibilities.data_ptr(),
                                      td.uvws.data_ptr(), freq, pol, dom_low, hi,
                                      _lib.OSKAR_REFERENCE_UVW_INDEX if reference_uvw_index
                                      else 0, out.data_ptr(), _stream()), "gb_oskar_records")
    return out


def extract(td: TaskData, freq=0, pol=0, f64=False):
    """(uvw (n, 3) float64, vis (n,) complex64/complex128) of one channel and
    polarisation, baseline-major: the gridding engine's inputs."""
    L = _lib.load()
    n = td.baselines * td.times
    dev = td.visibilities.device
    uvw = torch.empty((n, 3), dtype=torch.float64, device=dev)
    vis = torch.empty(n, dtype=torch.complex128 if f64 else torch.complex64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(L.gb_oskar_extract(C.byref(td.header), td.visibilities.data_ptr(),
                                      td.uvws.data_ptr(), freq, pol, uvw.data_ptr(),
                                      vis.data_ptr(), int(f64), _stream()), "gb_oskar_extract")
    return uvw, vis


def crc32c(t: torch.Tensor, code: int = 0xFFFFFFFF) -> int:
    """CRC-32C of a device tensor's bytes (16-byte aligned), computed on the GPU."""
    L = _lib.load()
    out = C.c_uint32()
    with torch.cuda.device(t.device):
        _lib.check(L.gb_crc32c_device(t.data_ptr(), t.numel() * t.element_size(), code,
                                      C.byref(out), _stream()), "gb_crc32c_device")
    return out.value
