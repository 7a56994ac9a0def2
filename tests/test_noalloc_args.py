"""gb_grid_f32_noalloc's argument and capacity checks, which return before any
GPU work (so they run without a GPU): a grid more than 32767 tiles wide or
high (work items hold int16 tile indices), more footprint pieces than the
static scratch holds, and more (tile, class) bins than it holds.  The device
pointers are never dereferenced on these paths."""
import ctypes as C

import numpy as np

from rc_gb300 import lib

FAKE = 1 << 20  # a non-NULL stand-in for device pointers the call must not touch


def _geometry(sup, ext_x, ext_y, tile=0, cap=0):
    g = lib.Geometry()
    g.scale = 1.0
    g.grid_size = max(ext_x, ext_y)
    g.margin = int(max(sup))
    g.ext_x, g.ext_y, g.pitch = ext_x, ext_y, ext_x
    g.n_planes = len(sup)
    g.tile, g.threads, g.period_cap, g.bundles_per_cta = tile, 0, cap, 0
    g._sup = np.ascontiguousarray(sup, np.int32)
    g._offs = np.ascontiguousarray(np.cumsum([0] + [64 * s * s for s in sup[:-1]]), np.int64)
    g.supports = g._sup.ctypes.data_as(C.POINTER(C.c_int32))
    g.gcf_offsets = g._offs.ctypes.data_as(C.POINTER(C.c_int64))
    g.w_low, g.w_high = -np.inf, np.inf
    return g


def _call(g, n):
    L = lib.load()
    return L.gb_grid_f32_noalloc(C.byref(g), n, FAKE, 3, None, FAKE, FAKE, FAKE, None)


def test_rejects_a_grid_wider_than_32767_tiles():
    L = lib.load()
    g = _geometry([8], 524288, 8, tile=8)  # 65536 tiles of 8 pixels across
    assert _call(g, 100) == lib.ERR_ARG
    assert b"32767 tiles" in L.gb_last_error()
    g = _geometry([8], 8, 32767 * 8 + 1, tile=8)
    assert _call(g, 100) == lib.ERR_ARG


def test_rejects_more_pieces_than_the_scratch_holds():
    L = lib.load()
    # support 16 at period cap 8: 2 x 2 pieces per visibility (small classes,
    # so the shared-memory check passes whatever the device)
    n = lib.NOALLOC_MAX_PIECES // 4 + 1
    assert n <= lib.NOALLOC_MAX_VIS
    g = _geometry([16], 256, 256, tile=8, cap=8)
    assert _call(g, n) == lib.ERR_CAPACITY
    assert b"allocation-free limits" in L.gb_last_error()


def test_rejects_more_bins_than_the_scratch_holds():
    L = lib.load()
    # 4096^2 in tiles of 8: 262144 tiles, one class
    g = _geometry([8], 4096, 4096, tile=8)
    assert _call(g, 1000) == lib.ERR_CAPACITY
    assert b"tile bins" in L.gb_last_error()


def test_rejects_too_many_visibilities_or_planes():
    g = _geometry([8], 256, 256)
    assert _call(g, lib.NOALLOC_MAX_VIS + 1) == lib.ERR_CAPACITY
    g = _geometry([8] * (lib.NOALLOC_MAX_PLANES + 1), 256, 256)
    assert _call(g, 10) == lib.ERR_CAPACITY
