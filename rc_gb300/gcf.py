"""GCF (gridding convolution function) helpers.

* layout(): offsets of per-plane GCFs ([64][S][S] complex each, phase
  ou + 8*ov, MS6 layout MS6/kernel/cpu/gridding/scatter.cpp:34-41) in one flat
  array;
* plane_supports(): the w-plane support rule of the synthetic workloads;
* pswf(): prolate spheroidal wave function (order 0) via scipy.special.pro_ang1;
* pswf_uv_gcf(): an oversampled uv-domain PSWF GCF for the no-w-term case;
* generate(): on-GPU w-kernel generation through gb_gcf_generate (FP64 phase
  screens + cuFFT), returning complex128 and/or complex64 device tensors.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import lib as _lib

OVER = 8


def layout(supports):
    """(offsets int64[n_planes], total complex elements)."""
    s = np.asarray(supports, np.int64)
    sizes = 64 * s * s
    offs = np.zeros(len(s), np.int64)
    if len(s) > 1:
        offs[1:] = np.cumsum(sizes)[:-1]
    return offs, int(sizes.sum())


def ceil_even(x):
    return int(2 * math.ceil(x / 2.0))


def plane_supports(w_low, w_high, n_planes, s_min=8, s_max=64):
    """Support of each uniform w-bin over [w_low, w_high]: s_min + (s_max - s_min) *
    sqrt(|w|/w_max) at the bin edge nearest w = 0, rounded up to even, clamped.
    Also returns the bin centres (the w each plane's GCF is generated at)."""
    edges = np.linspace(w_low, w_high, n_planes + 1)
    wmax = max(abs(w_low), abs(w_high), 1e-300)
    sup = []
    for p in range(n_planes):
        a, b = edges[p], edges[p + 1]
        inner = 0.0 if a <= 0.0 <= b else min(abs(a), abs(b))
        s = ceil_even(s_min + (s_max - s_min) * math.sqrt(inner / wmax))
        sup.append(int(min(max(s, s_min), s_max)))
    centres = 0.5 * (edges[:-1] + edges[1:])
    return np.array(sup, np.int32), centres


def pswf(x, c, outside=0.0):
    """Order-0 prolate spheroidal angular function, normalised to 1 at x = 0.
    For |x| >= 1 it is `outside` (0: a kernel's support ends there), or, with
    outside=None, its limit at the interval's edge (a taper sampled on
    [-1, 1) keeps a non-zero first sample, so grid correction can divide)."""
    from scipy.special import pro_ang1

    x = np.asarray(x, np.float64)
    xc = np.clip(x, -1 + 1e-12, 1 - 1e-12)
    v = pro_ang1(0, 0, c, xc)[0] / pro_ang1(0, 0, c, 0.0)[0]
    if outside is None:
        return v
    return np.where(np.abs(x) < 1.0, v, outside)


def pswf_taper(max_support, width=7.0):
    """Image-domain taper sampled where the w-kernel screen is (x = i/r,
    i in [-r, r)), for a uv-kernel of about `width` cells."""
    r = max_support // 2
    x = np.arange(-r, r + max_support % 2, dtype=np.float64) / r
    return pswf(x, math.pi * width / 2.0, outside=None)


def pswf_uv_gcf(support=8, width=7, over=OVER):
    """uv-domain PSWF GCF [ou + 8 ov][sy][sx] (complex128): tap i of phase ou
    sits at offset i - support/2 - ou/over cells from the visibility; zero
    beyond width/2 (so a 7-wide kernel padded to 8 has tap 0 zero)."""
    half = width / 2.0
    c = math.pi * width / 2.0
    o = np.arange(over)
    i = np.arange(support)
    off = i[None, :] - support // 2 - o[:, None] / over  # [phase][tap]
    k1 = pswf(off / half, c)  # [o][i]
    g = np.einsum("vj,ui->vuji", k1, k1)  # [ov][ou][sy][sx]
    return np.ascontiguousarray(g.reshape(over * over, support, support)).astype(np.complex128)


def generate(w_planes, supports, max_support, t2, taper=None, want64=True, want32=True,
             device="cuda", stream=None):
    """All planes' GCFs on the GPU.  Returns (gcf64 or None, gcf32 or None, offsets)."""
    import torch

    L = _lib.load()
    w = np.ascontiguousarray(w_planes, np.float64)
    s = np.ascontiguousarray(supports, np.int32)
    offs, total = layout(s)
    g64 = torch.empty(total, dtype=torch.complex128, device=device) if want64 else None
    g32 = torch.empty(total, dtype=torch.complex64, device=device) if want32 else None
    tap = None
    if taper is not None:
        tap = torch.as_tensor(np.ascontiguousarray(taper, np.float64), device=device)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _lib.check(L.gb_gcf_generate(len(s), w.ctypes.data_as(C.POINTER(C.c_double)),
                                 s.ctypes.data_as(C.POINTER(C.c_int32)),
                                 offs.ctypes.data_as(C.POINTER(C.c_int64)), int(max_support),
                                 float(t2), tap.data_ptr() if tap is not None else None,
                                 g64.data_ptr() if g64 is not None else None,
                                 g32.data_ptr() if g32 is not None else None, st),
               "gb_gcf_generate")
    return g64, g32, offs


def grid_correction(gcf_plane, n, offsets="generator", over=OVER):
    """Image-domain grid-correction function of an oversampled GCF plane.

    gcf_plane: one plane's GCF, [64][S][S] complex (phase ou + 8 ov, MS6
    layout), normally a w = 0 kernel.  The kernel is taken as separable: the
    1-D kernel of phase ou is the column sum of phase (ou, 0).  `offsets` says
    where tap sx of phase ou was sampled: "generator" d = sx - S/2 + ou/8 cells
    (the w-kernel generator, GCF.cpp:39-47) or "centred" d = sx - S/2 - ou/8
    (a kernel centred on the visibility under the MS6 index math, as
    pswf_uv_gcf builds it).  Returns c(j) = Re sum_d K(d) exp(2 pi i d
    (j - n/2) / n) / over for the n image pixels: the transform of the kernel
    the samples come from, 1 at the centre if the kernel sums to 1."""
    g = np.asarray(gcf_plane).reshape(over * over, -1)
    S = int(round(np.sqrt(g.shape[1])))
    g = g.reshape(over, over, S, S)  # [ov][ou][sy][sx]
    k = g[0].sum(axis=1)  # [ou][sx]: sum over sy of phase (ou, ov=0)
    sign = {"generator": 1.0, "centred": -1.0}[offsets]
    d = (np.arange(S)[None, :] - S // 2 + sign * np.arange(over)[:, None] / over).ravel()
    kv = k.ravel()
    l = (np.arange(n) - n // 2) / n
    return np.real(np.exp(2j * np.pi * np.outer(l, d)) @ kv) / over


def w0_correction(max_support, t2, taper, n, support=8, device="cuda"):
    """Grid correction of a w-projection GCF set: the image response of its
    w = 0 kernel (same generator, field of view and taper), generated on the
    GPU and transformed by grid_correction()."""
    _, g32, _ = generate([0.0], [support], max_support, t2, taper=taper, want64=False,
                         device=device)
    return grid_correction(g32.cpu().numpy(), n)


def select(w_files, w0, w1):
    """(index, conjugate) of the GCF for the w-region [w0, w1] (gb_gcf_select)."""
    w = np.ascontiguousarray(w_files, np.float64)
    idx, conj = C.c_int32(), C.c_int32()
    L = _lib.load()
    _lib.check(L.gb_gcf_select(len(w), w.ctypes.data_as(C.POINTER(C.c_double)), float(w0),
                               float(w1), C.byref(idx), C.byref(conj)), "gb_gcf_select")
    return idx.value, bool(conj.value)
