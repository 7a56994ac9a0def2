"""ORACLE — test infrastructure only.

Python face of the CPU FP64 restatement of the reference's gridding path.  Only
tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs
may import this module, and only as the checker (or the timed CPU baseline);
the rc_gb300 product never does.

Contents
  * ctypes bindings of oracle/gridref.c (kern_scatter / kern_degrid semantics,
    multi-plane forms, w-binning);
  * gcf_layers(): numpy restatement of the reference's w-kernel generator,
    MS4/kernel/cpu/gcf/GCF.cpp:58-117 (screen, centred FFT) and :16-52
    (per-phase normalisation, extraction), with FFTW's backward transform
    (MS4/kernel/cpu/fft/fft_dyn_padded.cpp:76-103: fftshift, unnormalised
    exp(+2*pi*i) DFT, fftshift) written as numpy's ifft2 times N^2;
  * binsizer(): the w-range rule of MS6/programs/Kernel/Binning.hs:51-60;
  * kern_fft() / kern_ifft(): the reference's Halide FFT kernels
    (MS6/kernel/cpu/gridding/fft.cpp:546-662) with exact twiddles;
  * ms4_* wrappers of the reference's own compiled MS4 gridder/degridder
    (oracle/_ref, built from the reference sources by `make -C oracle ref`),
    used to pin the restatement where the two index conventions coincide.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OVER = 8

_lib = None
_ms4 = None

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32, _i64, _f64 = C.c_int32, C.c_int64, C.c_double


def reference_root() -> str:
    """The reference checkout the `ref` target compiles from: RC_REFERENCE in
    the environment, else the Makefile's default."""
    root = os.environ.get("RC_REFERENCE")
    if root:
        return root
    r = subprocess.run(["make", "-s", "-C", HERE, "refroot"], capture_output=True, text=True)
    return r.stdout.strip()


def build(ref: bool = True) -> None:
    """Compile oracle/liboracle.so (and oracle/_ref when the reference is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    root = reference_root() if ref else ""
    if root and os.path.isdir(os.path.join(root, "MS4")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REFROOT=" + root], check=True)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref=False)
        L = C.CDLL(path)
        L.orc_index.argtypes = [_i64, _f64p, _i64, _f64, _i32, _i32, _i32, _i32, _i32, _i32, _i32, _i32p]
        L.orc_scatter.argtypes = [_f64, _i32, _i32, _i32, _i64, _f64p, _i64, _f64p, _f64p,
                                  _i32, _i32, _i32, _i32, _i64]
        L.orc_degrid.argtypes = [_f64, _i32, _i32, _i32, _i64, _f64p, _i64, _f64p, _f64p,
                                 _i32, _i32, _i32, _i32, _i64, _f64p, _i64]
        L.orc_scatter_planes.argtypes = [_f64, _i32, _i32, _i64, _f64p, _i64, _f64p, _i32p, _i32p,
                                         _i64p, _f64p, _f64p, _i32, _i32, _i64]
        L.orc_scatter_planes_omp.argtypes = L.orc_scatter_planes.argtypes + [C.c_int]
        L.orc_scatter_planes_omp.restype = C.c_int
        L.orc_degrid_planes.argtypes = [_f64, _i32, _i32, _i64, _f64p, _i64, _i32p, _i32p, _i64p,
                                        _f64p, _f64p, _i32, _i32, _i64, _i32, _f64p, C.c_int]
        L.orc_wbin.argtypes = [_i64, _f64p, _i64, _f64, _f64, _i32, _i32p]
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---------------------------------------------------------------- single GCF (ABI form)
def index(vis5, scale, grid_size, S, margin, min_x=0, min_y=0, ext_x=None, ext_y=None):
    """(N,5) int32: x0, y0, ou, ov, in-bound — scatter.cpp:56-76."""
    vis5 = _c(vis5, np.float64)
    n = vis5.shape[0]
    out = np.zeros((n, 5), np.int32)
    lib().orc_index(n, vis5.reshape(-1), 5, scale, grid_size, S, margin, min_x, min_y,
                    ext_x, ext_y, out.reshape(-1))
    return out


def scatter(scale, grid_size, margin, vis5, gcf, grid, min_x=0, min_y=0):
    """kern_scatter semantics, in place on `grid` (complex128 [ext_y][ext_x])."""
    vis5 = _c(vis5, np.float64)
    S = gcf.shape[-1]
    g = _c(gcf, np.complex128).view(np.float64).reshape(-1)
    ext_y, ext_x = grid.shape
    assert grid.dtype == np.complex128 and grid.flags.c_contiguous
    lib().orc_scatter(scale, grid_size, margin, S, vis5.shape[0], vis5.reshape(-1), 5, g,
                      grid.view(np.float64).reshape(-1), min_x, min_y, ext_x, ext_y, ext_x)
    return grid


def degrid(scale, grid_size, margin, gcf, grid, vis5, min_x=0, min_y=0):
    """kern_degrid semantics: returns vis_out (N,5)."""
    vis5 = _c(vis5, np.float64)
    S = gcf.shape[-1]
    g = _c(gcf, np.complex128).view(np.float64).reshape(-1)
    grid = _c(grid, np.complex128)
    ext_y, ext_x = grid.shape
    out = np.zeros_like(vis5)
    lib().orc_degrid(scale, grid_size, margin, S, vis5.shape[0], vis5.reshape(-1), 5, g,
                     grid.view(np.float64).reshape(-1), min_x, min_y, ext_x, ext_y, ext_x,
                     out.reshape(-1), 5)
    return out


# ---------------------------------------------------------------- multi-plane (engine form)
def scatter_planes(scale, grid_size, margin, uvw, vis, plane, supports, gcf_flat, gcf_off,
                   grid, nthreads=1):
    """grid += G(vis) over all planes.  vis complex128 (N,), gcf_flat complex128."""
    uvw = _c(uvw, np.float64)
    vis = _c(vis, np.complex128)
    ext_y, ext_x = grid.shape
    args = (scale, grid_size, margin, uvw.shape[0], uvw.reshape(-1), uvw.shape[1],
            vis.view(np.float64), _c(plane, np.int32), _c(supports, np.int32),
            _c(gcf_off, np.int64), _c(gcf_flat, np.complex128).view(np.float64),
            grid.view(np.float64).reshape(-1), ext_x, ext_y, ext_x)
    if nthreads == 1:
        lib().orc_scatter_planes(*args)
        return 1
    return lib().orc_scatter_planes_omp(*args, nthreads)


def degrid_planes(scale, grid_size, margin, uvw, plane, supports, gcf_flat, gcf_off, grid,
                  mode=0, nthreads=1):
    """Predicted visibilities (complex128 (N,)).  mode 0: exact adjoint (conj GCF);
    mode 1: the reference kern_degrid product with its sign (-sum grid*gcf)."""
    uvw = _c(uvw, np.float64)
    grid = _c(grid, np.complex128)
    ext_y, ext_x = grid.shape
    pred = np.zeros(uvw.shape[0], np.complex128)
    lib().orc_degrid_planes(scale, grid_size, margin, uvw.shape[0], uvw.reshape(-1),
                            uvw.shape[1], _c(plane, np.int32), _c(supports, np.int32),
                            _c(gcf_off, np.int64), _c(gcf_flat, np.complex128).view(np.float64),
                            grid.view(np.float64).reshape(-1), ext_x, ext_y, ext_x, mode,
                            pred.view(np.float64), nthreads)
    return pred


def wbin(uvw, low, high, bins):
    uvw = _c(uvw, np.float64)
    out = np.zeros(uvw.shape[0], np.int32)
    lib().orc_wbin(uvw.shape[0], uvw.reshape(-1), uvw.shape[1], low, high, bins, out)
    return out


def binsizer(w):
    """Binning.hs:51-60: low = min(0, min w), high0 = max(0, max w) (the fold starts
    at (0,0)), high = high0 + (high0-low)*1e-4."""
    low = min(0.0, float(np.min(w))) if len(w) else 0.0
    high0 = max(0.0, float(np.max(w))) if len(w) else 0.0
    return low, high0 + (high0 - low) * 0.0001


def xy2uv(height, scale, z):
    """gridXY2UV (MS6/programs/Kernel/Config.hs:211-212)."""
    return float(z - height // 2) / scale


def tile_bins(vis5, height, scale, u_range, v_range, bins):
    """binSizer + binner (MS6/programs/Kernel/Binning.hs:34-99, 102-181) for one
    (u, v) tile of pixel ranges [lo, hi): returns [(low, high, count, records)]
    per w-bin, records padded with zero rows to count."""
    vis5 = np.asarray(vis5, np.float64)
    u, v, w = vis5[:, 0], vis5[:, 1], vis5[:, 2]
    umin, umax = xy2uv(height, scale, u_range[0]), xy2uv(height, scale, u_range[1])
    vmin, vmax = xy2uv(height, scale, v_range[0]), xy2uv(height, scale, v_range[1])
    inside = (u >= umin) & (u < umax) & (v >= vmin) & (v < vmax)
    low, high0 = 0.0, 0.0  # the fold's start
    for x in w[inside]:
        low, high0 = min(x, low), max(x, high0)
    high = high0 + (high0 - low) * 0.0001
    starts = [low + b * (high - low) / bins for b in range(bins + 1)]
    counts = [0] * bins
    for x in w[inside]:
        if not (low <= x <= high):
            continue
        f = np.floor((x - low) / (high - low) * bins) if high > low else 0.0
        counts[int(max(0, min(bins - 1, f)))] += 1
    recs = [[] for _ in range(bins)]
    for i in np.flatnonzero(inside):
        x = w[i]
        cand = [b for b in range(bins) if starts[b] <= x]  # Map.lookupLE on the lows
        if not cand:
            continue
        k = max(cand, key=lambda b: (starts[b], b))
        if x < starts[k + 1]:
            recs[k].append(vis5[i])
    out = []
    for b in range(bins):
        r = np.array(recs[b], np.float64).reshape(-1, 5)
        if len(r) < counts[b]:
            r = np.vstack([r, np.zeros((counts[b] - len(r), 5))])
        out.append((starts[b], starts[b + 1], counts[b], r))
    return out


def tile_bins_vec(vis5, height, scale, u_range, v_range, bins):
    """tile_bins for finite w, vectorised (the same arithmetic in the same
    order, so the same bins, counts and records): the lows are non-decreasing,
    so Map.lookupLE (the last bin whose low <= w, the last of equal lows) is a
    right-sided binary search."""
    vis5 = np.asarray(vis5, np.float64)
    u, v, w = vis5[:, 0], vis5[:, 1], vis5[:, 2]
    umin, umax = xy2uv(height, scale, u_range[0]), xy2uv(height, scale, u_range[1])
    vmin, vmax = xy2uv(height, scale, v_range[0]), xy2uv(height, scale, v_range[1])
    inside = (u >= umin) & (u < umax) & (v >= vmin) & (v < vmax)
    wi = w[inside]
    assert np.isfinite(wi).all(), "tile_bins_vec: finite w only (tile_bins handles the rest)"
    low = min(0.0, float(wi.min())) if len(wi) else 0.0
    high0 = max(0.0, float(wi.max())) if len(wi) else 0.0
    high = high0 + (high0 - low) * 0.0001
    starts = [low + b * (high - low) / bins for b in range(bins + 1)]
    ok = (wi >= low) & (wi <= high)
    if high > low:
        f = np.floor((wi[ok] - low) / (high - low) * bins)
    else:
        f = np.zeros(int(ok.sum()))
    counts = np.bincount(np.clip(f, 0, bins - 1).astype(np.int64), minlength=bins)
    idx = np.flatnonzero(inside)
    k = np.searchsorted(np.asarray(starts[:bins]), wi, side="right") - 1
    keep = k >= 0
    kk = np.where(keep, k, 0)
    keep &= wi < np.asarray(starts)[kk + 1]
    out = []
    for b in range(bins):
        r = vis5[idx[keep & (k == b)]]
        c = int(counts[b])
        if len(r) < c:
            r = np.vstack([r, np.zeros((c - len(r), 5))])
        out.append((starts[b], starts[b + 1], c, r))
    return out


# ---------------------------------------------------------------- GCF generation (MS4 spec)
def gcf_layers(w, support, max_support, t2, taper=None, over=OVER):
    """One w-plane's oversampled GCF in the MS6 layout [ou + 8*ov][sy][sx] (complex128).

    GCF.cpp:58-117: screen (cos 2*pi*ph, -sin 2*pi*ph), ph = w*(1-sqrt(1-x^2-y^2)),
    x = i*t2/(max_support/2) on rows, y = j*t2/(max_support/2) on columns, for
    i, j in [-r, r + max_support%2); centred in a (over*max_support)^2 zero arena;
    centred backward FFT; per-phase sums of real parts over the whole arena
    (GCF.cpp:25-32); centred support x support extraction (GCF.cpp:39-51).
    `taper` (optional, length max_support) multiplies the screen separably; the
    reference screen has none.
    """
    size = max_support * over
    r = max_support // 2
    i = np.arange(-r, r + max_support % 2, dtype=np.float64)
    x = i * (t2 / float(r))
    X = x[:, None]
    Y = x[None, :]
    ph = w * (1.0 - np.sqrt(1.0 - X * X - Y * Y))
    screen = np.cos(2.0 * np.pi * ph) - 1j * np.sin(2.0 * np.pi * ph)
    if taper is not None:
        t = np.asarray(taper, np.float64)
        screen = screen * (t[:, None] * t[None, :])
    arena = np.zeros((size, size), np.complex128)
    a0 = size // 2 - r
    arena[a0:a0 + max_support, a0:a0 + max_support] = screen
    arena = np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(arena))) * float(size * size)
    a4 = arena.reshape(max_support, over, max_support, over)  # [su][ou][sv][ov]
    sums = a4.real.sum(axis=(0, 2))  # [ou][ov]
    c = max_support // 2 - support // 2
    sub = a4[c:c + support, :, c:c + support, :]  # [su][ou][sv][ov]
    ms4 = sub.transpose(1, 3, 0, 2) / sums[:, :, None, None]  # [ou][ov][su][sv]
    # MS6 layout: [ov][ou][sy=sv][sx=su] flattened as phase ou + 8*ov
    return np.ascontiguousarray(ms4.transpose(1, 0, 3, 2)).reshape(over * over, support, support)


# ---------------------------------------------------------------- reference MS4 binary (pinning)
def _aligned_zeros(shape, dtype, align=64):
    """Zeroed array whose data starts on an `align`-byte boundary (the MS4 code
    uses aligned AVX loads/stores on the grid)."""
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    raw = np.zeros(n + align, np.uint8)
    off = (-raw.ctypes.data) % align
    return raw[off:off + n].view(dt).reshape(shape)


def ms4_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libms4ref.so"))


def ms4():
    global _ms4
    if _ms4 is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libms4ref.so"))
        sig = [_f64, _f64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
               C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.gridKernelCPUFullGCF.argtypes = sig
        L.gridKernelCPUFullGCF.restype = C.c_ulonglong
        L.deGridKernelCPUFullGCF.argtypes = sig
        L.deGridKernelCPUFullGCF.restype = C.c_ulonglong
        _ms4 = L
    return _ms4


def _ms4_args(scale, uvw_bl, vis_bl, layers_ms4, supp, grid_size):
    """Pointer tables for the MS4 calling convention, one w-plane (index 0)."""
    nbl, ts = uvw_bl.shape[:2]
    keep = []
    uvw_ptrs = (C.c_void_p * nbl)()
    vis_ptrs = (C.c_void_p * nbl)()
    for b in range(nbl):
        u = np.ascontiguousarray(uvw_bl[b], np.float64)
        v = np.ascontiguousarray(vis_bl[b], np.complex128)
        keep += [u, v]
        uvw_ptrs[b] = u.ctypes.data
        vis_ptrs[b] = v.ctypes.data
    lay = np.ascontiguousarray(layers_ms4, np.complex128)  # [ou][ov][su][sv]
    keep.append(lay)
    gptrs = (C.c_void_p * (OVER * OVER))()
    for k in range(OVER * OVER):
        gptrs[k] = lay.ctypes.data + k * supp * supp * 16
    bl_supps = np.full(nbl, supp, np.int32)
    gcf_supps = np.array([supp], np.int32)
    keep += [bl_supps, gcf_supps]
    return keep, uvw_ptrs, vis_ptrs, gptrs, bl_supps, gcf_supps


def ms4_grid(scale, uvw_bl, vis_bl, gcf_ms6, grid_size):
    """Reference MS4 gridKernelCPUFullGCF on one w-plane; returns the grid in the
    MS6 orientation [v][u] (complex128 grid_size^2)."""
    supp = gcf_ms6.shape[-1]
    layers = gcf_ms6.reshape(OVER, OVER, supp, supp).transpose(1, 0, 3, 2)  # -> [ou][ov][su][sv]
    keep, up, vp, gp, bls, gss = _ms4_args(scale, uvw_bl, vis_bl, layers, supp, grid_size)
    grid = _aligned_zeros((grid_size, grid_size), np.complex128)  # [u][v]
    ms4().gridKernelCPUFullGCF(scale, 1e300, uvw_bl.shape[0], bls.ctypes.data, grid.ctypes.data,
                               C.cast(gp, C.c_void_p), C.cast(up, C.c_void_p),
                               C.cast(vp, C.c_void_p), uvw_bl.shape[1], grid_size, grid_size,
                               gss.ctypes.data)
    del keep
    return np.ascontiguousarray(grid.T)


def ms4_degrid(scale, uvw_bl, grid_ms6, gcf_ms6):
    """Reference MS4 deGridKernelCPUFullGCF on one w-plane: sum grid*gcf per
    visibility (no conjugate).  grid_ms6 is [v][u]; returns (nbl, ts) complex128."""
    supp = gcf_ms6.shape[-1]
    grid_size = grid_ms6.shape[0]
    layers = gcf_ms6.reshape(OVER, OVER, supp, supp).transpose(1, 0, 3, 2)
    out = np.zeros(uvw_bl.shape[:2], np.complex128)
    keep, up, vp, gp, bls, gss = _ms4_args(scale, uvw_bl, out, layers, supp, grid_size)
    # the degridder writes through the visibility pointer table: point it at `out`
    for b in range(uvw_bl.shape[0]):
        vp[b] = out.ctypes.data + b * uvw_bl.shape[1] * 16
    g = _aligned_zeros((grid_size, grid_size), np.complex128)
    g[...] = grid_ms6.T  # -> [u][v]
    ms4().deGridKernelCPUFullGCF(scale, 1e300, uvw_bl.shape[0], bls.ctypes.data, g.ctypes.data,
                                 C.cast(gp, C.c_void_p), C.cast(up, C.c_void_p),
                                 C.cast(vp, C.c_void_p), uvw_bl.shape[1], grid_size, grid_size,
                                 gss.ctypes.data)
    del keep
    return out


# ---------------------------------------------------------------- Hogbom CLEAN
def hogbom_f32(res, psf, ppx, ppy, gain, threshold, n_iter):
    """The engine's CLEAN in numpy float32 (what gb_hogbom_f32 must reproduce
    bit for bit): peak = largest |res| (first in row-major order), stop under
    threshold, res -= (gain*peak/psf[ppy,ppx]) * shifted psf, model[peak] +=
    gain*peak.  Returns (residual, model, iterations)."""
    res = np.array(res, np.float32, copy=True)
    psf = np.asarray(psf, np.float32)
    model = np.zeros_like(res)
    ny, nx = res.shape
    pny, pnx = psf.shape
    g = np.float32(gain)
    th = np.float32(threshold)
    pp = psf[ppy, ppx]
    done = 0
    for _ in range(n_iter):
        a = np.abs(res)
        idx = int(np.argmax(a))
        if a.flat[idx] < th or pp == 0:
            break
        val = res.flat[idx]
        py, px = divmod(idx, nx)
        s = np.float32(np.float32(g * val) / pp)
        dx, dy = px - ppx, py - ppy
        x0, x1 = max(0, dx), min(nx, dx + pnx)
        y0, y1 = max(0, dy), min(ny, dy + pny)
        if x0 < x1 and y0 < y1:
            res[y0:y1, x0:x1] = res[y0:y1, x0:x1] - s * psf[y0 - dy:y1 - dy, x0 - dx:x1 - dx]
        model.flat[idx] = np.float32(model.flat[idx] + np.float32(g * val))
        done += 1
    return res, model, done


def hogbom_reference(gain, threshold, psf, res, model=None, cycles=12):
    """MS6/kernel/cpu/gridding/hogbom.cpp:30-109 restated (FP64): the "PSF
    peak" is argmax |res| over the PSF's extent (:58), peak values are
    absolute (:85-90), the shift is clamped (:99-100), the model gets
    gain*|peak| (:108); the residual is the one of the cycle at which the
    threshold is first crossed, else the last (:68-74).  Returns (model, residual)."""
    res = np.array(res, np.float64, copy=True)
    psf = np.asarray(psf, np.float64)
    model = np.zeros_like(res) if model is None else np.array(model, np.float64, copy=True)
    ny, nx = res.shape
    pny, pnx = psf.shape
    sub = np.abs(res[:min(pny, ny), :min(pnx, nx)])
    ppy, ppx = divmod(int(np.argmax(sub)), sub.shape[1])
    pval = sub[ppy, ppx]
    yy, xx = np.mgrid[0:ny, 0:nx]
    for _ in range(cycles):
        a = np.abs(res)
        idx = int(np.argmax(a))
        val = a.flat[idx]
        if val < threshold:
            break
        py, px = divmod(idx, nx)
        dx = min(max(px - ppx, -pnx), nx)
        dy = min(max(py - ppy, -pny), ny)
        qx, qy = xx - dx, yy - dy
        inside = (qx >= 0) & (qx < pnx) & (qy >= 0) & (qy < pny)
        shifted = np.zeros_like(res)
        shifted[inside] = psf[qy[inside], qx[inside]]
        res = res - (gain * val / pval) * shifted
        model[min(max(py, 0), ny - 1), min(max(px, 0), nx - 1)] += gain * val
    return model, res


# ---------------------------------------------------------------- kern_fft / kern_ifft
# The reference's Halide FFT kernels (MS6/kernel/cpu/gridding/fft.cpp) restated
# with numpy's exact transforms.  Parity unpinned: the Halide generator cannot
# run here, and its twiddle angles are built from float(2 pi) and
# float(sqrt(2)/2) (fft.cpp:120, 126, 204-205, 229), about 1e-8 (relative) from
# these exact transforms.  Arrays are [y][x] (image) and [v][u] (grid).

def kern_fft(img):
    """fftKernel (fft.cpp:607-662): the image rotated by half its size
    (repeat_image, :617-619), its forward DFT kept for rows v <= n/2 (the
    half spectrum of fft2d_r2c, :367-428, zero beyond: :634), then
    out(u,v) = (B(u-h, v-h) + conj(B(h-u-1, h-v-1))) / n  (:635-638)."""
    img = np.asarray(img, np.float64)
    n = img.shape[0]
    h = n // 2
    F = np.fft.fft2(np.roll(img, (h, h), axis=(0, 1)))
    F[h + 1:, :] = 0
    v = np.arange(n)[:, None]
    u = np.arange(n)[None, :]
    return (F[(v - h) % n, (u - h) % n] + np.conj(F[(h - v - 1) % n, (h - u - 1) % n])) / n


def kern_ifft(g):
    """ifftKernel (fft.cpp:546-589): the grid "hermitised" about
    (n-1-u, n-1-v) (:557-558), rotated by half (:561-563), fft2d_c2r
    (:430-509: the inverse DFT along u of rows 0..n/2, the other rows by
    conjugate symmetry, two real columns x and x+n/2 packed into one complex
    inverse DFT along v), rotated back and divided by n (:572-573)."""
    g = np.asarray(g, np.complex128)
    n = g.shape[0]
    h = n // 2
    herm = (g + np.conj(g[::-1, ::-1])) / 2
    S = np.roll(herm, (-h, -h), axis=(0, 1))
    D = n * np.fft.ifft(S[:h + 1], axis=1)
    X = np.empty((n, n), np.complex128)
    X[:h] = D[:h]
    X[h:] = np.conj(D[n - np.arange(h, n)])
    T = n * np.fft.ifft(X, axis=0)
    image = np.empty((n, n))
    image[:, :h] = T[:, :h].real - T[:, h:].imag
    image[:, h:] = T[:, :h].imag + T[:, h:].real
    return np.roll(image, (-h, -h), axis=(0, 1)) / n


# ---------------------------------------------------------------- detile / rotate
def detile(in_grid, in_min, out_grid, out_min):
    """MS6/kernel/cpu/gridding/detile.cpp:16-30: out += in over the overlap of
    the two (min, extent) regions.  Grids are complex [H][W]; mins (x, y)."""
    out = np.array(out_grid, copy=True)
    ih, iw = in_grid.shape
    oh, ow = out.shape
    x0, x1 = max(in_min[0], out_min[0]), min(in_min[0] + iw, out_min[0] + ow)
    y0, y1 = max(in_min[1], out_min[1]), min(in_min[1] + ih, out_min[1] + oh)
    if x1 > x0 and y1 > y0:
        out[y0 - out_min[1]:y1 - out_min[1], x0 - out_min[0]:x1 - out_min[0]] += \
            in_grid[y0 - in_min[1]:y1 - in_min[1], x0 - in_min[0]:x1 - in_min[0]]
    return out


def _rx(p):
    s, c = np.sin(p), np.cos(p)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def _rz(p):
    s, c = np.sin(p), np.cos(p)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def rotate(in_lon, in_lat, out_lon, out_lat, uvproj, vis5):
    """MS6/kernel/cpu/gridding/rotate.cpp:36-66 with utils.h:119-163: R =
    xyz2uvw(out) uvw2xyz(in); uvw' = (R^T inv2x2(R)^T R) uvw if uvproj else
    uvw; vis' = vis * exp(2 pi i ((0,0,1) - R (0,0,1)) . uvw)."""
    xyz2uvw = _rx(-np.pi / 2 + out_lat) @ _rz(-np.pi / 2 - out_lon)
    uvw2xyz = _rz(np.pi / 2 + in_lon) @ _rx(np.pi / 2 - in_lat)
    R = xyz2uvw @ uvw2xyz
    if uvproj:
        det = R[0, 0] * R[1, 1] - R[0, 1] * R[1, 0]
        inv = np.array([[R[1, 1] / det, -R[0, 1] / det, 0], [-R[1, 0] / det, R[0, 0] / det, 0],
                        [0, 0, 1]])
        M = R.T @ (inv.T @ R)
    else:
        M = np.eye(3)
    uvw = vis5[:, :3]
    pc = np.array([0.0, 0.0, 1.0]) - R @ np.array([0.0, 0.0, 1.0])
    path = uvw @ pc
    v = (vis5[:, 3] + 1j * vis5[:, 4]) * np.exp(2j * np.pi * path)
    out = np.empty_like(vis5)
    out[:, :3] = uvw @ M.T
    out[:, 3], out[:, 4] = v.real, v.imag
    return out


# ---------------------------------------------------------------- GCF choice
def gcf_select(w_files, w0, w1):
    """Config.hs:128-132 (maximumBy (comparing gcfW) . filter ((<= w) . gcfW),
    w = max |w0| |w1|; maximumBy keeps the last of equal maxima) and
    IO.hs:110-113 (conjugate when low < -high).  Raises if nothing qualifies."""
    w = max(abs(w0), abs(w1))
    cand = [i for i, x in enumerate(w_files) if x <= w]
    if not cand:
        raise ValueError("no GCF with w <= %g" % w)
    best = cand[0]
    for i in cand[1:]:
        if w_files[i] >= w_files[best]:
            best = i
    return best, w0 < -w1
