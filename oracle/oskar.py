"""ORACLE — test infrastructure only.

OSKAR 2.6 visibility files: Python face of oracle/oskarref.c (the C
restatement of the reference reader MS6/kernel/oskar/OskarBinReader.cpp and
its container library MS6/kernel/oskar/oskar_binary/, plus a writer of that
layout), the reference's own reader compiled from its sources into
oracle/_ref/liboskarref.so (present only where the reference checkout is),
and a numpy restatement of the pipeline's record extraction
(MS6/programs/Kernel/IO.hs:22-74).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this
module; the rc_gb300 product never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import oracle as _o

HERE = os.path.dirname(os.path.abspath(__file__))
C_LIGHT = 299792458.0

# container status codes (MS6/kernel/oskar/oskar_binary/oskar_binary.h:96-114)
ST_OPEN_FAIL, ST_READ_FAIL, ST_FILE_INVALID, ST_FORMAT_BAD = -100, -102, -106, -107
ST_VERSION, ST_TYPE, ST_MEMORY, ST_NOT_FOUND, ST_CRC = -109, -110, -114, -115, -118
ST_NOT_DOUBLE = 0xDEADBEEF - (1 << 32)  # OskarBinReader.cpp:183-186, as a C int

DOUBLE_COMPLEX_MATRIX = 0x68
SINGLE_COMPLEX_MATRIX = 0x64


class VisHeader(C.Structure):
    """The fields of the reference's VisData after its file handle."""
    _fields_ = [("num_baselines", C.c_int), ("num_channels", C.c_int),
                ("num_stations", C.c_int), ("num_times", C.c_int),
                ("num_times_baselines", C.c_int), ("num_points", C.c_int),
                ("phase_centre", C.c_double * 2), ("telescope_centre", C.c_double * 3),
                ("freq_start_inc", C.c_double * 2), ("time_start_inc", C.c_double * 2),
                ("channel_bandwidth_hz", C.c_double), ("time_average_sec", C.c_double)]


class RefVisData(C.Structure):
    """MS6/kernel/oskar/OskarBinReader.h:34-52."""
    _fields_ = [("h", C.c_void_p)] + VisHeader._fields_


class VisLayout(C.Structure):
    _fields_ = [("num_stations", C.c_int), ("num_times", C.c_int), ("num_channels", C.c_int),
                ("max_times_per_block", C.c_int), ("amp_type", C.c_int),
                ("write_autocorr", C.c_int), ("trim_last_block", C.c_int),
                ("extended_tags", C.c_int), ("freq_start_hz", C.c_double),
                ("freq_inc_hz", C.c_double), ("channel_bandwidth_hz", C.c_double),
                ("time_start_mjd_utc", C.c_double), ("time_inc_sec", C.c_double),
                ("time_average_sec", C.c_double), ("phase_centre", C.c_double * 2),
                ("telescope_centre", C.c_double * 3)]


_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_bound = False
_ref = None


def _lib():
    global _bound
    L = _o.lib()
    if not _bound:
        L.orc_crc32c.restype = C.c_uint32
        L.orc_crc32c.argtypes = [C.c_void_p, C.c_size_t]
        L.orc_crc32c_update.restype = C.c_uint32
        L.orc_crc32c_update.argtypes = [C.c_uint32, C.c_void_p, C.c_size_t]
        L.orc_oskar_header.argtypes = [C.c_char_p, C.POINTER(VisHeader)]
        L.orc_oskar_read.argtypes = [C.c_char_p, _f64p, _f64p, _f64p, _f64p]
        L.orc_oskar_write.argtypes = [C.c_char_p, C.POINTER(VisLayout), _f64p, _f64p, _f64p,
                                      _f64p]
        _bound = True
    return L


def crc32c(data: bytes | np.ndarray, code: int | None = None) -> int:
    """CRC-32C of a byte string; `code` continues a finished code the way the
    container does (oskar_crc.c:109-160)."""
    b = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8) if isinstance(data, bytes)
                             else data).view(np.uint8)
    L = _lib()
    if code is None:
        return int(L.orc_crc32c(b.ctypes.data, b.nbytes))
    return int(L.orc_crc32c_update(code, b.ctypes.data, b.nbytes))


def layout(num_stations, num_times, num_channels=1, max_times_per_block=8,
           amp_type=DOUBLE_COMPLEX_MATRIX, write_autocorr=False, trim_last_block=False,
           extended_tags=False, freq_start_hz=150e6, freq_inc_hz=1e6,
           channel_bandwidth_hz=1e6, time_start_mjd_utc=57000.0, time_inc_sec=10.0,
           time_average_sec=10.0, phase_centre=(0.0, -45.0),
           telescope_centre=(116.76, -26.82, 0.0)) -> VisLayout:
    L = VisLayout()
    L.num_stations, L.num_times, L.num_channels = num_stations, num_times, num_channels
    L.max_times_per_block, L.amp_type = max_times_per_block, amp_type
    L.write_autocorr, L.trim_last_block = int(write_autocorr), int(trim_last_block)
    L.extended_tags = int(extended_tags)
    L.freq_start_hz, L.freq_inc_hz = freq_start_hz, freq_inc_hz
    L.channel_bandwidth_hz = channel_bandwidth_hz
    L.time_start_mjd_utc, L.time_inc_sec = time_start_mjd_utc, time_inc_sec
    L.time_average_sec = time_average_sec
    L.phase_centre[:] = phase_centre
    L.telescope_centre[:] = telescope_centre
    return L


def write(path, lay: VisLayout, amps, uu, vv, ww) -> int:
    """amps: (T, C, B, 4) complex128 cross-correlations; uu/vv/ww: (T, B) metres."""
    T, Cn, B = lay.num_times, lay.num_channels, lay.num_stations * (lay.num_stations - 1) // 2
    a = np.ascontiguousarray(amps, np.complex128).reshape(T, Cn, B, 4).view(np.float64)
    a = np.ascontiguousarray(a).reshape(-1)
    u, v, w = (np.ascontiguousarray(x, np.float64).reshape(T, B) for x in (uu, vv, ww))
    return int(_lib().orc_oskar_write(os.fsencode(path), C.byref(lay), a, u.reshape(-1),
                                      v.reshape(-1), w.reshape(-1)))


def synth(num_stations, num_times, num_channels=1, seed=0, w_scale=1.0):
    """Seeded cross-correlations and baselines in metres (T, C, B, 4), (T, B) x 3."""
    rng = np.random.default_rng(seed)
    B = num_stations * (num_stations - 1) // 2
    amps = (rng.standard_normal((num_times, num_channels, B, 4)) +
            1j * rng.standard_normal((num_times, num_channels, B, 4)))
    base = rng.uniform(-3000, 3000, (3, B))
    t = np.arange(num_times)[:, None] * 0.01
    uu = base[0] * np.cos(t) - base[1] * np.sin(t)
    vv = base[0] * np.sin(t) + base[1] * np.cos(t)
    ww = w_scale * base[2] * np.cos(0.5 * t) + 0.0 * t
    return amps, uu, vv, ww


def header(path):
    h = VisHeader()
    st = _lib().orc_oskar_header(os.fsencode(path), C.byref(h))
    return st, h


def read(path):
    """mkFromFile + readAndReshuffle restated.  Returns (status, header,
    amps (P, 4) complex128, uvw (P, 3), metrix (6,), blws (B, 2))."""
    st, h = header(path)
    if st:
        return st, h, None, None, None, None
    P, B = h.num_points, h.num_baselines
    amps = np.zeros(P * 8, np.float64)
    uvw = np.zeros(P * 3, np.float64)
    mx = np.zeros(6, np.float64)
    bl = np.zeros(max(B, 1) * 2, np.float64)
    st = _lib().orc_oskar_read(os.fsencode(path), amps, uvw, mx, bl)
    return (st, h, amps.view(np.complex128).reshape(P, 4), uvw.reshape(P, 3), mx,
            bl[:2 * B].reshape(B, 2))


# ------------------------------------------------------------ the reference itself
def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "liboskarref.so"))


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "liboskarref.so"))
        L.mkFromFile.argtypes = [C.POINTER(RefVisData), C.c_char_p]
        L.freeBinHandler.argtypes = [C.POINTER(RefVisData)]
        L.readAndReshuffle.argtypes = [C.POINTER(RefVisData), _f64p, _f64p, _f64p, _f64p]
        L.oskar_binary_create.restype = C.c_void_p
        L.oskar_binary_create.argtypes = [C.c_char_p, C.c_char, C.POINTER(C.c_int)]
        L.oskar_binary_write.argtypes = [C.c_void_p, C.c_ubyte, C.c_ubyte, C.c_ubyte, C.c_int,
                                         C.c_size_t, C.c_void_p, C.POINTER(C.c_int)]
        L.oskar_binary_write_ext.argtypes = [C.c_void_p, C.c_ubyte, C.c_char_p, C.c_char_p,
                                             C.c_int, C.c_size_t, C.c_void_p,
                                             C.POINTER(C.c_int)]
        L.oskar_binary_free.argtypes = [C.c_void_p]
        _ref = L
    return _ref


def ref_read(path):
    """The reference's mkFromFile + readAndReshuffle, same return shape as read()."""
    L = ref()
    vd = RefVisData()
    st = L.mkFromFile(C.byref(vd), os.fsencode(path))
    if st:
        return st, None, None, None, None, None
    P, B = vd.num_points, vd.num_baselines
    amps = np.zeros(P * 8, np.float64)
    uvw = np.zeros(P * 3, np.float64)
    mx = np.zeros(6, np.float64)
    bl = np.zeros(max(B, 1) * 2, np.float64)
    st = L.readAndReshuffle(C.byref(vd), amps, uvw, mx, bl)
    L.freeBinHandler(C.byref(vd))
    h = VisHeader()
    C.memmove(C.byref(h), C.addressof(vd) + RefVisData.num_baselines.offset, C.sizeof(h))
    return (st, h, amps.view(np.complex128).reshape(P, 4), uvw.reshape(P, 3), mx,
            bl[:2 * B].reshape(B, 2))


def ref_write_chunks(path, chunks):
    """Write a container with the reference's own writer: chunks are
    (type, group, tag, user, bytes) or (type, "group name", "tag name", user, bytes)."""
    L = ref()
    st = C.c_int(0)
    h = L.oskar_binary_create(os.fsencode(path), b"w", C.byref(st))
    if st.value:
        return st.value
    for ty, g, t, user, data in chunks:
        buf = C.create_string_buffer(bytes(data), len(data))
        if isinstance(g, str):
            L.oskar_binary_write_ext(h, ty, g.encode(), t.encode(), user, len(data), buf,
                                     C.byref(st))
        else:
            L.oskar_binary_write(h, ty, g, t, user, len(data), buf, C.byref(st))
    L.oskar_binary_free(h)
    return st.value


# ------------------------------------------------------------ pipeline records
def records(amps, uvw, num_times, num_channels, freq, pol, dom_low, dom_high,
            reference_uvw_index=False):
    """5-double records (u, v, w, re, im) of points [dom_low, dom_high) in
    [baseline][time] order for one channel and polarisation
    (MS6/programs/Kernel/IO.hs:36-70).  reference_uvw_index reproduces that
    kernel's u,v,w address, 3 * (time + T * baseline), which ignores the
    channel stride of the reshuffled array (the same point only for
    single-channel files)."""
    T, Cn = num_times, num_channels
    n = dom_high - dom_low
    out = np.zeros((n, 5), np.float64)
    p = np.arange(dom_low, dom_high)
    bl, t = p // T, p % T
    full = (bl * T + t) * Cn + freq
    uv = uvw.reshape(-1)
    ui = 3 * (t + T * bl) if reference_uvw_index else 3 * full
    out[:, 0], out[:, 1], out[:, 2] = uv[ui], uv[ui + 1], uv[ui + 2]
    v = amps.reshape(-1, 4)[full, pol]
    out[:, 3], out[:, 4] = v.real, v.imag
    return out


# ------------------------------------------------------------ layout as chunks
def vis_chunks(lay: VisLayout, amps, uu, vv, ww):
    """The chunk list orc_oskar_write emits, as (type, group, tag, user, bytes)
    (named chunks carry group/tag names), so that the reference's own
    container writer can produce the same file (ref_write_chunks)."""
    S, T, Cn, M = lay.num_stations, lay.num_times, lay.num_channels, lay.max_times_per_block
    B = S * (S - 1) // 2
    a = np.ascontiguousarray(amps, np.complex128).reshape(T, Cn, B, 4)
    u, v, w = (np.ascontiguousarray(x, np.float64).reshape(T, B) for x in (uu, vv, ww))
    ntpb = 7 + int(lay.write_autocorr) + int(lay.extended_tags)
    i4 = lambda *x: np.array(x, np.int32).tobytes()  # noqa: E731
    f8 = lambda *x: np.array(x, np.float64).tobytes()  # noqa: E731
    H, BK, DCM = 11, 12, DOUBLE_COMPLEX_MATRIX
    out = [(0x01, H, 1, 0, b"synthetic.tm\0"), (0x02, H, 2, 0, i4(ntpb)),
           (0x02, H, 3, 0, i4(int(lay.write_autocorr))), (0x02, H, 4, 0, i4(lay.amp_type)),
           (0x02, H, 5, 0, i4(M)), (0x02, H, 6, 0, i4(T)), (0x02, H, 7, 0, i4(Cn)),
           (0x02, H, 8, 0, i4(S)), (0x08, H, 9, 0, f8(lay.freq_start_hz)),
           (0x08, H, 10, 0, f8(lay.freq_inc_hz)), (0x08, H, 11, 0, f8(lay.channel_bandwidth_hz)),
           (0x08, H, 12, 0, f8(lay.time_start_mjd_utc)), (0x08, H, 13, 0, f8(lay.time_inc_sec)),
           (0x08, H, 14, 0, f8(lay.time_average_sec)), (0x08, H, 15, 0, f8(*lay.phase_centre)),
           (0x08, H, 16, 0, f8(*lay.telescope_centre))]
    out += [(0x08, H, 17 + k, 0, np.zeros(S).tobytes()) for k in range(3)]
    if lay.extended_tags:
        out.append((0x02, "rc_test", "header_note", 0, i4(1)))
    for blk in range((T + M - 1) // M):
        t0 = blk * M
        nt = min(M, T - t0)
        rows = nt if lay.trim_last_block else M
        ab = np.zeros((M, Cn, B, 4), np.complex128)
        ab[:nt] = a[t0:t0 + nt]
        ub = np.zeros((3, M, B))
        ub[0, :nt], ub[1, :nt], ub[2, :nt] = u[t0:t0 + nt], v[t0:t0 + nt], w[t0:t0 + nt]
        out += [(0x02, BK, 1, blk, i4(t0, 0, nt, Cn, B, S)),
                (0x08, BK, 2, blk, f8(lay.freq_start_hz, lay.freq_inc_hz)),
                (0x08, BK, 3, blk, f8(lay.time_start_mjd_utc + t0 * lay.time_inc_sec / 86400.0,
                                      lay.time_inc_sec / 86400.0))]
        if lay.write_autocorr:
            out.append((DCM, BK, 4, blk, np.zeros((rows, Cn, S, 4), np.complex128).tobytes()))
        out += [(DCM, BK, 5, blk, ab[:rows].tobytes()),
                (0x08, BK, 6, blk, ub[0, :rows].tobytes()),
                (0x08, BK, 7, blk, ub[1, :rows].tobytes()),
                (0x08, BK, 8, blk, ub[2, :rows].tobytes())]
        if lay.extended_tags:
            out.append((0x02, "rc_test", "block_note", blk, i4(blk)))
    return out


def chunk_index(path):
    """[(tag offset, payload offset, payload size, type, group, tag, user)] of a
    container file, for tests that alter single bytes."""
    data = open(path, "rb").read()
    pos, out = 64, []
    while pos + 20 <= len(data):
        t = data[pos:pos + 20]
        flags, ty, g, tg = t[4], t[5], t[6], t[7]
        user = int.from_bytes(t[8:12], "little", signed=True)
        block = int.from_bytes(t[12:20], "little")
        names = (g + tg) if flags & 0x80 else 0
        size = block - (4 if flags & 0x40 else 0) - names
        out.append((pos, pos + 20 + names, size, ty, g, tg, user))
        pos += 20 + block
    return out
