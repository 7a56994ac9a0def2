"""ctypes binding of librc_gb300.so (the C ABI declared in include/rc_gb300.h
and include/rc_oskar.h).

The library is the only compute path: if it is missing this module raises at
load time; there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librc_gb300.so")

GB_OK = 0
ERR_SCATTER_SIZE = -444
ERR_DEGRID_SIZE = -555
ERR_SCATTER_GPU_SIZE = -222
ERR_DEGRID_GPU_SIZE = -333
ERR_ARG = -1001
ERR_CUDA = -1002
ERR_TIMEOUT = -1003
ERR_NOMEM = -1004
ERR_CAPACITY = -1005
ERR_FFT_SIZE = -666
# staging forms of FP32 degridding (gb_plan_set_stage)
STAGE_AUTO, STAGE_SPLIT, STAGE_TMA, STAGE_ROWS = -1, 0, 1, 2

MAX_SUPPORT = 256
NOALLOC_MAX_VIS = 1 << 17
NOALLOC_MAX_PIECES = 1 << 18
NOALLOC_MAX_BINS = 1 << 16
NOALLOC_MAX_PLANES = 256
MAX_PLANES = 4096


class BufferT(C.Structure):
    """Legacy Halide buffer_t, 72 bytes (MS6/kernel/common/halide_buf.h:17-27)."""

    _fields_ = [
        ("dev", C.c_uint64),
        ("host", C.c_void_p),
        ("extent", C.c_int32 * 4),
        ("stride", C.c_int32 * 4),
        ("min", C.c_int32 * 4),
        ("elem_size", C.c_int32),
        ("host_dirty", C.c_bool),
        ("dev_dirty", C.c_bool),
        ("_padding", C.c_uint8 * 2),
    ]


assert C.sizeof(BufferT) == 72


class Geometry(C.Structure):
    _fields_ = [
        ("scale", C.c_double),
        ("grid_size", C.c_int32),
        ("margin", C.c_int32),
        ("ext_x", C.c_int32),
        ("ext_y", C.c_int32),
        ("pitch", C.c_int64),
        ("n_planes", C.c_int32),
        ("tile", C.c_int32),
        ("threads", C.c_int32),
        ("period_cap", C.c_int32),
        ("bundles_per_cta", C.c_int32),
        ("supports", C.POINTER(C.c_int32)),
        ("gcf_offsets", C.POINTER(C.c_int64)),
        ("w_low", C.c_double),
        ("w_high", C.c_double),
    ]


class BatchMember(C.Structure):
    _fields_ = [
        ("geo", Geometry),
        ("n_vis", C.c_int64),
        ("d_uvw", C.c_void_p),
        ("uvw_stride", C.c_int64),
        ("d_plane", C.c_void_p),
    ]


MAX_BATCH = 96


class VisData(C.Structure):
    """MS6/kernel/oskar/OskarBinReader.h:34-52 (`h` is the open file)."""
    _fields_ = [("h", C.c_void_p), ("num_baselines", C.c_int), ("num_channels", C.c_int),
                ("num_stations", C.c_int), ("num_times", C.c_int),
                ("num_times_baselines", C.c_int), ("num_points", C.c_int),
                ("phase_centre", C.c_double * 2), ("telescope_centre", C.c_double * 3),
                ("freq_start_inc", C.c_double * 2), ("time_start_inc", C.c_double * 2),
                ("channel_bandwidth_hz", C.c_double), ("time_average_sec", C.c_double)]


class Metrix(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("maxu", "maxv", "maxw", "minu", "minv", "minw")]


class WMaxMin(C.Structure):
    _fields_ = [("maxw", C.c_double), ("minw", C.c_double)]


OSKAR_READ_FAIL = -102
OSKAR_FILE_INVALID = -106
OSKAR_FORMAT_BAD = -107
OSKAR_MEMORY_NOT_ALLOCATED = -114
OSKAR_TAG_NOT_FOUND = -115
OSKAR_CRC_FAIL = -118
OSKAR_NOT_DOUBLE = 0xDEADBEEF - (1 << 32)
OSKAR_REFERENCE_UVW_INDEX = 1

# every exported symbol of include/rc_gb300.h: name -> (restype, argtypes)
_VP = C.c_void_p
_BP = C.POINTER(BufferT)
SIGNATURES = {
    "gb_last_error": (C.c_char_p, []),
    "gb_version": (C.c_char_p, []),
    "kern_scatter_gpu1": (C.c_int, [C.c_double, C.c_int32, C.c_int32, _BP, _BP, _BP]),
    "kern_scatter": (C.c_int, [C.c_double, C.c_int32, C.c_int32, _BP, _BP, _BP]),
    "nvGridder": (C.c_int, [C.c_double, C.c_int32, C.c_int32, _BP, _BP, _BP]),
    "kern_degrid_gpu1": (C.c_int, [C.c_double, C.c_int32, C.c_int32, _BP, _BP, _BP, _BP]),
    "kern_degrid": (C.c_int, [C.c_double, C.c_int32, C.c_int32, _BP, _BP, _BP, _BP]),
    "kern_init": (C.c_int, [_BP]),
    "kern_psf_vis": (C.c_int, [_BP, _BP]),
    "gb_plan_create": (C.c_int, [C.POINTER(Geometry), C.c_int64, _VP, C.c_int64, _VP, _VP,
                                 C.POINTER(_VP)]),
    "gb_plan_destroy": (C.c_int, [_VP]),
    "gb_plan_stats": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "gb_plan_device_status": (C.c_int, [_VP, C.POINTER(C.c_int32), _VP]),
    "gb_plan_set_stage": (C.c_int, [_VP, C.c_int32]),
    "gb_debug_fail_allocs": (C.c_int, [C.c_int32, C.c_int32]),
    "gb_host_direct": (C.c_int, []),
    "gb_checked_violations": (C.c_int, [C.POINTER(C.c_int64)]),
    "gb_checked_selftest": (C.c_int, []),
    "kern_fft": (C.c_int, [_VP, _VP]),
    "kern_ifft": (C.c_int, [_VP, _VP]),
    "gb_plan_export_index": (C.c_int, [_VP, _VP, _VP]),
    "gb_grid_f32": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_degrid_f32": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int32, _VP]),
    "gb_degrid_forward": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_degrid_backward": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_grid_forward": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_grid_backward": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_grid_forward_f64": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_grid_backward_f64": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_degrid_forward_f64": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_degrid_backward_f64": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_grid_f64": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "gb_degrid_f64": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int32, _VP]),
    "gb_gcf_generate": (C.c_int, [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int64), C.c_int32, C.c_double, _VP, _VP, _VP,
                                  _VP]),
    "gb_grid_zero_f32": (C.c_int, [_VP, C.c_int64, _VP]),
    "gb_gcf_select": (C.c_int, [C.c_int32, C.POINTER(C.c_double), C.c_double, C.c_double,
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "gb_gcf_conjugate_f32": (C.c_int, [_VP, C.c_int64, _VP]),
    "gb_gcf_conjugate_f64": (C.c_int, [_VP, C.c_int64, _VP]),
    "gb_hogbom_work_bytes": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "gb_hogbom_f32": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP, C.c_int32, C.c_int32, C.c_int32,
                                C.c_int32, C.c_float, C.c_float, C.c_int32, _VP, _VP, C.c_int64,
                                _VP]),
    "gb_hogbom_iterations": (C.c_int, [_VP, C.POINTER(C.c_int32), _VP]),
    "kern_hogbom_model": (C.c_int, [C.c_double, C.c_double, _BP, _BP, _BP]),
    "kern_detile": (C.c_int, [_BP, _BP]),
    "kern_rotate": (C.c_int, [C.c_double] * 6 + [C.c_int32, _BP, _BP]),
    "gb_detile_f32": (C.c_int, [_VP, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _VP,
                                C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _VP]),
    "gb_rotate_f64": (C.c_int, [C.c_double] * 4 + [C.c_int32, C.c_int64, _VP, _VP, _VP]),
    "kern_hogbom_residual": (C.c_int, [C.c_double, C.c_double, _BP, _BP, _BP]),
    "gb_batch_create": (C.c_int, [C.c_int32, C.POINTER(BatchMember), _VP, C.POINTER(_VP)]),
    "gb_batch_destroy": (C.c_int, [_VP]),
    "gb_batch_stats": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "gb_batch_grid_f32": (C.c_int, [_VP, C.POINTER(_VP), _VP, C.POINTER(_VP), _VP]),
    "gb_batch_degrid_f32": (C.c_int, [_VP, _VP, C.POINTER(_VP), C.POINTER(_VP), C.c_int32,
                                      _VP]),
    "gb_batch_grid_f64": (C.c_int, [_VP, C.POINTER(_VP), _VP, C.POINTER(_VP), _VP]),
    "gb_batch_degrid_f64": (C.c_int, [_VP, _VP, C.POINTER(_VP), C.POINTER(_VP), C.c_int32,
                                      _VP]),
    "gb_image_to_grid_f32": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP]),
    "gb_grid_to_image_f32": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP, _VP]),
    "gb_image_to_grid_f64": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP]),
    "gb_grid_to_image_f64": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP, _VP]),
    "gb_grid_f32_noalloc": (C.c_int, [C.POINTER(Geometry), C.c_int64, _VP, C.c_int64, _VP, _VP,
                                      _VP, _VP, _VP]),
    # include/rc_oskar.h
    "mkFromFile": (C.c_int, [C.POINTER(VisData), C.c_char_p]),
    "freeBinHandler": (None, [C.POINTER(VisData)]),
    "readAndReshuffle": (C.c_int, [C.POINTER(VisData), _VP, _VP, C.POINTER(Metrix),
                                   C.POINTER(WMaxMin)]),
    "_aligned_malloc": (_VP, [C.c_size_t, C.c_size_t]),
    "gb_oskar_read_device": (C.c_int, [C.POINTER(VisData), _VP, _VP, C.POINTER(Metrix),
                                       C.POINTER(WMaxMin), _VP]),
    "gb_oskar_records": (C.c_int, [C.POINTER(VisData), _VP, _VP, C.c_int32, C.c_int32, C.c_int64,
                                   C.c_int64, C.c_int32, _VP, _VP]),
    "gb_oskar_extract": (C.c_int, [C.POINTER(VisData), _VP, _VP, C.c_int32, C.c_int32, _VP, _VP,
                                   C.c_int32, _VP]),
    "gb_crc32c_device": (C.c_int, [_VP, C.c_int64, C.c_uint32, C.POINTER(C.c_uint32), _VP]),
    "gb_oskar_last_timings": (C.c_int, [C.POINTER(C.c_double)]),
}

_lib = None


class GbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"rc_gb300 error {code}: {msg}")
        self.code = code


def load(path: str = None):
    """Load librc_gb300.so (building it first if the sources are newer).
    RC_GB300_CHECKED=1 loads the bounds-checked variant instead."""
    global _lib
    if _lib is not None:
        return _lib
    checked = os.environ.get("RC_GB300_CHECKED", "0") == "1"
    if path is None:
        path = os.path.join(HERE, "librc_gb300_checked.so") if checked else LIB_PATH
    if not os.path.exists(path) or os.environ.get("RC_GB300_AUTOBUILD", "1") == "1":
        try:
            from . import build as _b
            _b.build(checked=checked)
        except Exception as e:  # no toolchain: a prebuilt library must exist
            if not os.path.exists(path):
                raise RuntimeError(f"librc_gb300.so is missing and could not be built: {e}")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


# MS5's two bindings that differ from MS6's (include/rc_gb300_ms5.h)
MS5_SIGNATURES = dict(SIGNATURES)
MS5_SIGNATURES["kern_scatter"] = (C.c_int, [C.c_double, C.c_int32, _BP, _BP, _BP])
MS5_SIGNATURES["kern_fft"] = (C.c_int, [_VP, _VP])

_lib_ms5 = None


def load_ms5():
    """Load librc_gb300_ms5.so, the MS5 binding variant (built first if the
    sources are newer).  Its own handle: the MS6 library can be loaded in the
    same process."""
    global _lib_ms5
    if _lib_ms5 is not None:
        return _lib_ms5
    path = os.path.join(HERE, "librc_gb300_ms5.so")
    if not os.path.exists(path) or os.environ.get("RC_GB300_AUTOBUILD", "1") == "1":
        try:
            from . import build as _b
            _b.build(ms5=True)
        except Exception as e:
            if not os.path.exists(path):
                raise RuntimeError(f"librc_gb300_ms5.so is missing and could not be built: {e}")
    L = C.CDLL(path)
    for name, (res, args) in MS5_SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib_ms5 = L
    return L


def last_error() -> str:
    return load().gb_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> int:
    if rc != GB_OK:
        raise GbError(rc, f"{what}: {last_error()}")
    return rc
