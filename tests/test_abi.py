"""The C ABI library builds, loads, and exports every entry point that
include/*.h declares; buffer_t and the OSKAR reader's structs have the
reference's byte layouts.  No compute calls (these run without a GPU)."""
import ctypes as C
import glob
import os
import re
import subprocess

from rc_gb300 import lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rc_gb300.h")
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def declared_functions():
    names = set()
    for h in HEADERS:
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(\w+)\s*\(", src, flags=re.M))
    return sorted(n for n in names if n not in ("if", "sizeof"))


def test_header_declares_the_reference_slots():
    names = declared_functions()
    for ref in ["kern_scatter_gpu1", "kern_degrid_gpu1", "nvGridder", "kern_scatter",
                "kern_degrid", "kern_init", "kern_psf_vis", "mkFromFile", "freeBinHandler",
                "readAndReshuffle", "_aligned_malloc"]:
        assert ref in names


def test_oskar_struct_layouts_match_the_reference():
    # MS6/kernel/oskar/OskarBinReader.h:34-72 on an LP64 host; the Haskell side
    # reads num_baselines .. num_points at these offsets (OskarBinReaderFFI.hsc:56-60)
    V = lib.VisData
    assert C.sizeof(V) == 8 + 6 * 4 + 11 * 8
    assert [getattr(V, f).offset for f in ("num_baselines", "num_channels", "num_stations",
                                           "num_times", "num_times_baselines",
                                           "num_points")] == [8, 12, 16, 20, 24, 28]
    assert V.phase_centre.offset == 32 and V.time_average_sec.offset == 112
    assert C.sizeof(lib.Metrix) == 48 and C.sizeof(lib.WMaxMin) == 16


def test_aligned_malloc_without_gpu():
    L = lib.load()
    p = L._aligned_malloc(1000, 64)
    assert p and p % 64 == 0
    C.CDLL(None).free(C.c_void_p(p))


def test_library_exports_every_declared_symbol():
    L = lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    # and the binding table covers them all
    assert set(declared_functions()) <= set(lib.SIGNATURES)


def test_exported_symbols_have_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for name in declared_functions():
        assert name in exported, name


def test_buffer_t_layout_matches_reference_offsets():
    # offsets written by MS6/dna/flow/Flow/Halide/BufferT.hs:26-99
    B = lib.BufferT
    assert C.sizeof(B) == 72
    assert B.host.offset == 8
    assert B.extent.offset == 16
    assert B.stride.offset == 32
    assert B.min.offset == 48
    assert B.elem_size.offset == 64
    assert B.host_dirty.offset == 68
    assert B.dev_dirty.offset == 69


def test_version_and_error_string_without_gpu():
    L = lib.load()
    assert b"sm_103a" in L.gb_version()
    assert isinstance(L.gb_last_error(), bytes)


def test_legacy_codes_are_the_reference_values():
    assert (lib.ERR_SCATTER_SIZE, lib.ERR_DEGRID_SIZE, lib.ERR_SCATTER_GPU_SIZE,
            lib.ERR_DEGRID_GPU_SIZE) == (-444, -555, -222, -333)
    hdr = open(HEADER).read()
    for code in ["-444", "-555", "-222", "-333"]:
        assert f"({code})" in hdr


def test_empty_calls_need_no_gpu():
    """Zero visibilities: the reference-ABI gridders and degridders check their
    buffers and return 0 without GPU work; the grid is left as it was."""
    import numpy as np

    from rc_gb300 import compat

    lib.load()
    vis5 = np.zeros((0, 5))
    gcf = np.ones((64, 8, 8), np.complex128)
    grid = np.full((16, 16), 1 + 2j)
    for name in ("kern_scatter_gpu1", "kern_scatter", "nvGridder"):
        assert compat.call_scatter(name, 1.0, 16, 8, vis5, gcf, grid) == 0
    assert (grid == 1 + 2j).all()
    out = np.zeros((0, 5))
    for name in ("kern_degrid_gpu1", "kern_degrid"):
        assert compat.call_degrid(name, 1.0, 16, 8, gcf, grid, vis5, out) == 0
    # the size codes still come first
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, 16, 8, vis5,
                               np.ones((64, 12, 12), np.complex128), grid) == -222


def test_kern_init_zeroes_a_large_grid_on_host_threads():
    """kern_init (MS6/kernel/cpu/gridding/init.cpp:8-15) is host work: a 64 MB
    grid with a row pitch wider than its rows is zeroed (rows split between
    host threads) and the columns past the rows stay as they were."""
    import numpy as np

    from rc_gb300 import compat

    L = lib.load()
    big = np.full((4096, 1024), 3 + 4j)
    b = compat.buf(big.view(np.float64), [(2, 1), (1000, 2), (4096, 2048)], (0, 0, 0, 0))
    assert L.kern_init(C.byref(b)) == 0
    assert (big[:, :1000] == 0).all() and (big[:, 1000:] == 3 + 4j).all()
