"""The C++ host layer (include/rc_kernels.hpp) without a GPU: its binSizer and
binner (MS6/programs/Kernel/Binning.hs:34-181) against the oracle's
restatement, bit for bit, over a tiled grid with visibilities on tile edges,
outside the grid, and a tile whose visibilities all have w = 0 (a zero-width
w range: the reference counts them into bin 0 and its binner, whose bins all
start at 0, drops them, so bin 0 is padded with zero records); and
gcfKernel's error when no GCF file covers a bin (gcfGet, Config.hs:128-132)."""
import numpy as np
import pytest

from tests import host_cpp as H

G, THETA = 256, 0.05


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return H.build_program(tmp_path_factory.mktemp("cpp"))


def test_binning_matches_the_oracle(exe, tmp_path):
    vis5 = H.synthetic(1, 5000, G, THETA, 80.0)
    # on tile edges (u = xy2uv of a boundary pixel), outside the grid, and a
    # zero-w quarter: every visibility of the (0, 0) tile gets w = 0
    edges = [H.O.xy2uv(G, THETA, z) for z in (0, 128, 256)]
    vis5[:30, 0] = np.repeat(edges, 10)
    vis5[30:40, 1] = 1e6
    first = (vis5[:, 0] < edges[1]) & (vis5[:, 1] < edges[1])
    vis5[first, 2] = 0.0
    H.write_case(tmp_path, G, THETA, 2, 4, vis5, [(0.0, np.zeros((64, 8, 8), np.complex128))])
    r = H.run(exe, tmp_path, "bins")
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "bins.bin")
    k = 0
    zero_bin_seen = False
    for tile in H.expected_bins(vis5, G, THETA, 2, 4):
        for low, high, count, recs in tile:
            assert got[k] == low and got[k + 1] == high and got[k + 2] == count
            n = int(got[k + 3])
            assert n == len(recs)
            assert np.array_equal(got[k + 4:k + 4 + 5 * n].reshape(n, 5), recs)
            zero_bin_seen |= low == high and count > 0 and not recs.any()
            k += 4 + 5 * n
    assert k == len(got)
    assert zero_bin_seen


def test_gcf_kernel_fails_like_gcfget(exe, tmp_path):
    """GCF files only for w >= 50 and every w >= 0, so the first bin, [0, 20],
    has none: the call fails there, before any GPU work."""
    vis5 = H.synthetic(2, 500, G, THETA, 80.0)
    vis5[:, 2] = np.abs(vis5[:, 2])
    H.write_case(tmp_path, G, THETA, 1, 4, vis5, [(50.0, np.zeros((64, 8, 8), np.complex128))])
    r = H.run(exe, tmp_path, "grid")
    assert r.returncode == 1
    assert "gcfGet" in r.stderr and "no GCF" in r.stderr


@pytest.mark.parametrize("flags", [[], ["-DGB_MS5_ABI"]])
def test_headers_compile_as_cxx17_and_c(tmp_path, flags):
    """rc_kernels.hpp as C++17 (with the MS5 variant's declarations too), and
    the C headers as plain C99, warning-free."""
    import os
    import subprocess

    inc = os.path.join(H.ROOT, "include")
    src = tmp_path / "t.cpp"
    src.write_text('#include "rc_kernels.hpp"\n#include "rc_gb300_ms5.h"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc,
                        str(src)] + flags, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    csrc = tmp_path / "t.c"
    csrc.write_text('#include "rc_gb300.h"\n#include "rc_oskar.h"\n#include "rc_gb300_ms5.h"\n'
                    'int main(void) { return 0; }\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc,
                        str(csrc)] + flags, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_strategy_program_builds_against_both_libraries(tmp_path):
    """The strategy program links against librc_gb300.so and, with
    -DGB_MS5_ABI, against librc_gb300_ms5.so (MS5's bindings), warning-free."""
    import os

    for ms5 in (False, True):
        assert os.path.exists(H.build_program(tmp_path, ms5=ms5))


def test_binning_of_empty_tiles(exe, tmp_path):
    """Visibilities in one quadrant only: the other tiles' w range stays
    (0, 0) from the fold's start, every bin is empty and nothing is padded."""
    vis5 = H.synthetic(3, 800, G, THETA, 60.0)
    vis5[:, 0] = -np.abs(vis5[:, 0]) - 1.0
    vis5[:, 1] = -np.abs(vis5[:, 1]) - 1.0
    H.write_case(tmp_path, G, THETA, 2, 3, vis5, [(0.0, np.zeros((64, 8, 8), np.complex128))])
    r = H.run(exe, tmp_path, "bins")
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "bins.bin")
    k = 0
    empty = 0
    for tile in H.expected_bins(vis5, G, THETA, 2, 3):
        for low, high, count, recs in tile:
            assert got[k] == low and got[k + 1] == high and got[k + 2] == count
            n = int(got[k + 3])
            assert n == len(recs)
            assert np.array_equal(got[k + 4:k + 4 + 5 * n].reshape(n, 5), recs)
            empty += low == 0.0 and high == 0.0 and count == 0 and n == 0
            k += 4 + 5 * n
    assert k == len(got) and empty == 9  # three empty tiles x three bins


def test_vectorised_binning_equals_the_loop_restatement():
    """oracle.tile_bins_vec (used by the full-size strategy test) gives the same
    bins, counts and records, bit for bit, as the loop restatement tile_bins,
    on tiles with edge visibilities, duplicate w values and a zero-width w range."""
    vis5 = H.synthetic(11, 4000, G, THETA, 60.0)
    edges = [H.O.xy2uv(G, THETA, z) for z in (0, 128, 256)]
    vis5[:30, 0] = np.repeat(edges, 10)
    vis5[40:400, 2] = np.round(vis5[40:400, 2])  # many equal w values
    first = (vis5[:, 0] < edges[1]) & (vis5[:, 1] < edges[1])
    vis5[first, 2] = 0.0
    for bins in (1, 3, 7):
        for v in H.tiles_of(G, 2):
            for u in H.tiles_of(G, 2):
                a = H.O.tile_bins(vis5, G, THETA, u, v, bins)
                b = H.O.tile_bins_vec(vis5, G, THETA, u, v, bins)
                assert len(a) == len(b)
                for (l1, h1, c1, r1), (l2, h2, c2, r2) in zip(a, b):
                    assert l1 == l2 and h1 == h2 and c1 == c2
                    assert np.array_equal(r1, r2)
