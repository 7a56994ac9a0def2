"""The oracle (CPU FP64 restatement) against known answers, the reference's own
compiled MS4 gridder (oracle/_ref, where it builds), committed golden
fixtures, and an independent DFT for the GCF generator's FFT convention."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def v5(u, v, re=1.0, im=0.0, w=0.0):
    return np.array([[u, v, w, re, im]], np.float64)


# ---------------------------------------------------------------- index math KATs
def test_index_centre_and_phases():
    # grid 64, S 8, scale 1: us = u.  x0 = round(us) + 32 - 4
    for k in range(8):
        u = 3.0 + k / 8.0 + 1e-3  # fraction k/8 (+eps): ou = k for k < 4
        ix = O.index(v5(u, -2.0 + 0.25), 1.0, 64, 8, 8, 0, 0, 64, 64)[0]
        frac = u - math.floor(u)
        ou = min(7, int(np.rint(8 * frac)))
        assert ix[2] == ou
        assert ix[0] == int(np.rint(u)) + 28
        assert ix[1] == -2 + 28 and ix[3] == 2
        assert ix[4] == 1


def test_index_mixed_rounding_quirk():
    # fraction 0.75: the pixel rounds up (round) while the phase measures from the floor
    ix = O.index(v5(5.75, 0.0), 1.0, 64, 8, 8, 0, 0, 64, 64)[0]
    assert ix[0] == 6 + 28 and ix[2] == 6
    # fraction 15/16 + eps: round(8*0.94) = 8, clamped to 7
    ix = O.index(v5(5.999, 0.0), 1.0, 64, 8, 8, 0, 0, 64, 64)[0]
    assert ix[0] == 6 + 28 and ix[2] == 7


def test_index_round_half_even():
    # us = 2.5 -> round 2 (even), 3.5 -> 4; oversample 8*0.5 = 4 exactly
    a = O.index(v5(2.5, 3.5), 1.0, 64, 8, 8, 0, 0, 64, 64)[0]
    assert a[0] == 2 + 28 and a[1] == 4 + 28
    assert a[2] == 4 and a[3] == 4
    # 8*frac = 0.5 exactly (frac 1/16): rounds to 0
    b = O.index(v5(1.0625, 1.1875), 1.0, 64, 8, 8, 0, 0, 64, 64)[0]
    assert b[2] == 0 and b[3] == 2


def test_index_bounds_minus_one_and_margin():
    G, S = 64, 8
    # lo = 0, hi = 64 - 8 - 1 = 55 for margin <= S
    def keep(x0, margin=S, ext=64, mn=0):
        u = x0 - (G // 2 - S // 2)  # integral us -> x0
        return O.index(v5(float(u), 0.0), 1.0, G, S, margin, mn, 0, ext, 64)[0][4]
    assert keep(0) == 1 and keep(-1) == 0
    assert keep(55) == 1 and keep(56) == 0  # 56 would fit: the reference's extra -1
    # margin 16: gm = 4 -> [4, 51]
    assert keep(3, 16) == 0 and keep(4, 16) == 1 and keep(51, 16) == 1 and keep(52, 16) == 0
    # tile buffer with min 10, extent 20: [10, 10 + 20 - 8 - 1]
    assert keep(10, S, 20, 10) == 1 and keep(9, S, 20, 10) == 0
    assert keep(21, S, 20, 10) == 1 and keep(22, S, 20, 10) == 0


def test_index_nonfinite_and_huge_are_skipped():
    for u in [np.nan, np.inf, -np.inf, 1e300, -3e9]:
        assert O.index(v5(u, 0.0), 1.0, 64, 8, 8, 0, 0, 64, 64)[0][4] == 0


# ---------------------------------------------------------------- gridding KATs (MS2 style)
def test_point_visibility_lands_on_footprint():
    """MS2/lib/halide-gridding/test_conformance.cpp pattern: a point visibility
    with an all-ones GCF covers exactly its S x S footprint with vis*1."""
    G, S = 32, 4
    gcf = np.ones((64, S, S), np.complex128)
    grid = np.zeros((G, G), np.complex128)
    O.scatter(1.0, G, S, v5(3.0, -5.0, 2.0, -1.0), gcf, grid)
    x0, y0 = 3 + 16 - 2, -5 + 16 - 2
    exp = np.zeros_like(grid)
    exp[y0:y0 + S, x0:x0 + S] = 2.0 - 1.0j
    assert np.array_equal(grid, exp)


def test_gcf_phase_and_orientation():
    """Tap (i, j) of phase ou + 8 ov lands on grid[y0 + j][x0 + i]."""
    G, S = 32, 4
    gcf = np.zeros((64, S, S), np.complex128)
    gcf[3 + 8 * 1, 2, 1] = 1.0 + 2.0j  # ou 3, ov 1, sy 2, sx 1
    grid = np.zeros((G, G), np.complex128)
    O.scatter(1.0, G, S, v5(0.375 + 1e-9, 0.125 + 1e-9, 1.0, 1.0), gcf, grid)
    nz = np.argwhere(grid != 0)
    assert nz.tolist() == [[0 + 14 + 2, 0 + 14 + 1]]
    assert grid[16, 15] == (1 + 1j) * (1 + 2j)


def test_degrid_is_reference_form_and_passthrough():
    rng = np.random.default_rng(0)
    G, S = 48, 8
    gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    grid = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    vis = np.array([[1.3, -2.7, 5.0, 0.5, -0.25], [1e6, 0.0, 1.0, 3.0, 4.0]])
    out = O.degrid(1.0, G, S, gcf, grid, vis)
    assert np.array_equal(out[1], vis[1])  # out of bounds: unchanged
    ix = O.index(vis, 1.0, G, S, S, 0, 0, G, G)[0]
    pred = (grid[ix[1]:ix[1] + S, ix[0]:ix[0] + S] * gcf[ix[2] + 8 * ix[3]]).sum()
    assert np.allclose(out[0, 3] + 1j * out[0, 4], (0.5 - 0.25j) - pred, rtol=1e-13)
    assert np.array_equal(out[0, :3], vis[0, :3])


def test_planes_adjoint_identity():
    """mode 0 degridding is the exact adjoint of multi-plane gridding."""
    ob_rng = np.random.default_rng(3)
    n, G = 500, 96
    uvw = np.column_stack([ob_rng.uniform(-40, 40, n), ob_rng.uniform(-40, 40, n),
                           ob_rng.uniform(-1, 1, n)])
    sup = np.array([4, 6, 10], np.int32)
    offs = np.array([0, 64 * 16, 64 * 16 + 64 * 36], np.int64)
    total = int(offs[-1] + 64 * 100)
    gcf = ob_rng.standard_normal(total) + 1j * ob_rng.standard_normal(total)
    plane = ob_rng.integers(-1, 3, n).astype(np.int32)
    x = ob_rng.standard_normal((G, G)) + 1j * ob_rng.standard_normal((G, G))
    y = ob_rng.standard_normal(n) + 1j * ob_rng.standard_normal(n)
    Dx = O.degrid_planes(1.0, G, 10, uvw, plane, sup, gcf, offs, x, mode=0)
    Gy = np.zeros((G, G), np.complex128)
    O.scatter_planes(1.0, G, 10, uvw, y, plane, sup, gcf, offs, Gy)
    lhs = np.vdot(Dx, y)
    rhs = np.vdot(x, Gy)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # and the multi-thread gridder agrees with the single-thread one
    Gy2 = np.zeros((G, G), np.complex128)
    O.scatter_planes(1.0, G, 10, uvw, y, plane, sup, gcf, offs, Gy2, nthreads=4)
    assert rel_l2(Gy2, Gy) < 1e-14


def test_wbin_rule():
    w = np.array([-3.0, -1.0, 0.0, 0.5, 2.0, 2.0002, 5.0])
    uvw = np.column_stack([np.zeros_like(w), np.zeros_like(w), w])
    lo, hi = O.binsizer(w[:5])
    assert lo == -3.0 and abs(hi - (2.0 + 5.0 * 1e-4)) < 1e-15
    b = O.wbin(uvw, lo, hi, 4)
    exp = [min(3, max(0, int(math.floor((x - lo) / (hi - lo) * 4)))) if lo <= x <= hi else -1
           for x in w]
    assert b.tolist() == exp


# ---------------------------------------------------------------- GCF generator pin
def test_gcf_fft_convention_against_direct_dft():
    """The numpy restatement uses FFTW's backward (exp(+2 pi i)) unnormalised
    transform between fftshifts (fft_dyn_padded.cpp:76-103); check it against
    a direct DFT of the screen."""
    smax, over, w, t2 = 4, 8, 37.0, 0.3
    N = smax * over
    r = smax // 2
    i = np.arange(-r, r)
    x = i * (t2 / r)
    ph = w * (1 - np.sqrt(1 - x[:, None] ** 2 - x[None, :] ** 2))
    screen = np.cos(2 * np.pi * ph) - 1j * np.sin(2 * np.pi * ph)
    # arena value at final index (a, b) = sum_{p,q} screen[p,q] e^{+2 pi i (a' p' + b' q')/N}
    # with centred coordinates a' = a - N/2, p' = p - r
    a = np.arange(N) - N // 2
    E = np.exp(2j * np.pi * np.outer(a, i) / N)  # [a][p]
    arena = E @ screen @ E.T
    a4 = arena.reshape(smax, over, smax, over)
    sums = a4.real.sum(axis=(0, 2))
    S = 2
    c = smax // 2 - S // 2
    ms4 = a4[c:c + S, :, c:c + S, :].transpose(1, 3, 0, 2) / sums[:, :, None, None]
    ref = ms4.transpose(1, 0, 3, 2).reshape(64, S, S)
    got = O.gcf_layers(w, S, smax, t2)
    assert rel_l2(got, ref) < 1e-13


def test_gcf_phase_normalisation():
    # with the whole support extracted, every phase's real parts sum to 1
    # (GCF.cpp:25-32 divides each phase by the sum over the arena)
    g = O.gcf_layers(40.0, 8, 8, 0.1)
    assert np.allclose(g.real.sum(axis=(1, 2)), 1.0, atol=1e-12)


# ---------------------------------------------------------------- reference MS4 binary
def _coinciding_case(seed, G=128, S=8, nbl=23, ts=9, edges=False, lattice=False):
    """Inputs where floor- and round-based conventions coincide: fractional
    part in [k/8, k/8 + 1/16), k <= 3 (the two conventions of MS4 and MS6).
    edges: some footprints at the first and the last corner that MS6's
    bounds rule keeps (x0 = 0 and x0 = G - S - 1, either axis).  lattice:
    GCF values on a grid of 2^-10 (12 significant bits, so the fixtures that
    store them compress; the products with the visibilities still round)."""
    rng = np.random.default_rng(seed)
    scale = 50.0
    pix = rng.integers(-G // 3, G // 3, size=(nbl, ts, 2)).astype(np.float64)
    if edges:
        lo, hi = S // 2 - G // 2, G // 2 - S // 2 - 1  # x0 = 0 and x0 = G - S - 1
        corners = [(lo, lo), (hi, hi), (lo, hi), (hi, lo), (lo, 0), (0, hi)]
        for c, (a, b) in enumerate(corners[:nbl * ts]):
            pix[c % nbl, c // nbl] = (a, b)
    k = rng.integers(0, 4, size=(nbl, ts, 2))
    fr = k / 8 + rng.uniform(0, 1 / 16 - 1e-9, size=(nbl, ts, 2))
    uvw = np.zeros((nbl, ts, 3))
    uvw[..., :2] = (pix + fr) / scale
    vis = rng.standard_normal((nbl, ts)) + 1j * rng.standard_normal((nbl, ts))
    if lattice:
        gcf = (rng.integers(-2048, 2049, (64, S, S)) +
               1j * rng.integers(-2048, 2049, (64, S, S))) / 1024.0
    else:
        gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    v5_ = np.zeros((nbl * ts, 5))
    v5_[:, :3] = uvw.reshape(-1, 3)
    v5_[:, 3] = vis.real.ravel()
    v5_[:, 4] = vis.imag.ravel()
    return scale, uvw, vis, gcf, v5_


@pytest.mark.skipif(not O.ms4_available(), reason="oracle/_ref not built (needs the reference, x86-64)")
@pytest.mark.parametrize("seed,S", [(1, 8), (2, 16), (3, 4)])
def test_oracle_matches_reference_ms4_binary(seed, S):
    G = 128
    scale, uvw, vis, gcf, vis5 = _coinciding_case(seed, G, S)
    g_ref = O.ms4_grid(scale, uvw, vis, gcf, G)
    g = np.zeros((G, G), np.complex128)
    O.scatter(scale, G, S, vis5, gcf, g)
    assert rel_l2(g, g_ref) < 1e-14
    d_ref = O.ms4_degrid(scale, uvw, g_ref, gcf).ravel()
    out = O.degrid(scale, G, S, gcf, g_ref, vis5)
    pred = -((out[:, 3] - vis5[:, 3]) + 1j * (out[:, 4] - vis5[:, 4]))
    assert rel_l2(pred, d_ref) < 1e-13


# ---------------------------------------------------------------- golden fixtures
def test_oracle_against_golden_fixtures():
    path = os.path.join(GOLDEN, "ms4_reference.npz")
    if not os.path.exists(path):
        pytest.skip("golden fixtures not generated")
    z = np.load(path)
    for tag in sorted({k.split("_")[0] for k in z.files}):
        scale = float(z[f"{tag}_scale"])
        G = int(z[f"{tag}_G"])
        vis5, gcf = z[f"{tag}_vis5"], z[f"{tag}_gcf"]
        S = gcf.shape[-1]
        ref = np.zeros(G * G, np.complex128)
        ref[z[f"{tag}_gridnz"]] = z[f"{tag}_gridval"]
        ref = ref.reshape(G, G)
        g = np.zeros((G, G), np.complex128)
        O.scatter(scale, G, S, vis5, gcf, g)
        assert np.array_equal(g != 0, ref != 0), tag
        assert rel_l2(g, ref) < 1e-14, tag
        out = O.degrid(scale, G, S, gcf, ref, vis5)
        pred = -((out[:, 3] - vis5[:, 3]) + 1j * (out[:, 4] - vis5[:, 4]))
        assert rel_l2(pred, z[f"{tag}_pred"]) < 1e-13, tag
