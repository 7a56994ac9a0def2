"""The gridding strategy of MS6/programs/gridding.hs run through the C++ host
layer (include/rc_kernels.hpp, rc_gb300/host/gridding_strategy.cpp) on the GPU,
against the same strategy composed from the oracle: per (u, v) tile, the
oracle's binSizer + binner, kern_scatter semantics per w-bin with the GCF
that gcfGet picks (conjugated for negative w) into the tile with its margin,
detiling into the full grid; then kern_ifft.  And degridding every binned
visibility against the model grid; imaging the visibilities and their PSF
and CLEANing (psfVisKernel, cleanModel, cleanResidual); phase rotation to a
facet (rotateKernel).  All within relative L2 1e-12 (FP64); u, v, w of the
predictions exact."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import host_cpp as H
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

G, THETA, TILES, BINS = 1024, 0.05, 2, 24
W_FILES = [(0.0, 8), (15.0, 16), (40.0, 16), (90.0, 32)]
TOL64 = 1e-12


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = tmp_path_factory.mktemp("strategy")
    exe = H.build_program(d)
    vis5 = H.synthetic(3, 20000, G, THETA, 150.0)
    gcfs = [(w, O.gcf_layers(w, S, 32, THETA / 2)) for w, S in W_FILES]
    model = (np.random.default_rng(4).standard_normal((G, G)) +
             1j * np.random.default_rng(5).standard_normal((G, G)))
    H.write_case(d, G, THETA, TILES, BINS, vis5, gcfs, model=model)
    return exe, d, vis5, gcfs, model


def _gcf_for(gcfs, low, high):
    i, conj = O.gcf_select([w for w, _ in gcfs], low, high)
    g = gcfs[i][1]
    return np.conj(g) if conj else g


def oracle_grid(vis5, gcfs):
    """The strategy composed from the oracle: the full grid and the records used."""
    m = max(S for _, S in W_FILES)  # gcfMaxSize: the margin argument
    full = np.zeros((G, G), np.complex128)
    used = 0
    for v in H.tiles_of(G, TILES):
        for u in H.tiles_of(G, TILES):
            tile = np.zeros((v[1] - v[0] + m, u[1] - u[0] + m), np.complex128)
            mx, my = u[0] - m // 2, v[0] - m // 2
            for low, high, count, recs in O.tile_bins(vis5, G, THETA, u, v, BINS):
                if count == 0 and len(recs) == 0:
                    continue
                O.scatter(THETA, G, m, recs, _gcf_for(gcfs, low, high), tile, mx, my)
                used += len(recs)
            full = O.detile(tile, (mx, my), full, (0, 0))
    return full, used


@pytest.mark.parametrize("kernel", [1, 0, 2])  # kern_scatter_gpu1, kern_scatter, nvGridder
def test_gridding_strategy(case, kernel):
    exe, d, vis5, gcfs, model = case
    H.write_case(d, G, THETA, TILES, BINS, vis5, gcfs, gk=kernel)
    r = H.run(exe, d, "grid")
    assert r.returncode == 0, r.stderr
    full, used = oracle_grid(vis5, gcfs)
    assert used > 0.9 * len(vis5)
    got = np.fromfile(d / "grid.bin").view(np.complex128).reshape(G, G)
    assert np.abs(full).max() > 0
    assert rel_l2(got, full) < TOL64
    img = np.fromfile(d / "image.bin").reshape(G, G)
    assert rel_l2(img, O.kern_ifft(full)) < TOL64


@pytest.mark.parametrize("kernel", [1, 0])  # kern_degrid_gpu1, kern_degrid
def test_degridding_strategy(case, kernel):
    exe, d, vis5, gcfs, model = case
    H.write_case(d, G, THETA, TILES, BINS, vis5, gcfs, dk=kernel, model=model)
    r = H.run(exe, d, "degrid")
    assert r.returncode == 0, r.stderr
    m = max(S for _, S in W_FILES)
    exp = []
    for v in H.tiles_of(G, TILES):
        for u in H.tiles_of(G, TILES):
            for low, high, count, recs in O.tile_bins(vis5, G, THETA, u, v, BINS):
                if len(recs):
                    exp.append(O.degrid(THETA, G, m, _gcf_for(gcfs, low, high), model, recs))
    exp = np.vstack(exp)
    got = np.fromfile(d / "pred.bin").reshape(-1, 5)
    assert got.shape == exp.shape
    assert np.array_equal(got[:, :3], exp[:, :3])
    assert rel_l2(got[:, 3:], exp[:, 3:]) < TOL64


def test_imaging_and_clean(case):
    exe, d, vis5, gcfs, model = case
    H.write_case(d, G, THETA, TILES, BINS, vis5, gcfs)
    (d / "clean.txt").write_text("0.1 0.0\n")
    r = H.run(exe, d, "clean")
    assert r.returncode == 0, r.stderr
    dirty = O.kern_ifft(oracle_grid(vis5, gcfs)[0])
    psf5 = vis5.copy()
    psf5[:, 3], psf5[:, 4] = 1.0, 0.0
    psf = O.kern_ifft(oracle_grid(psf5, gcfs)[0])
    em, er = O.hogbom_reference(0.1, 0.0, psf, dirty, np.zeros_like(dirty))
    got_m = np.fromfile(d / "clean_model.bin").reshape(G, G)
    got_r = np.fromfile(d / "clean_residual.bin").reshape(G, G)
    assert np.abs(em).max() > 0
    assert rel_l2(got_m, em) < TOL64
    assert rel_l2(got_r, er) < TOL64


def test_rotate_to_a_facet(case):
    exe, d, vis5, gcfs, model = case
    H.write_case(d, G, THETA, TILES, BINS, vis5, gcfs)
    facets, lon, lat, l_low, m_low = 3, 1.2, -0.52, 1024, 2048
    (d / "rotate.txt").write_text("%d %.17g %.17g %d %d\n" % (facets, lon, lat, l_low, m_low))
    r = H.run(exe, d, "rotate")
    assert r.returncode == 0, r.stderr
    # Facet.hs:38-42
    lon_incr, lat_incr = THETA / G / facets, THETA / G / facets
    lon0 = lon - lon_incr * ((G * facets) // 2 - G // 2)
    lat0 = lat - lat_incr * ((G * facets) // 2 - G // 2)
    exp = O.rotate(lon, lat, lon0 + l_low * lon_incr, lat0 + m_low * lat_incr, 0, vis5)
    got = np.fromfile(d / "rot.bin").reshape(-1, 5)
    assert np.array_equal(got[:, :3], vis5[:, :3])
    assert rel_l2(got[:, 3:], exp[:, 3:]) < 1e-11  # the kern_rotate bar (test_gpu_facet.py)


@pytest.mark.parametrize("freq,pol,low,high", [(0, 0, 0, 70), (1, 3, 14, 63), (1, 2, 7, 8)])
def test_oskar_reader(tmp_path, freq, pol, low, high):
    """readOskarData + oskarReader on the committed golden file (10 baselines,
    7 times, 2 channels), against the oracle's records of the reference
    reader's own arrays (tests/golden/oskar_small_ref.npz), with the u,v,w
    address of Kernel/IO.hs."""
    import os

    from oracle import oskar as K

    exe = H.build_program(tmp_path)
    path = os.path.join(H.ROOT, "tests", "golden", "oskar_small.vis")
    (tmp_path / "oskar.txt").write_text("%s %d %d %d %d\n" % (path, freq, pol, low, high))
    r = H.run(exe, tmp_path, "oskar")
    assert r.returncode == 0, r.stderr
    ref = np.load(os.path.join(H.ROOT, "tests", "golden", "oskar_small_ref.npz"))
    exp = K.records(ref["amps"], ref["uvw"], 7, 2, freq, pol, low, high, True)
    got = np.fromfile(tmp_path / "oskar.bin").reshape(-1, 5)
    assert np.array_equal(got, exp)


def test_oskar_reader_rejects_bad_regions(tmp_path):
    import os

    exe = H.build_program(tmp_path)
    path = os.path.join(H.ROOT, "tests", "golden", "oskar_small.vis")
    for args, msg in [((2, 0, 0, 7), "non-existent frequency"), ((0, 0, 3, 10), "baseline-aligned"),
                      ((0, 0, 0, 71), "out of bounds")]:
        (tmp_path / "oskar.txt").write_text("%s %d %d %d %d\n" % ((path,) + args))
        r = H.run(exe, tmp_path, "oskar")
        assert r.returncode == 1 and msg in r.stderr, r.stderr
    (tmp_path / "oskar.txt").write_text("%s 0 0 0 7\n" % os.path.join(str(tmp_path), "none.vis"))
    r = H.run(exe, tmp_path, "oskar")
    assert r.returncode == 1 and "While trying to read binary file" in r.stderr


def test_ms5_gridding_strategy(tmp_path):
    """The same strategy against librc_gb300_ms5.so (-DGB_MS5_ABI): the CPU
    gridder type binds MS5's kern_scatter (no margin argument; GCF size 16, so
    gcfMaxSize = 16 and the tiles' margins are MS5's), and ifftKern binds MS5's
    kern_fft, 2n times MS6's kern_ifft, at 2048^2."""
    g2, files = 2048, [(0.0, 16), (30.0, 16), (80.0, 16)]
    exe = H.build_program(tmp_path, ms5=True)
    vis5 = H.synthetic(6, 12000, g2, THETA, 120.0)
    gcfs = [(w, O.gcf_layers(w, S, 16, THETA / 2)) for w, S in files]
    H.write_case(tmp_path, g2, THETA, TILES, 8, vis5, gcfs, gk=0)
    r = H.run(exe, tmp_path, "grid")
    assert r.returncode == 0, r.stderr
    full = np.zeros((g2, g2), np.complex128)
    for v in H.tiles_of(g2, TILES):
        for u in H.tiles_of(g2, TILES):
            tile = np.zeros((v[1] - v[0] + 16, u[1] - u[0] + 16), np.complex128)
            mx, my = u[0] - 8, v[0] - 8
            for low, high, count, recs in O.tile_bins(vis5, g2, THETA, u, v, 8):
                if len(recs):
                    O.scatter(THETA, g2, 16, recs, _gcf_for(gcfs, low, high), tile, mx, my)
            full = O.detile(tile, (mx, my), full, (0, 0))
    got = np.fromfile(tmp_path / "grid.bin").view(np.complex128).reshape(g2, g2)
    assert np.abs(full).max() > 0
    assert rel_l2(got, full) < TOL64
    img = np.fromfile(tmp_path / "image.bin").reshape(g2, g2)
    assert rel_l2(img, 2 * g2 * O.kern_ifft(full)) < TOL64


def test_continuum_major_loop(case):
    """The major loop of MS6/programs/continuum.hs:80-98 on the C++ host layer
    (`continuum` mode, two iterations): degridModel (kern_fft of the model,
    kern_degrid_gpu1 per w-bin: vis - D fft(model)), the corrected
    visibilities gridded and imaged, CLEAN against the PSF (cleanModel, then
    cleanResidual in the last iteration), against the same loop composed from
    the oracle.  FP64, relative L2 1e-12 for the model and the residual."""
    exe, d, vis5, gcfs, model = case
    gain, thr, loops = 0.1, 0.0, 2
    H.write_case(d, G, THETA, TILES, BINS, vis5, gcfs, gk=1, dk=1)
    (d / "clean.txt").write_text("%g %g\n" % (gain, thr))
    (d / "continuum.txt").write_text("%d\n" % loops)
    r = H.run(exe, d, "continuum")
    assert r.returncode == 0, r.stderr

    m = max(S for _, S in W_FILES)

    def degrid_all(grid):
        out = []
        for v in H.tiles_of(G, TILES):
            for u in H.tiles_of(G, TILES):
                for low, high, count, recs in O.tile_bins(vis5, G, THETA, u, v, BINS):
                    if len(recs):
                        out.append(O.degrid(THETA, G, m, _gcf_for(gcfs, low, high), grid, recs))
        return np.vstack(out)

    psf5 = vis5.copy()
    psf5[:, 3], psf5[:, 4] = 1.0, 0.0
    psf = O.kern_ifft(oracle_grid(psf5, gcfs)[0])
    mdl = np.zeros((G, G))
    res = None
    for it in range(loops):
        corrected = degrid_all(O.kern_fft(mdl))
        dirty = O.kern_ifft(oracle_grid(corrected, gcfs)[0])
        if it + 1 < loops:
            mdl, _ = O.hogbom_reference(gain, thr, psf, dirty, mdl)
        else:
            _, res = O.hogbom_reference(gain, thr, psf, dirty, np.zeros((G, G)))
    got_m = np.fromfile(d / "cont_model.bin").reshape(G, G)
    got_r = np.fromfile(d / "cont_residual.bin").reshape(G, G)
    assert np.abs(mdl).max() > 0
    assert rel_l2(got_m, mdl) < TOL64
    assert rel_l2(got_r, res) < TOL64
