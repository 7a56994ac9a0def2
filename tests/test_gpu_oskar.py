"""OSKAR ingest on the GPU (include/rc_oskar.h) against the oracle's
restatement of the reference reader and the golden records of the reference
reader itself: outputs bit-exact, statuses equal, CRC-32C on the device equal
to the host restatement, and the extracted inputs grid like the oracle."""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import oskar as K
from tests.conftest import rel_l2
from tests.golden import oskar_variants as V

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def _digest(amps, uvw, mx, bl):
    h = hashlib.sha256()
    for a in (amps, uvw, mx, bl):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _mx(m):
    return np.array([m.maxu, m.maxv, m.maxw, m.minu, m.minv, m.minw])


def _write(tmp_path, S, T, Cn, M, seed=0, **kw):
    amps, uu, vv, ww = K.synth(S, T, Cn, seed=seed)
    lay = K.layout(S, T, Cn, M, **kw)
    p = str(tmp_path / f"f{S}_{T}_{Cn}_{M}.vis")
    assert K.write(p, lay, amps, uu, vv, ww) == 0
    return p


@pytest.mark.parametrize("S,T,Cn,M,kw", [
    (6, 7, 2, 3, {}), (9, 11, 3, 4, dict(trim_last_block=True, write_autocorr=True,
                                          extended_tags=True, freq_inc_hz=-3.3e5)),
    (20, 16, 1, 8, {}), (2, 1, 1, 1, {}), (40, 33, 2, 10, dict(trim_last_block=True))])
def test_read_and_reshuffle_host_abi_matches_oracle(tmp_path, S, T, Cn, M, kw):
    from rc_gb300 import oskar as R
    p = _write(tmp_path, S, T, Cn, M, seed=S, **kw)
    st, h, a, uvw, mx, bl = K.read(p)
    assert st == 0
    vd, a2, uvw2, mx2, bl2 = R.read_and_reshuffle(p)
    assert (vd.num_points, vd.num_baselines, vd.num_times) == (h.num_points, h.num_baselines,
                                                               h.num_times)
    _same(a2, a)
    _same(uvw2, uvw)
    _same(_mx(mx2), mx)
    _same(bl2, bl)


def test_device_read_matches_golden_reference_outputs():
    from rc_gb300 import oskar as R
    g = np.load(os.path.join(GOLDEN, "oskar_small_ref.npz"))
    td = R.read_oskar_data(os.path.join(GOLDEN, "oskar_small.vis"))
    h = td.header
    assert [h.num_baselines, h.num_channels, h.num_stations, h.num_times,
            h.num_times_baselines, h.num_points] == list(g["counts"])
    _same(td.visibilities.cpu().numpy(), g["amps"])
    _same(td.uvws.cpu().numpy(), g["uvw"])
    _same(np.array([td.metrix[k] for k in ("maxu", "maxv", "maxw", "minu", "minv", "minw")]),
          g["metrix"])
    _same(td.bl_minmax, g["blws"])


def test_statuses_match_golden_reference_statuses(tmp_path):
    """Corrupted payloads (CRC on the device), missing tags, oversize blocks,
    bad headers, single precision: the reference's status for each."""
    from rc_gb300 import lib
    g = np.load(os.path.join(GOLDEN, "oskar_small_ref.npz"))
    vis = os.path.join(GOLDEN, "oskar_small.vis")
    var = V.variants(open(vis, "rb").read(), K.chunk_index(vis))
    L = lib.load()
    for name, want, dig in zip(g["variant_names"], g["variant_status"], g["variant_digest"]):
        p = str(tmp_path / (name + ".vis"))
        open(p, "wb").write(var[name])
        vd = lib.VisData()
        st = L.mkFromFile(C.byref(vd), p.encode())
        if st == 0:
            P, B = vd.num_points, vd.num_baselines
            amps = np.zeros((P, 4), np.complex128)
            uvw = np.zeros((P, 3))
            mx = lib.Metrix()
            blw = (lib.WMaxMin * max(B, 1))()
            st = L.readAndReshuffle(C.byref(vd), amps.ctypes.data, uvw.ctypes.data, C.byref(mx),
                                    blw)
            L.freeBinHandler(C.byref(vd))
            if want == 0:
                bl = np.frombuffer(blw, np.float64).reshape(-1, 2)[:B]
                assert _digest(amps, uvw, _mx(mx), bl) == dig, name
        assert st == want, (name, st, lib.last_error())


def test_device_crc_equals_host_restatement():
    from rc_gb300 import oskar as R
    rng = np.random.default_rng(5)
    buf = rng.integers(0, 256, (1 << 20) + 4099, dtype=np.uint8)
    d = torch.tensor(buf, device="cuda")
    for n in (1, 3, 15, 16, 17, 4095, 4096, 4097, 8192, 12289, 65536 + 7, (1 << 20) + 4099):
        assert R.crc32c(d[:n]) == K.crc32c(buf[:n]), n
    for code in (0x12345678, 0xFFFFFFFF, 0, 0xE3069283):
        assert R.crc32c(d[:50000], code) == K.crc32c(buf[:50000], code)
    assert R.crc32c(d[:0], 0xABCDEF01) == 0xABCDEF01


def test_multi_piece_multi_thread_read(tmp_path):
    """Payloads above the 8 MiB staging slot and many CRC chunks per payload."""
    from rc_gb300 import oskar as R
    p = _write(tmp_path, 128, 48, 2, 16, seed=9, freq_inc_hz=2.1e6)  # 8128 bl: 16.6 MB blocks
    st, h, a, uvw, mx, bl = K.read(p)
    assert st == 0
    td = R.read_oskar_data(p)
    _same(td.visibilities.cpu().numpy(), a)
    _same(td.uvws.cpu().numpy(), uvw)
    _same(np.array(list(td.metrix.values())), mx)
    _same(td.bl_minmax, bl)
    # the same VisData can be read twice (each read searches from the first chunk)
    vd, a2, uvw2, _, _ = R.read_and_reshuffle(p)
    _same(a2, a)


def test_records_and_extract_match_the_pipeline_restatement(tmp_path):
    from rc_gb300 import lib
    from rc_gb300 import oskar as R
    p = _write(tmp_path, 8, 10, 3, 4, seed=4)
    st, h, a, uvw, mx, bl = K.read(p)
    td = R.read_oskar_data(p)
    T = h.num_times
    for freq, pol, lo, hi, ref_idx in [(0, 0, 0, 280, False), (2, 3, 30, 200, False),
                                       (1, 1, 10 * T, 20 * T + 3, True), (0, 2, 50, 50, False)]:
        got = R.oskar_reader(td, freq, pol, lo, hi, reference_uvw_index=ref_idx).cpu().numpy()
        _same(got, K.records(a, uvw, T, h.num_channels, freq, pol, lo, hi, ref_idx))
    uvw64, vis128 = R.extract(td, 1, 2, f64=True)
    exp = K.records(a, uvw, T, h.num_channels, 1, 2, 0, h.num_baselines * T)
    _same(uvw64.cpu().numpy(), exp[:, :3])
    _same(vis128.cpu().numpy(), exp[:, 3] + 1j * exp[:, 4])
    _, vis64 = R.extract(td, 1, 2)
    _same(vis64.cpu().numpy(), (exp[:, 3] + 1j * exp[:, 4]).astype(np.complex64))
    for bad in [(3, 0, 0, 10), (0, 4, 0, 10), (0, 0, 5, 20), (0, 0, 0, 10 ** 6), (0, 0, -10, 0)]:
        with pytest.raises(lib.GbError):
            R.oskar_reader(td, *bad)


def test_ingested_visibilities_grid_like_the_oracle(tmp_path):
    """File -> device reshuffle -> extraction -> FP64 gridding engine equals the
    oracle gridding the oracle reader's records."""
    from rc_gb300 import engine as E
    from rc_gb300 import gcf as G
    from rc_gb300 import oskar as R
    p = _write(tmp_path, 24, 20, 2, 8, seed=12)
    st, h, a, uvw, mx, bl = K.read(p)
    td = R.read_oskar_data(p)
    uvw_d, vis_d = R.extract(td, 1, 0, f64=True)
    rec = K.records(a, uvw, h.num_times, h.num_channels, 1, 0, 0, h.num_baselines * h.num_times)
    n = 256
    scale = 0.45 * n / np.abs(rec[:, :2]).max()
    sup = np.array([8], np.int32)
    gcf = G.pswf_uv_gcf(8)
    plan = E.Plan(uvw_d, scale=scale, grid_size=n, grid_shape=(n, n), supports=sup, margin=0)
    grid = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    plan.grid64(vis_d, torch.tensor(gcf.reshape(-1), device="cuda"), grid)
    exp = np.zeros((n, n), np.complex128)
    O.scatter_planes(scale, n, 0, rec[:, :3], rec[:, 3] + 1j * rec[:, 4],
                     np.zeros(len(rec), np.int32), sup, gcf.reshape(-1), np.array([0], np.int64),
                     exp)
    assert np.abs(exp).max() > 0
    assert rel_l2(grid.cpu().numpy(), exp) < 1e-12
