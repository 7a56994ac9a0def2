"""OSKAR visibility files on the CPU: the oracle's restatement of the
reference reader (oracle/oskarref.c) against the reference's own compiled
reader and container writer (oracle/_ref, where the reference checkout is) and
against the committed golden fixtures; the CRC-32C and the container layout.
No GPU."""
import hashlib
import os

import numpy as np
import pytest

from oracle import oskar as K
from tests.golden import oskar_variants as V

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
needs_ref = pytest.mark.skipif(not K.ref_available(),
                               reason="reference reader not built (no reference checkout)")


def _digest(amps, uvw, mx, bl):
    h = hashlib.sha256()
    for a in (amps, uvw, mx, bl):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _same(a, b):
    assert a.shape == b.shape
    assert np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                          np.ascontiguousarray(b).view(np.uint8))


def test_crc32c_check_value_and_continuation():
    assert K.crc32c(b"123456789") == 0xE3069283  # the published CRC-32C check value
    assert K.crc32c(b"") == 0
    rng = np.random.default_rng(1)
    data = rng.integers(0, 256, 1000, dtype=np.uint8).tobytes()
    for cut in (0, 1, 7, 8, 9, 500, 999, 1000):
        c = K.crc32c(data[:cut])
        if c != 0xFFFFFFFF:  # the container re-opens every other finished code
            assert K.crc32c(data[cut:], c) == K.crc32c(data)


@pytest.mark.parametrize("S,T,Cn,M,trim,auto,ext", [
    (6, 7, 2, 3, False, False, False), (6, 7, 2, 3, True, True, True),
    (5, 4, 1, 8, False, False, False), (12, 17, 3, 5, True, False, True),
    (2, 1, 1, 1, False, False, False)])
def test_oracle_reader_reshuffles_its_input(tmp_path, S, T, Cn, M, trim, auto, ext):
    amps, uu, vv, ww = K.synth(S, T, Cn, seed=S * T + Cn)
    lay = K.layout(S, T, Cn, M, trim_last_block=trim, write_autocorr=auto, extended_tags=ext,
                   freq_inc_hz=1.37e6)
    p = str(tmp_path / "a.vis")
    assert K.write(p, lay, amps, uu, vv, ww) == 0
    st, h, a, uvw, mx, bl = K.read(p)
    assert st == 0
    B, P = S * (S - 1) // 2, S * (S - 1) // 2 * T * Cn
    assert (h.num_baselines, h.num_points, h.num_times_baselines) == (B, P, B * T)
    # [t][c][b] -> [b][t][c]; u,v,w metres x f_c / c with f_c by repeated addition
    _same(a, amps.transpose(2, 0, 1, 3).reshape(P, 4))
    f, fs = 150e6, []
    for _ in range(Cn):
        fs.append(f / K.C_LIGHT)
        f += 1.37e6
    il = np.array(fs)
    for k, m in enumerate((uu, vv, ww)):
        _same(uvw[:, k], (m.T[:, :, None] * il).reshape(P))
    w = uvw[:, 2].reshape(B, T * Cn)
    assert np.array_equal(mx, [max(-1e12, uvw[:, 0].max()), max(-1e12, uvw[:, 1].max()),
                               max(-1e12, w.max()), min(1e12, uvw[:, 0].min()),
                               min(1e12, uvw[:, 1].min()), min(1e12, w.min())])
    assert np.array_equal(bl, np.stack([w.max(1), w.min(1)], 1))


def test_oracle_matches_golden_reference_outputs():
    g = np.load(os.path.join(GOLDEN, "oskar_small_ref.npz"))
    st, h, a, uvw, mx, bl = K.read(os.path.join(GOLDEN, "oskar_small.vis"))
    assert st == 0
    assert [h.num_baselines, h.num_channels, h.num_stations, h.num_times,
            h.num_times_baselines, h.num_points] == list(g["counts"])
    _same(a, g["amps"])
    _same(uvw, g["uvw"])
    _same(mx, g["metrix"])
    _same(bl, g["blws"])


def test_oracle_statuses_match_golden_reference_statuses(tmp_path):
    g = np.load(os.path.join(GOLDEN, "oskar_small_ref.npz"))
    vis = os.path.join(GOLDEN, "oskar_small.vis")
    var = V.variants(open(vis, "rb").read(), K.chunk_index(vis))
    assert sorted(var) == list(g["variant_names"])
    for name, want, dig in zip(g["variant_names"], g["variant_status"], g["variant_digest"]):
        p = str(tmp_path / (name + ".vis"))
        open(p, "wb").write(var[name])
        r = K.read(p)
        assert r[0] == want, name
        if want == 0:
            assert _digest(*r[2:]) == dig, name


def test_container_bytes_of_the_golden_file_are_reproduced():
    lay, amps, uu, vv, ww = V.base_inputs()
    data = V._container(K.vis_chunks(lay, amps, uu, vv, ww))
    assert data == open(os.path.join(GOLDEN, "oskar_small.vis"), "rb").read()


@needs_ref
@pytest.mark.parametrize("trim,auto,ext", [(False, False, False), (True, True, True)])
def test_writer_is_byte_identical_to_the_reference_writer(tmp_path, trim, auto, ext):
    amps, uu, vv, ww = K.synth(7, 9, 2, seed=3)
    lay = K.layout(7, 9, 2, 4, trim_last_block=trim, write_autocorr=auto, extended_tags=ext)
    p1, p2 = str(tmp_path / "ours.vis"), str(tmp_path / "ref.vis")
    assert K.write(p1, lay, amps, uu, vv, ww) == 0
    assert K.ref_write_chunks(p2, K.vis_chunks(lay, amps, uu, vv, ww)) == 0
    assert open(p1, "rb").read() == open(p2, "rb").read()


@needs_ref
@pytest.mark.parametrize("S,T,Cn,M,trim,auto,ext,finc", [
    (6, 7, 2, 3, False, False, False, 1e6), (9, 11, 3, 4, True, True, True, -3.3e5),
    (20, 16, 1, 8, False, False, False, 0.0), (4, 5, 4, 5, True, False, False, 7.7e5)])
def test_oracle_reader_matches_the_reference_reader(tmp_path, S, T, Cn, M, trim, auto, ext,
                                                    finc):
    amps, uu, vv, ww = K.synth(S, T, Cn, seed=S + T)
    lay = K.layout(S, T, Cn, M, trim_last_block=trim, write_autocorr=auto, extended_tags=ext,
                   freq_inc_hz=finc)
    p = str(tmp_path / "a.vis")
    assert K.write(p, lay, amps, uu, vv, ww) == 0
    mine, ref = K.read(p), K.ref_read(p)
    assert mine[0] == ref[0] == 0
    for x, y in zip(mine[2:], ref[2:]):
        _same(x, y)


@needs_ref
def test_oracle_statuses_match_the_reference_on_variants(tmp_path):
    vis = os.path.join(GOLDEN, "oskar_small.vis")
    for name, data in V.variants(open(vis, "rb").read(), K.chunk_index(vis)).items():
        p = str(tmp_path / (name + ".vis"))
        open(p, "wb").write(data)
        mine, ref = K.read(p), K.ref_read(p)
        assert mine[0] == ref[0], name
        if ref[0] == 0:
            for x, y in zip(mine[2:], ref[2:]):
                _same(x, y)


def test_records_restatement_reference_index_only_differs_with_channels():
    amps, uu, vv, ww = K.synth(5, 6, 1, seed=2)
    P = 10 * 6
    a = amps.transpose(2, 0, 1, 3).reshape(P, 4)
    uvw = np.stack([uu.T.reshape(P), vv.T.reshape(P), ww.T.reshape(P)], 1)
    r0 = K.records(a, uvw, 6, 1, 0, 2, 12, 60)
    r1 = K.records(a, uvw, 6, 1, 0, 2, 12, 60, reference_uvw_index=True)
    assert np.array_equal(r0, r1)
    assert np.array_equal(r0[:, 3] + 1j * r0[:, 4], a[12:60, 2])
