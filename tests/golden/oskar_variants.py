"""OSKAR file variants shared by tests/golden/make_golden_oskar.py (which
records what the reference's own reader returns for each) and the tests
(which compare the oracle and librc_gb300 with those records).

The base file is tests/golden/oskar_small.vis: 5 stations (10 baselines),
7 times in blocks of 3 (the last block trimmed to its one time), 2 channels,
written chunk by chunk by the reference's own container writer.  Each variant
is a deterministic change of it, or a small file built from the same chunk
list.
"""
from __future__ import annotations

import numpy as np

STATIONS, TIMES, CHANNELS, BLOCK_TIMES = 5, 7, 2, 3
SEED = 20261203


def base_inputs():
    from oracle import oskar as K
    amps, uu, vv, ww = K.synth(STATIONS, TIMES, CHANNELS, seed=SEED)
    lay = K.layout(STATIONS, TIMES, CHANNELS, BLOCK_TIMES, trim_last_block=True,
                   freq_start_hz=1.4e8, freq_inc_hz=3.7e5)
    return lay, amps, uu, vv, ww


def _find(index, group, tag, user):
    for e in index:
        if e[4] == group and e[5] == tag and e[6] == user:
            return e
    raise KeyError((group, tag, user))


def _flip(data, pos):
    b = bytearray(data)
    b[pos] ^= 0x5A
    return bytes(b)


def variants(base: bytes, index):
    """name -> file bytes.  index: oracle.oskar.chunk_index of the base file."""
    from oracle import oskar as K
    v = {}
    cross1 = _find(index, 12, 5, 1)
    v["crc_cross_block1"] = _flip(base, cross1[1] + 100)
    v["crc_dim_block0"] = _flip(base, _find(index, 12, 1, 0)[1] + 2)
    v["crc_num_stations"] = _flip(base, _find(index, 11, 8, 0)[1])
    v["bad_magic"] = b"OSKARBAD" + base[8:]
    v["version_3"] = base[:9] + bytes([3]) + base[10:]
    t = _find(index, 12, 6, 2)[0]
    v["reserved_flag"] = base[:t + 4] + bytes([base[t + 4] | 0x01]) + base[t + 5:]
    v["truncated"] = base[:cross1[1] + 37]
    # a zero stored code means "no code": the corrupted payload is read as is
    b = bytearray(_flip(base, cross1[1] + 8))
    b[cross1[1] + cross1[2]:cross1[1] + cross1[2] + 4] = b"\0\0\0\0"
    v["zero_crc_unchecked"] = bytes(b)
    lay, amps, uu, vv, ww = base_inputs()
    chunks = K.vis_chunks(lay, amps, uu, vv, ww)
    v["missing_vv_block1"] = _container([c for c in chunks if not (c[1] == 12 and c[2] == 7
                                                                    and c[3] == 1)])
    v["block_larger_than_header"] = _container(
        [(c[0], c[1], c[2], c[3], np.array([2], np.int32).tobytes())
         if (c[1] == 11 and c[2] == 5) else c for c in chunks])
    lay_s = K.layout(STATIONS, TIMES, CHANNELS, BLOCK_TIMES, trim_last_block=True,
                     amp_type=K.SINGLE_COMPLEX_MATRIX)
    v["single_precision"] = _container(K.vis_chunks(lay_s, amps, uu, vv, ww))
    lay_x = K.layout(STATIONS, TIMES, CHANNELS, BLOCK_TIMES, trim_last_block=False,
                     write_autocorr=True, extended_tags=True, freq_inc_hz=-2.5e5)
    v["autocorr_named_tags_full_last_block"] = _container(K.vis_chunks(lay_x, amps, uu, vv, ww))
    return v


def _container(chunks) -> bytes:
    """Container bytes of a chunk list, written by the project's own writer
    (byte-identical to the reference's writer: tests/test_oskar.py)."""
    out = [b"OSKARBIN\0" + bytes([2]) + bytes(54)]
    for ty, g, t, user, data in chunks:
        out.append(chunk_bytes(ty, g, t, user, data))
    return b"".join(out)


def chunk_bytes(ty, g, t, user, data) -> bytes:
    from oracle import oskar as K
    es = 1 if ty & 0x01 else 4 if ty & 0x02 else 4 if ty & 0x04 else 8
    es *= 2 if ty & 0x20 else 1
    es *= 4 if ty & 0x40 else 1
    ext = isinstance(g, str)
    names = (g.encode() + b"\0" + t.encode() + b"\0") if ext else b""
    flags = 0x40 | (0x80 if ext else 0)
    gid = len(g) + 1 if ext else g
    tid = len(t) + 1 if ext else t
    block = len(data) + len(names) + 4
    tag = (b"T" + bytes([0x42]) + b"G" + bytes([es, flags, ty, gid, tid]) +
           int(user).to_bytes(4, "little", signed=True) + block.to_bytes(8, "little"))
    crc = K.crc32c(tag)
    if ext:
        crc = K.crc32c(g.encode() + b"\0", crc)
        crc = K.crc32c(t.encode() + b"\0", crc)
    crc = K.crc32c(data, crc)
    return tag + names + data + crc.to_bytes(4, "little")
