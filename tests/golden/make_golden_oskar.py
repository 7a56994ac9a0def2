"""Generate tests/golden/oskar_small.vis and tests/golden/oskar_small_ref.npz
from the reference's own OSKAR code (oracle/_ref/liboskarref.so, built by
`make -C oracle ref` from MS6/kernel/oskar/OskarBinReader.cpp and the vendored
oskar_binary C sources):

  * oskar_small.vis is written chunk by chunk by the reference's container
    writer (oskar_binary_write), with the header/block tag layout its reader
    expects (tests/golden/oskar_variants.py);
  * the npz holds what the reference's mkFromFile + readAndReshuffle return
    for it (header counts, amplitudes, u,v,w, extrema), and, for every variant
    of tests/golden/oskar_variants.py, the reference's status and a SHA-256
    digest of its outputs when the status is 0.

    python tests/golden/make_golden_oskar.py
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import oskar as K  # noqa: E402
from tests.golden import oskar_variants as V  # noqa: E402


def digest(amps, uvw, mx, bl):
    h = hashlib.sha256()
    for a in (amps, uvw, mx, bl):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    O.build(ref=True)
    if not K.ref_available():
        raise SystemExit("oracle/_ref/liboskarref.so is not available")
    lay, amps, uu, vv, ww = V.base_inputs()
    vis_path = os.path.join(HERE, "oskar_small.vis")
    st = K.ref_write_chunks(vis_path, K.vis_chunks(lay, amps, uu, vv, ww))
    assert st == 0, st
    st, h, a, uvw, mx, bl = K.ref_read(vis_path)
    assert st == 0, st
    out = {"amps": a, "uvw": uvw, "metrix": mx, "blws": bl,
           "counts": np.array([h.num_baselines, h.num_channels, h.num_stations, h.num_times,
                               h.num_times_baselines, h.num_points], np.int64),
           "freq_start_inc": np.array(h.freq_start_inc[:]),
           "time_start_inc": np.array(h.time_start_inc[:])}
    base = open(vis_path, "rb").read()
    names, statuses, digests = [], [], []
    with tempfile.TemporaryDirectory() as d:
        for name, data in sorted(V.variants(base, K.chunk_index(vis_path)).items()):
            p = os.path.join(d, name + ".vis")
            open(p, "wb").write(data)
            r = K.ref_read(p)
            names.append(name)
            statuses.append(r[0])
            digests.append(digest(*r[2:]) if r[0] == 0 else "")
    out["variant_names"] = np.array(names)
    out["variant_status"] = np.array(statuses, np.int64)
    out["variant_digest"] = np.array(digests)
    path = os.path.join(HERE, "oskar_small_ref.npz")
    np.savez_compressed(path, **out)
    for n, s in zip(names, statuses):
        print(f"{n:40s} {s}")
    print(vis_path, os.path.getsize(vis_path), "bytes;", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
