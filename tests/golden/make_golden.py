"""Generate tests/golden/ms4_reference.npz from the reference's own compiled
MS4 gridder/degridder (oracle/_ref/libms4ref.so, built by `make -C oracle
ref` from the reference sources; x86-64 only).

Cases are drawn so that the MS4 floor-based and MS6 round-based index
conventions coincide (fractional pixel part in [k/8, k/8 + 1/16), k <= 3),
so the fixtures pin the oracle's restatement of MS6 kern_scatter /
kern_degrid.  Stored per case: scale, grid size, vis5 records, GCF, the
reference grid and the reference degridded sums (sum grid*gcf, no conjugate).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.test_oracle import _coinciding_case  # noqa: E402


def main():
    O.build(ref=True)
    if not O.ms4_available():
        raise SystemExit("oracle/_ref/libms4ref.so is not available")
    out = {}
    for tag, seed, G, S, nbl, ts in [("a", 11, 64, 8, 7, 5), ("b", 12, 96, 16, 5, 6),
                                     ("c", 13, 48, 4, 9, 4)]:
        scale, uvw, vis, gcf, vis5 = _coinciding_case(seed, G, S, nbl, ts)
        grid = O.ms4_grid(scale, uvw, vis, gcf, G)
        pred = O.ms4_degrid(scale, uvw, grid, gcf).ravel()
        out.update({f"{tag}_scale": scale, f"{tag}_G": G, f"{tag}_vis5": vis5,
                    f"{tag}_gcf": gcf, f"{tag}_grid": grid, f"{tag}_pred": pred})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ms4_reference.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
