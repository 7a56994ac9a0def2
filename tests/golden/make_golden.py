"""Generate tests/golden/ms4_reference.npz from the reference's own compiled
MS4 gridder/degridder (oracle/_ref/libms4ref.so, built by `make -C oracle
ref` from the reference sources; x86-64 only).

Cases are drawn so that the MS4 floor-based and MS6 round-based index
conventions coincide (fractional pixel part in [k/8, k/8 + 1/16), k <= 3),
so the fixtures pin the oracle's restatement of MS6 kern_scatter /
kern_degrid.  Stored per case: scale, grid size, vis5 records, GCF, the
reference grid (its non-zero pixels) and the reference degridded sums (sum
grid*gcf, no conjugate).

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
    cases = [("a", 11, 64, 8, 7, 5, False), ("b", 12, 96, 16, 5, 6, False),
             ("c", 13, 48, 4, 9, 4, False),
             # more seeds and supports, and footprints at the corners the
             # MS6 bounds rule keeps (first and last, either axis)
             ("d", 14, 64, 8, 11, 7, True), ("e", 15, 96, 16, 9, 8, True),
             ("f", 16, 48, 4, 13, 5, True), ("g", 17, 80, 20, 5, 4, True),
             ("h", 18, 80, 2, 10, 10, True), ("i", 19, 72, 12, 8, 9, True),
             ("j", 20, 96, 24, 6, 5, True), ("k", 21, 40, 6, 12, 3, True),
             ("l", 22, 112, 16, 15, 6, False), ("m", 23, 64, 10, 9, 9, True),
             ("n", 24, 56, 14, 6, 7, True)]
    for tag, seed, G, S, nbl, ts, edges in cases:
        scale, uvw, vis, gcf, vis5 = _coinciding_case(seed, G, S, nbl, ts, edges,
                                                      lattice=tag > "c")
        grid = O.ms4_grid(scale, uvw, vis, gcf, G)
        pred = O.ms4_degrid(scale, uvw, grid, gcf).ravel()
        nz = np.flatnonzero(grid)  # the grid is stored sparse: its non-zero pixels
        out.update({f"{tag}_scale": scale, f"{tag}_G": G, f"{tag}_vis5": vis5,
                    f"{tag}_gcf": gcf, f"{tag}_gridnz": nz.astype(np.int32),
                    f"{tag}_gridval": grid.ravel()[nz], f"{tag}_pred": pred})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ms4_reference.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
