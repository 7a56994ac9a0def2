"""Helpers of the C++ host-layer tests: build rc_gb300/host/gridding_strategy.cpp
against include/rc_kernels.hpp and librc_gb300.so, and lay out its inputs."""
import os
import subprocess

import numpy as np

from oracle import oracle as O
from rc_gb300 import lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_program(out_dir, ms5=False):
    """ms5: against librc_gb300_ms5.so with -DGB_MS5_ABI (MS5's bindings)."""
    from rc_gb300 import build as B

    if ms5:
        lib.load_ms5()  # builds librc_gb300_ms5.so if needed
    else:
        lib.load()  # builds librc_gb300.so if needed
    return B.strategy_program(str(out_dir), ms5=ms5)


def write_case(d, G, theta, tiles, bins, vis5, gcf_files, gk=1, dk=1, model=None):
    """gcf_files: [(w, complex128 [64][S][S])]; returns the files' (path, S, w)."""
    files = []
    for i, (w, g) in enumerate(gcf_files):
        path = os.path.join(str(d), "gcf%d.dat" % i)
        np.ascontiguousarray(g, np.complex128).tofile(path)
        files.append((path, g.shape[-1], w))
    with open(os.path.join(str(d), "params.txt"), "w") as f:
        f.write("%d %d %.17g %d %d %d %d %d\n" % (G, G, theta, tiles, bins, len(files), gk, dk))
        for path, S, w in files:
            f.write("%s %d %.17g\n" % (path, S, w))
    np.ascontiguousarray(vis5, np.float64).tofile(os.path.join(str(d), "vis.bin"))
    if model is not None:
        np.ascontiguousarray(model, np.complex128).tofile(os.path.join(str(d), "model.bin"))
    return files


def run(exe, d, mode):
    return subprocess.run([exe, str(d), mode], capture_output=True, text=True)


def tiles_of(G, tiles):
    """Flow/Domain.hs:36-39: region i of [0, G) split n ways."""
    return [(G * i // tiles, G * (i + 1) // tiles) for i in range(tiles)]


def expected_bins(vis5, G, theta, tiles, bins):
    """Per tile (v outer, u inner), per bin: the oracle's binSizer + binner."""
    out = []
    for v in tiles_of(G, tiles):
        for u in tiles_of(G, tiles):
            out.append(O.tile_bins(vis5, G, theta, u, v, bins))
    return out


def synthetic(seed, n, G, theta, w_max):
    rng = np.random.default_rng(seed)
    lim = 0.47 * G / theta
    vis5 = np.zeros((n, 5))
    vis5[:, 0] = rng.uniform(-lim, lim, n)
    vis5[:, 1] = rng.uniform(-lim, lim, n)
    vis5[:, 2] = rng.uniform(-w_max, w_max, n) * rng.uniform(0, 1, n) ** 2
    vis5[:, 3:] = rng.standard_normal((n, 2))
    return vis5
