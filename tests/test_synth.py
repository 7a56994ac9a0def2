"""The seeded synthetic workloads on the CPU: the sizes the benchmark
configurations state, the w-plane supports rule (ceil-even of
s_min + (s_max - s_min) sqrt(|w| / w_max) at each bin's edge nearest w = 0),
the w range by the Binning.hs rule, the scale that puts the longest baseline
at 0.9 of the half grid, and determinism under the seed."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import gcf as Gm
from rc_gb300 import synth


def test_plane_supports_rule():
    sup, centres = Gm.plane_supports(-100.0, 300.0, 8, 8, 64)
    edges = np.linspace(-100.0, 300.0, 9)
    assert np.allclose(centres, 0.5 * (edges[:-1] + edges[1:]))
    for p, s in enumerate(sup):
        a, b = edges[p], edges[p + 1]
        inner = 0.0 if a <= 0.0 <= b else min(abs(a), abs(b))
        want = 8 + 56 * math.sqrt(inner / 300.0)
        assert s % 2 == 0 and 8 <= s <= 64
        assert s == min(64, max(8, 2 * math.ceil(want / 2)))
    assert sup[1] == 8  # the bin holding w = 0
    assert list(sup[1:]) == sorted(sup[1:])  # grows away from w = 0


@pytest.mark.parametrize("name,n,grid,planes,smax", [("c1", 516_096, 2048, 1, 8),
                                                     ("small", 276 * 32, 512, 8, 32)])
def test_workload_shapes(name, n, grid, planes, smax):
    ob = synth.config(name)
    assert ob.n == n and ob.grid_size == grid and ob.n_planes == planes
    assert ob.max_support == int(ob.supports.max()) <= smax
    assert ob.uvw.shape == (n, 3) and ob.vis.shape == (n,) and ob.vis.dtype == np.complex128
    maxuv = np.sqrt(ob.uvw[:, 0] ** 2 + ob.uvw[:, 1] ** 2).max()
    assert abs(maxuv * ob.scale - 0.9 * grid / 2) < 1e-6 * grid
    if planes > 1:
        assert (ob.w_low, ob.w_high) == pytest.approx(O.binsizer(ob.uvw[:, 2]), rel=0, abs=0)
    # every visibility lands on the grid with its footprint
    S = ob.max_support
    ix = O.index(ob.vis5(), ob.scale, grid, S, S, 0, 0, grid, grid)
    assert ix[:, 4].all()


def test_seeded_and_reproducible():
    a, b = synth.config("small"), synth.config("small")
    assert np.array_equal(a.uvw, b.uvw) and np.array_equal(a.vis, b.vis)
    c = synth.config("small", seed=5)
    assert not np.array_equal(a.uvw, c.uvw)
