"""The drop-in path at the headline workload's full size: the 4.18 M-visibility
w-projection observation (4096^2 grid, 32 w-bins) through the C++ host layer's
gridding strategy (rc_gb300/host/gridding_strategy.cpp, `time` mode, the pass
the benchmark times): binSizer + binner over the uv-tile, one
kern_scatter_gpu1 per w-bin into the margin tile with the GCF gcfGet picks
(supports 16 / 32 / 64), detiling, and one kern_degrid_gpu1 per w-bin against
a model grid.  Against the same strategy composed from the oracle (its
binning restatement, kern_scatter and kern_degrid semantics): FP64, relative
L2 1e-12; u, v, w of the predictions exact."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import host_cpp as H
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def test_config2_strategy_through_the_reference_abi(tmp_path):
    from rc_gb300 import gcf as Gm
    from rc_gb300 import synth

    ob = synth.config("c2")
    G, bins, m = ob.grid_size, ob.n_planes, 64
    files = synth.abi_gcf_files(ob)
    tp = Gm.pswf_taper(m)
    gcfs = [(w, O.gcf_layers(w, S, m, ob.scale / 2, taper=tp)) for w, S in files]
    rng = np.random.default_rng(12)
    model = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    vis5 = ob.vis5()
    H.write_case(tmp_path, G, ob.scale, 1, bins, vis5, gcfs, model=model)
    (tmp_path / "time.txt").write_text("0 1\n")
    exe = H.build_program(tmp_path)
    r = H.run(exe, tmp_path, "time")
    assert r.returncode == 0, r.stderr

    tile = np.zeros((G + m, G + m), np.complex128)
    mx = my = -m // 2
    preds, used = [], 0
    for low, high, count, recs in O.tile_bins_vec(vis5, G, ob.scale, (0, G), (0, G), bins):
        if len(recs) == 0:
            continue
        i, conj = O.gcf_select([w for w, _ in gcfs], low, high)
        g = np.conj(gcfs[i][1]) if conj else gcfs[i][1]
        O.scatter(ob.scale, G, m, recs, g, tile, mx, my)
        preds.append(O.degrid(ob.scale, G, m, g, model, recs))
        used += count
    assert used > 0.99 * ob.n
    full = O.detile(tile, (mx, my), np.zeros((G, G), np.complex128), (0, 0))
    got = np.fromfile(tmp_path / "grid.bin").view(np.complex128).reshape(G, G)
    assert np.abs(full).max() > 0
    assert rel_l2(got, full) < TOL64
    exp = np.vstack(preds)
    got_p = np.fromfile(tmp_path / "pred.bin").reshape(-1, 5)
    assert got_p.shape == exp.shape
    assert np.array_equal(got_p[:, :3], exp[:, :3])
    assert rel_l2(got_p[:, 3:], exp[:, 3:]) < TOL64
